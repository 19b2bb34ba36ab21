"""Shared test helpers: golden-fixture loading and error norms."""
import os

import numpy as np

from mpm_gb300.scenes import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def scene_from_golden(g):
    bcs = []
    for i in range(int(g["nbc"])):
        bcs.append((int(g[f"bc{i}_comp"]), g[f"bc{i}_nodes"].astype(np.int32), g[f"bc{i}_vals"]))
    return Scene(xyelem=tuple(int(v) for v in g["xyelem"]), xymin=tuple(g["xymin"]), dxy=tuple(g["dxy"]),
                 idimc=tuple(int(v) for v in g["idimc"]), npxye=tuple(int(v) for v in g["npxye"]),
                 dt=float(g["dt"]), mtol=float(g["mtol"]), gravity=tuple(g["gravity"]),
                 iprop=g["iprop"].astype(np.int32), mat_prop=g["mat_prop"], coord=g["coord"].copy(),
                 vel=g["vel"].copy(), mass=g["mass"].copy(), vol0=g["vol0"].copy(),
                 matid=g["matid"].astype(np.int32), scheme=int(g["scheme"]), bcs=bcs)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
