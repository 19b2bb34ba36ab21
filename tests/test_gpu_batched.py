"""Batched independent scenes (the 256-scene workload) packed into one grid
and advanced by one context: each scene's slice of the packed run against
the oracle run of that scene alone (shifting off, as batched runs use it).

* FP64: relative L2 <= 1e-10 per scene on x, v, sigma after 30 steps -- the
  packing introduces no coupling between scenes.
* FP32: per scene x <= 3e-6, v <= 1e-4, sigma <= 2e-3.  Positions live in
  the packed grid's coordinates, whose FP32 spacing is coarser than in a
  scene's own coordinates, hence the looser x bound than for single scenes.
"""
import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes
from oracle import port

pytestmark = pytest.mark.gpu

STEPS = 30


def _batch():
    sc = scenes.batch_scenes(n_scenes=10, n_min=200, n_max=6000, sizes=(12, 16, 20), seed=77)
    return scenes.pack_scenes(sc)


@pytest.mark.parametrize("prec,tol", [(64, {"x": 1e-10, "v": 1e-10, "sigma": 1e-10}),
                                      (32, {"x": 3e-6, "v": 1e-4, "sigma": 2e-3})])
def test_packed_scenes_match_single_runs(prec, tol):
    b = _batch()
    gpu = capi.GpuSolid(b.scene, precision=prec, shifting=False)
    gpu.steps(STEPS)
    p = gpu.particles()
    gpu.sync()
    for i, s in enumerate(b.scenes):
        o = port.PortSolid(s, shifting=False)
        o.steps(STEPS)
        q = o.particles()
        sl = slice(b.begin[i], b.end[i])
        got = {"x": b.local(i, p["x"][sl]), "v": p["v"][sl], "sigma": p["sigma"][sl]}
        for k, t in tol.items():
            assert rel_l2(got[k], q[k]) <= t, (i, k, rel_l2(got[k], q[k]))
