"""Weakly compressible Tait fluid (material model 4; the dam-break
workload) on the GPU against the oracle restatement.

The reference has no explicit fluid MPM, so parity here is unpinned by the
reference: the oracle (oracle/mpm_oracle.c, mat_tait) restates the same
equation of state on the same transfer primitives.  A small dam break
(16 x 8 x 8-cell box, 8 x 8 x 6-cell column at 8 particles per cell, slip
walls) runs 20 steps:

* FP64 GPU mode vs oracle: relative L2 <= 1e-10 on x, v, F, sigma, vol.
* FP32 GPU mode vs FP64 oracle: x <= 1e-6, v <= 1e-3, sigma <= 2e-3,
  vol <= 1e-5 (relative L2; the pressure comes from J - 1 ~ 1e-4, whose
  FP32 rounding sets the stress tolerance).
"""
import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes
from oracle import port

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.dam_break(grid=(16, 8, 8), cells=(8, 8, 6), npc=2, jitter=0.1)


def _run(prec, steps=20):
    s = _scene()
    g = capi.GpuSolid(s, precision=prec)
    g.steps(steps)
    p = g.particles()
    g.sync()
    o = port.PortSolid(s)
    o.steps(steps)
    return p, o.particles()


def test_fluid_fp64_matches_oracle():
    p, q = _run(64)
    for k in ("x", "v", "F", "sigma", "vol"):
        assert rel_l2(p[k], q[k]) <= 1e-10, (k, rel_l2(p[k], q[k]))


def test_fluid_fp32_within_tolerance():
    p, q = _run(32)
    tol = {"x": 1e-6, "v": 1e-3, "sigma": 2e-3, "vol": 1e-5}
    for k, t in tol.items():
        assert rel_l2(p[k], q[k]) <= t, (k, rel_l2(p[k], q[k]))
