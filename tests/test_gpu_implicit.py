"""Parity of the CUDA implicit solid (FP64, through the C ABI) with the reference.

* The assembled, diagonally scaled system of the first Newton iteration
  (matrix in the reference's CSR layout, D^-1/2, RHS) and the matvec against
  the reference's own outputs: relative L2 <= 1e-12.
* Linear solves and whole implicit steps against the oracle with both sides
  converged far below the reference's default (eps = 1e-24 on squared norms):
  relative L2 <= 1e-9.  The reference's GPBiCGSafe and this conjugate
  gradient solver are different Krylov methods, so they agree only as far as
  both are converged.
"""
import numpy as np
import pytest

from helpers import load_golden, rel_l2, scene_from_golden
from mpm_gb300 import capi
from oracle import port

pytestmark = pytest.mark.gpu

IMPLICIT = ["implicit_linear", "implicit_neohookean"]
TIGHT = 1.0e-24


@pytest.mark.parametrize("name", IMPLICIT)
def test_assembled_system_matches_reference(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    gpu = capi.GpuImplicitSolid(s, nr_flag=bool(g["nr_flag"]))
    gpu.assemble()
    stencil, adiag, b = gpu.system()
    amat = capi.stencil_to_csr(stencil, s.xynodec, g["matrow"], g["matcolid"])
    assert rel_l2(amat, g["amat"]) <= 1e-12
    assert rel_l2(adiag, g["adiag"]) <= 1e-12
    assert rel_l2(b, g["b_rhs"]) <= 1e-12
    assert rel_l2(gpu.matvec(g["mv_x"]), g["mv_y"]) <= 1e-12
    gpu.sync()


@pytest.mark.parametrize("name", IMPLICIT)
def test_linear_solve_matches_oracle(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    gpu = capi.GpuImplicitSolid(s, nr_flag=bool(g["nr_flag"]))
    gpu.assemble()
    x, it = gpu.solve(eps=TIGHT)
    o = port.PortSolid(s, implicit=True, nr_flag=bool(g["nr_flag"]))
    o.assemble()
    xo, ito = o.solve(eps=TIGHT)
    assert it > 0 and ito > 0
    assert rel_l2(x, xo) <= 1e-9
    # at the reference's own tolerance both solvers reach ||r||/||r0|| < 1e-4
    x8, it8 = gpu.solve(eps=1e-8)
    assert rel_l2(x8, xo) <= 1e-3
    gpu.sync()


@pytest.mark.parametrize("name", IMPLICIT)
def test_implicit_steps_match_oracle(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    nr = bool(g["nr_flag"])
    gpu = capi.GpuImplicitSolid(s, nr_flag=nr)
    kry, newton, rel = gpu.implicit_steps(int(g["nsteps"]), eps=TIGHT)
    o = port.PortSolid(s, implicit=True, nr_flag=nr)
    o.implicit_steps(int(g["nsteps"]), eps=TIGHT)
    p, q = gpu.particles(), o.particles()
    gpu.sync()
    for k in ("x", "v", "F", "sigma", "vol"):
        assert rel_l2(p[k], q[k]) <= 1e-9, (k, rel_l2(p[k], q[k]))
    # one linear solve per step at least; with NR_flag the reference's check
    # (solver.cpp:565-593) measures the residual of the solved linear system,
    # which a tight solve makes small at the first iteration
    assert newton >= int(g["nsteps"]) and kry > 0
