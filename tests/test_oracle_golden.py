"""The plain-C oracle restatement against the reference's own outputs.

The fixtures were produced by the reference's compiled translation units
(tests/golden/make_golden.py); these tests pin oracle/mpm_oracle.c to them.
The x86 build agrees bit for bit; the tolerance leaves room for fused
multiply-adds on other hosts.
"""
import numpy as np
import pytest

from helpers import load_golden, rel_l2, scene_from_golden
from oracle import port

TOL = 1.0e-12
EXPLICIT = ["explicit_pic", "explicit_flip", "explicit_quadratic", "explicit_neohookean", "explicit_stvk",
            "explicit_mooney_rivlin", "explicit_tpic", "explicit_apic", "explicit_tpic_quadratic",
            "explicit_apic_quadratic", "explicit_fbar_linear", "explicit_fbar_neohookean"]
IMPLICIT = ["implicit_linear", "implicit_neohookean", "implicit_beam_quadratic", "implicit_stvk", "implicit_mooney_rivlin"]


@pytest.mark.parametrize("name", EXPLICIT)
def test_explicit_p2g_matches_reference(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    o = port.PortSolid(s)
    o.p2g(float(g["facl"]))
    for f in ("nmass", "nvof", "nmome", "nforce", "nvel", "naccel", "nvol"):
        assert rel_l2(o.nodal(f), g[f"p2g_{f}"]) <= TOL, f


@pytest.mark.parametrize("name", EXPLICIT)
def test_explicit_steps_match_reference(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    fbar = "fbar" in g
    o = port.PortSolid(s, fbar=fbar)
    o.steps(1, float(g["facl"]))
    p = o.particles()
    for k in ("x", "v", "F", "sigma", "vol"):
        assert rel_l2(p[k], g[f"step1_{k}"]) <= TOL, k
    if "step1_affine" in g:   # TPIC vel_grad / APIC vel_Bmat . inv_Dmat
        assert rel_l2(o.affine(), g["step1_affine"]) <= TOL
    if fbar:                  # def_grad_bar, det_def_grad_bar
        Fb, Jb = o.fbar()
        assert rel_l2(Fb, g["step1_Fbar"]) <= TOL and rel_l2(Jb, g["step1_Jbar"]) <= TOL
    o.steps(int(g["nsteps"]) - 1, float(g["facl"]))
    p = o.particles()
    for k in ("x", "v", "F", "sigma", "vol"):
        assert rel_l2(p[k], g[f"stepN_{k}"]) <= 1.0e-10, k
    if "stepN_affine" in g:
        assert rel_l2(o.affine(), g["stepN_affine"]) <= 1.0e-10
    if fbar:
        Fb, Jb = o.fbar()
        assert rel_l2(Fb, g["stepN_Fbar"]) <= 1.0e-10 and rel_l2(Jb, g["stepN_Jbar"]) <= 1.0e-10


@pytest.mark.parametrize("name", IMPLICIT)
def test_implicit_matrix_and_matvec_match_reference(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    o = port.PortSolid(s, implicit=True, nr_flag=bool(g["nr_flag"]))
    o.assemble()
    matrow, matcol, amat, adiag, b = o.matrix()
    assert np.array_equal(matrow, g["matrow"])
    assert np.array_equal(matcol, g["matcolid"])
    assert rel_l2(amat, g["amat"]) <= TOL
    assert rel_l2(adiag, g["adiag"]) <= TOL
    assert rel_l2(b, g["b_rhs"]) <= TOL
    assert rel_l2(o.matvec(g["mv_x"]), g["mv_y"]) <= TOL
    x, it = o.solve()
    assert it == int(g["solve_iters"])
    assert rel_l2(x, g["solve_x"]) <= 1.0e-10


@pytest.mark.parametrize("name", IMPLICIT)
def test_implicit_steps_match_reference(name):
    g = load_golden(name)
    s = scene_from_golden(g)
    o = port.PortSolid(s, implicit=True, nr_flag=bool(g["nr_flag"]))
    o.implicit_steps(int(g["nsteps"]))
    p = o.particles()
    for k in ("x", "v", "F", "sigma", "vol"):
        assert rel_l2(p[k], g[f"stepN_{k}"]) <= 1.0e-9, k


def test_shape_functions_partition_of_unity():
    g = load_golden("explicit_quadratic")
    s = scene_from_golden(g)
    o = port.PortSolid(s)
    rng = np.random.default_rng(0)
    nex, ney, _ = s.xyelem
    for _ in range(50):
        m = int(rng.integers(0, s.xyelem[0] * s.xyelem[1] * s.xyelem[2]))
        ize, rem = divmod(m, nex * ney)
        iye, ixe = divmod(rem, nex)
        x = np.array([s.xymin[0] + s.dxy[0] * (ixe + rng.random()), s.xymin[1] + s.dxy[1] * (iye + rng.random()),
                      s.xymin[2] + s.dxy[2] * (ize + rng.random())])
        nc, sf, dsf = o.shape(m, x)
        assert len(nc) == 18  # 3 x 2 x 3 nodes for idimc (2, 1, 2)
        assert abs(sf.sum() - 1.0) < 1e-13
        assert np.abs(dsf.sum(axis=0)).max() < 1e-9


def test_tait_fluid_at_rest_without_gravity():
    """Oracle known answer: a fluid column at rest with no body force keeps
    J = 1, zero velocity and zero stress (shifting off: a uniform lattice)."""
    from mpm_gb300 import scenes
    from oracle import port

    s = scenes.dam_break(grid=(8, 8, 8), cells=(4, 4, 4), npc=2, gravity=(0.0, 0.0, 0.0))
    o = port.PortSolid(s, shifting=False)
    o.steps(5)
    q = o.particles()
    assert np.abs(q["v"]).max() == 0.0
    assert np.abs(q["sigma"]).max() == 0.0
    assert np.allclose(q["vol"], s.vol0, rtol=0, atol=0)
