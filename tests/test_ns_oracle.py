"""Stabilized fluid MPM assembly: the numpy oracle (oracle/ns_oracle.py)
against the reference's own compiled StabilizedMPM::MakNSStabCoeff /
AssembleNSSystem (fixture tests/golden/ns_assemble.npz, made by
tests/golden/make_golden.py --fluid).  CPU only."""
import os

import numpy as np

from mpm_gb300 import capi
from oracle import ns_oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_assemble.npz")
TOL = 1e-12   # FP64, summation order differs from the reference's element-ordered loop


def golden():
    return dict(np.load(GOLDEN))


def run_oracle(g):
    return ns_oracle.ns_assemble(g["xyelem"], g["xymin"], g["dxy"], float(g["rho"]), float(g["rmu"]), float(g["dt"]),
                                 float(g["beta"]), float(g["gamma"]), g["gravity"], float(g["facl"]),
                                 float(g["mtol"]), g["x"], g["mass"], g["vol"], g["nvel"], g["naccel"], g["ndispl"],
                                 g["npres"], g["nmass"])


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_ns_oracle_matches_reference_fixture():
    g = golden()
    tau1, tau2, st, b = run_oracle(g)
    assert rel(tau1, g["tau1"]) < TOL and rel(tau2, g["tau2"]) < TOL
    amat = capi.stencil_to_csr(st, tuple(g["xyelem"] + 1), g["matrow"], g["matcolid"])
    for k in range(16):
        assert rel(amat[k], g["amat"][k]) < TOL, k
    assert rel(b, g["b_rhs"]) < TOL
    # every stencil entry the graph does not hold is zero
    assert np.isclose(np.abs(amat).sum(), np.abs(st).sum(), rtol=1e-14)


def test_ns_fixture_covers_both_element_size_branches():
    g = golden()
    he0 = g["dxy"][0] * np.cbrt(6.0 / np.pi)
    zero_branch = np.isclose(g["tau2"], he0 * he0 / (4.0 * g["tau1"]), rtol=1e-12)
    assert 0 < zero_branch.sum() < len(zero_branch)


def test_ns_velocity_blocks_are_symmetric():
    """K_ab[r][c] = K_ba[c][r] for the velocity-velocity part (viscous and
    shock-capturing terms), and the pressure-pressure entry is symmetric."""
    g = golden()
    _, _, st, _ = run_oracle(g)
    nnc = tuple(g["xyelem"] + 1)
    nx, ny, nz = nnc
    N = nx * ny * nz
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for s in range(27):
        dx, dy, dz = s % 3 - 1, (s // 3) % 3 - 1, s // 9 - 1
        ok = ((ii + dx >= 0) & (ii + dx < nx) & (jj + dy >= 0) & (jj + dy < ny) & (kk + dz >= 0) & (kk + dz < nz))
        rows = (ii + nx * (jj + ny * kk))[ok]
        cols = rows + dx + nx * (dy + ny * dz)
        for r in range(3):
            for c in range(3):
                assert np.allclose(st[s, 4 * r + c, rows], st[26 - s, 4 * c + r, cols], rtol=1e-12, atol=1e-9)
        assert np.allclose(st[s, 15, rows], st[26 - s, 15, cols], rtol=1e-12, atol=1e-15)
    assert N == st.shape[2]


def test_ns_newton_oracle_matches_reference_fixture():
    """The numpy SolveNS (exact linear solves) against the reference's own
    Newton loop with GPBiCGSafe post-iterated to ||b - A x|| <= 1e-10 ||b||
    (fixture tests/golden/ns_solve.npz, made by make_golden.py --fluid-newton):
    the same Newton iteration count and the displacement and pressure within
    the reference's solve tolerance."""
    g = dict(np.load(os.path.join(os.path.dirname(GOLDEN), "ns_solve.npz")))
    bcs = [(g["bc_wall"], np.zeros(len(g["bc_wall"])))] * 3 + [(g["bc_top"], np.zeros(len(g["bc_top"])))]
    nd, npres, it, hist = ns_oracle.ns_solve(g["xyelem"], g["xymin"], g["dxy"], float(g["rho"]), float(g["rmu"]),
                                             float(g["dt"]), float(g["beta"]), float(g["gamma"]), g["gravity"],
                                             float(g["facl"]), float(g["mtol"]), g["x"], g["mass"], g["vol"],
                                             g["nvel"], g["naccel"], g["nmass"], bcs)
    assert it == int(g["newton"])
    assert rel(nd, g["ndispl"]) < 1e-10 and rel(npres, g["npres"]) < 1e-10


def ns_step_fixture():
    g = dict(np.load(os.path.join(os.path.dirname(GOLDEN), "ns_step.npz")))
    bcs = [(g["bc_wall"], np.zeros(len(g["bc_wall"])))] * 3 + [(g["bc_top"], np.zeros(len(g["bc_top"])))]
    return g, bcs


def test_ns_step_oracle_matches_reference_fixture():
    """Whole fluid time steps (Particle2Node, SolveNS, Node2Particle of
    module/fluid/MPM/var_trans_fluid.cpp and solve_ns_mpm.cpp) of the numpy
    oracle against the reference's own loop (fixture tests/golden/ns_step.npz,
    made by make_golden.py --fluid-step; linear systems solved to 1e-10 there,
    exactly here), PIC and FLIP, after 1 and 3 steps: the first Particle2Node's
    nodal fields to 1e-14, the particle displacement, velocity, acceleration
    and pressure to 1e-9 relative L2 (the reference's solve tolerance)."""
    g, bcs = ns_step_fixture()
    for scheme, tag in ((0, "pic"), (1, "flip")):
        for k in (1, int(g["nsteps"])):
            first, part = ns_oracle.ns_step(g["xyelem"], g["xymin"], g["dxy"], (2, 2, 2), float(g["rho"]),
                                            float(g["rmu"]), float(g["dt"]), float(g["beta"]), float(g["gamma"]),
                                            g["gravity"], float(g["facl"]), float(g["mtol"]), scheme, g["x"],
                                            g["mass"], g["vol"], g["vel"], g["accel"], bcs, nsteps=k)
            if k == 1:
                for f, v in first.items():
                    assert rel(v, g[f"{tag}_p2g_{f}"]) < 1e-14, (tag, f)
            want = {f: g[f"{tag}_s{k}_{f}"] for f in ("x", "v", "a", "pres")}
            assert rel(part["x"] - g["x"], want["x"] - g["x"]) < 1e-9, (tag, k)
            for f in ("v", "a", "pres"):
                assert rel(part[f], want[f]) < 1e-9, (tag, k, f)


def ns_lid_fixture():
    g = dict(np.load(os.path.join(os.path.dirname(GOLDEN), "ns_step_lid.npz")))
    vw = (g["bc_vw_nodes"], np.zeros(len(g["bc_vw_nodes"])))
    bcs = [(g["bc_u_nodes"], g["bc_u_vals"]), vw, vw, (g["bc_p_nodes"], g["bc_p_vals"])]
    return g, bcs


def test_ns_step_oracle_with_boundary_values_matches_reference():
    """The fluid loop with non-zero boundary values and a load factor of 0.6
    (a lid-driven cavity: the top face at u = 0.04 m/s, 5 Pa at one node;
    fixture tests/golden/ns_step_lid.npz from make_golden.py --fluid-step):
    BCSetVal and BCNRSet scale the values by facl (and dt) as the reference
    does; nodal fields of the first Particle2Node to 1e-14, the particle state
    after 2 FLIP steps to 1e-9."""
    g, bcs = ns_lid_fixture()
    first, part = ns_oracle.ns_step(g["xyelem"], g["xymin"], g["dxy"], (2, 2, 2), float(g["rho"]), float(g["rmu"]),
                                    float(g["dt"]), float(g["beta"]), float(g["gamma"]), g["gravity"],
                                    float(g["facl"]), float(g["mtol"]), 1, g["x"], g["mass"], g["vol"], g["vel"],
                                    g["accel"], bcs, nsteps=int(g["nsteps"]))
    for f, v in first.items():
        assert rel(v, g[f"p2g_{f}"]) < 1e-14, f
    assert rel(part["x"] - g["x"], g["s_x"] - g["x"]) < 1e-9
    for f in ("v", "a", "pres"):
        assert rel(part[f], g[f"s_{f}"]) < 1e-9, f
