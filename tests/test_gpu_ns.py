"""Stabilized fluid MPM assembly on the GPU (mpm_gpu_ns_assemble) against the
reference's own compiled AssembleNSSystem (fixture), against the numpy oracle
on a larger seeded case, and, at full size, against size-independent
properties of the system (symmetric velocity and pressure blocks).  FP64:
relative L2 tolerance 1e-12 (summation order differs from the reference)."""
import os
import sys

import numpy as np
import pytest

from mpm_gb300 import capi
from oracle import ns_oracle

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402  (seeded input generator only; the reference is not touched)

pytestmark = pytest.mark.gpu
TOL = 1e-12
KEYS = ("rho", "rmu", "dt", "beta", "gamma", "gravity", "facl", "mtol")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def gpu_run(c):
    torch = pytest.importorskip("torch")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
    out = capi.ns_assemble(c["xyelem"], c["xymin"], c["dxy"], *(c[k] for k in KEYS), t(c["x"].T.copy()),
                           t(c["mass"]), t(c["vol"]), t(c["nvel"]), t(c["naccel"]), t(c["ndispl"]), t(c["npres"]),
                           t(c["nmass"]))
    return [o.cpu().numpy() for o in out]


def test_gpu_ns_matches_reference_fixture():
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_assemble.npz")))
    tau1, tau2, st, b = gpu_run(g)
    assert rel(tau1, g["tau1"]) < TOL and rel(tau2, g["tau2"]) < TOL
    amat = capi.stencil_to_csr(st, tuple(g["xyelem"] + 1), g["matrow"], g["matcolid"])
    for k in range(16):
        assert rel(amat[k], g["amat"][k]) < TOL, k
    assert rel(b, g["b_rhs"]) < TOL
    assert np.isclose(np.abs(amat).sum(), np.abs(st).sum(), rtol=1e-14)


def test_gpu_ns_matches_oracle_ragged_grid():
    c = make_golden.ns_inputs(seed=3, xyelem=(13, 9, 7), dx=0.05, ppd=2)
    want = ns_oracle.ns_assemble(c["xyelem"], c["xymin"], c["dxy"], *(c[k] for k in KEYS), c["x"], c["mass"],
                                 c["vol"], c["nvel"], c["naccel"], c["ndispl"], c["npres"], c["nmass"])
    got = gpu_run(c)
    for w, g_ in zip(want, got):
        assert rel(g_.ravel(), w.ravel()) < TOL


def test_gpu_ns_no_particles_gives_inertia_only():
    c = make_golden.ns_inputs(seed=4, xyelem=(4, 4, 4))
    c = {**c, "x": np.zeros((0, 3)), "mass": np.zeros(0), "vol": np.zeros(0)}
    _, _, st, b = gpu_run(c)
    assert not st.any()
    nb = ns_oracle.newmark(c["dt"], c["beta"], c["gamma"])
    N = len(c["nmass"])
    acc = nb[3] * c["ndispl"] - nb[4] * c["nvel"] - nb[5] * c["naccel"]
    assert np.allclose(b[:3 * N], -(np.tile(c["nmass"], 3) * acc), rtol=1e-14, atol=0)
    assert not b[3 * N:].any()


def test_gpu_ns_out_of_grid_particle_is_reported():
    c = make_golden.ns_inputs(seed=5, xyelem=(4, 4, 4))
    c["x"] = c["x"].copy()
    c["x"][0, 0] = -1.0
    with pytest.raises(RuntimeError, match="outside the grid"):
        gpu_run(c)


def test_gpu_ns_full_size_symmetry_and_timing():
    """~4.1M particles (8 per cell in an 80^3-cell block of a 100^3 grid): the
    velocity-velocity blocks satisfy K_ab[r][c] = K_ba[c][r] and the
    pressure-pressure entries are symmetric; prints the mean assembly time."""
    torch = pytest.importorskip("torch")
    ne, blk = 100, 80
    dx = 1.0 / ne
    rng = np.random.default_rng(9)
    lo = (ne - blk) // 2
    cells = np.stack(np.meshgrid(*[np.arange(lo, lo + blk)] * 3, indexing="ij"), -1).reshape(-1, 3)
    sub = np.array([(i, j, k) for k in range(2) for j in range(2) for i in range(2)])
    x = ((cells[:, None, :] + (sub[None] + 0.5) / 2.0).reshape(-1, 3) + rng.uniform(-0.2, 0.2, (len(cells) * 8, 3)) / 2) * dx
    n = len(x)
    N = (ne + 1) ** 3
    dev = "cuda:0"
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    vol = np.full(n, dx ** 3 / 8)
    args = [t(x.T.copy()), t(1000.0 * vol), t(vol), t(rng.normal(0, 0.5, 3 * N)), t(rng.normal(0, 2, 3 * N)),
            t(rng.normal(0, 1e-3 * dx, 3 * N)), t(rng.normal(0, 50, N)), t(rng.uniform(0, 0.2, N))]
    prm = (1000.0, 0.05, 1e-3, 0.25, 0.5, (0.0, 0.0, -9.8), 1.0, 1e-12)
    geo = ((ne,) * 3, (0.0,) * 3, (dx,) * 3)
    for _ in range(3):
        capi.ns_assemble(*geo, *prm, *args)
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    reps = 5
    e0.record(s)
    for _ in range(reps):
        out = capi.ns_assemble(*geo, *prm, *args)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    print(f"\nmpm_gpu_ns_assemble: {n} particles, {N} nodes: {ms:.3f} ms per system "
          f"({n / ms * 1e3:.3e} particles/s, {n * 1056 / ms * 1e-6:.3e} FP64 atomics/ns)")
    st = out[2]
    nx = ne + 1
    idx = torch.arange(N, device=dev)
    ii, jj, kk = idx % nx, (idx // nx) % nx, idx // (nx * nx)
    worst = 0.0
    for sl in range(27):
        dx_, dy_, dz_ = sl % 3 - 1, (sl // 3) % 3 - 1, sl // 9 - 1
        ok = (ii + dx_ >= 0) & (ii + dx_ < nx) & (jj + dy_ >= 0) & (jj + dy_ < nx) & (kk + dz_ >= 0) & (kk + dz_ < nx)
        rows = idx[ok]
        cols = rows + dx_ + nx * (dy_ + nx * dz_)
        for r, c in [(r, c) for r in range(3) for c in range(3)] + [(3, 3)]:
            a = st[sl, 4 * r + c, rows]
            bt = st[26 - sl, 4 * c + r, cols]
            scale = float(a.abs().max()) + 1e-300
            worst = max(worst, float((a - bt).abs().max()) / scale)
    assert worst < 1e-12, worst


def _newton_gpu(c, bcs, rtol=1.0e-10):
    torch = pytest.importorskip("torch")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
    s = capi.NsSolver(c["xyelem"], c["xymin"], c["dxy"], *(c[k] for k in KEYS), bcs=bcs)
    (nd, npres, _, _), st = s.solve(t(c["x"].T.copy()), t(c["mass"]), t(c["vol"]), t(c["nvel"]), t(c["naccel"]),
                                    t(c["nmass"]), rtol=rtol)
    s.close()
    return nd.cpu().numpy(), npres.cpu().numpy(), st


def _box_bcs(c):
    return [(c["bc_wall"], np.zeros(len(c["bc_wall"])))] * 3 + [(c["bc_top"], np.zeros(len(c["bc_top"])))]


def test_gpu_ns_newton_matches_reference_fixture():
    """SolveNS on the GPU (mpm_ns_solve: Newton + GPBiCGSafe on the scaled
    4-DOF system) against the reference's own Newton loop, both solved to
    ||b - A x|| <= 1e-10 ||b||: displacement and pressure within 1e-9."""
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_solve.npz")))
    nd, npres, st = _newton_gpu(g, _box_bcs(g))
    print(f"\nSolveNS vs reference: ndispl {rel(nd, g['ndispl']):.2e}, npres {rel(npres, g['npres']):.2e}; {st}")
    assert st["newton_iters"] == int(g["newton"])
    assert rel(nd, g["ndispl"]) < 1e-9 and rel(npres, g["npres"]) < 1e-9
    assert st["last_residual"] < 1e-6   # CheckNRConvergence's residual of the solved system


def test_gpu_ns_newton_matches_oracle_larger_box():
    """A larger, ragged box against the numpy SolveNS with exact solves."""
    c = make_golden.ns_box_inputs(xyelem=(11, 8, 7), seed=7, amp=0.2)
    bcs = _box_bcs(c)
    want_d, want_p, it, _ = ns_oracle.ns_solve(c["xyelem"], c["xymin"], c["dxy"], *(c[k] for k in KEYS), c["x"],
                                               c["mass"], c["vol"], c["nvel"], c["naccel"], c["nmass"], bcs)
    nd, npres, st = _newton_gpu(c, bcs)
    print(f"\nSolveNS vs oracle ({len(c['mass'])} particles): ndispl {rel(nd, want_d):.2e}, "
          f"npres {rel(npres, want_p):.2e}; {st}")
    assert st["newton_iters"] == it
    assert rel(nd, want_d) < 1e-9 and rel(npres, want_p) < 1e-9


# ------------------------------------------------------------ whole time steps
def _fluid_gpu(c, bcs, vel, accel, scheme, nsteps, p2g_only=False, x=None):
    """The GPU fluid loop (mpm_ns_p2g / mpm_ns_step) on FP64 CUDA arrays;
    returns the nodal fields of the first Particle2Node, the particle state
    after nsteps and the last step's stats."""
    torch = pytest.importorskip("torch")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
    s = capi.NsSolver(c["xyelem"], c["xymin"], c["dxy"], *(c[k] for k in KEYS), bcs=bcs)
    X = t((c["x"] if x is None else x).T.copy())
    V, A = t(vel.T.copy()), t(accel.T.copy())
    P = t(np.zeros(len(c["mass"])))
    m, vol = t(c["mass"]), t(c["vol"])
    s.p2g(X, V, A, m, vol, scheme, c["facl"])
    first = {k: s.nodal(k) for k in ("nmass", "nvof", "nvel", "naccel")}
    st = None
    if not p2g_only:
        for _ in range(nsteps):
            st = s.step(X, V, A, P, m, vol, scheme, c["facl"], rtol=1.0e-10)
    s.close()
    h = lambda a: a.cpu().numpy().T.copy()
    return first, dict(x=h(X), v=h(V), a=h(A), pres=P.cpu().numpy()), st


def test_gpu_ns_step_matches_reference_fixture():
    """Whole fluid time steps on the GPU against the reference's own loop
    (MeshPointLinklist, Particle2Node, SolveNS, Node2Particle of
    module/fluid/MPM/; fixture tests/golden/ns_step.npz from make_golden.py
    --fluid-step), PIC and FLIP: Particle2Node's nodal fields to 1e-12 (the
    fixed-point sums), the particle displacement, velocity, acceleration and
    pressure after 1 and 3 steps to 1e-9 relative L2 (both sides solve each
    linear system to 1e-10)."""
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_step.npz")))
    bcs = _box_bcs(g)
    for scheme, tag in ((0, "pic"), (1, "flip")):
        for k in (1, int(g["nsteps"])):
            first, part, st = _fluid_gpu(g, bcs, g["vel"], g["accel"], scheme, k)
            if k == 1:
                for f, v in first.items():
                    assert rel(v, g[f"{tag}_p2g_{f}"]) < TOL, (tag, f, rel(v, g[f"{tag}_p2g_{f}"]))
            want = {f: g[f"{tag}_s{k}_{f}"] for f in ("x", "v", "a", "pres")}
            errs = {"dx": rel(part["x"] - g["x"], want["x"] - g["x"])}
            errs.update({f: rel(part[f], want[f]) for f in ("v", "a", "pres")})
            print(f"\nfluid step vs reference, {tag}, {k} steps: " + ", ".join(f"{f} {e:.2e}" for f, e in errs.items()))
            assert max(errs.values()) < 1e-9, (tag, k, errs)


def test_gpu_ns_step_matches_oracle_larger_box_and_is_reproducible():
    """A larger, ragged box (4,928 particles, faster flow) for 2 FLIP steps
    against the numpy oracle with exact solves, and a second run of the same
    steps bitwise identical (fixed-point P2G sums, block-ordered reductions).
    Tolerances: 1e-8 on the displacement and velocity; 1e-7 on the
    acceleration and pressure, which the Newmark update a = u / (beta dt^2) -
    ... and the pressure block take from the solve with its residual error
    (||b - A x|| <= 1e-10 ||b||) amplified (measured 1.8e-8 and 8.8e-9)."""
    c = make_golden.ns_box_inputs(xyelem=(11, 8, 7), seed=7, amp=0.2)
    bcs = _box_bcs(c)
    vel, acc = make_golden.ns_particle_kinematics(c["x"], c["dxy"][0], c["xyelem"], amp=0.2, seed=9)
    _, want = ns_oracle.ns_step(c["xyelem"], c["xymin"], c["dxy"], (2, 2, 2), *(c[k] for k in KEYS), 1, c["x"],
                                c["mass"], c["vol"], vel, acc, bcs, nsteps=2)
    _, got, st = _fluid_gpu(c, bcs, vel, acc, 1, 2)
    _, again, _ = _fluid_gpu(c, bcs, vel, acc, 1, 2)
    errs = {"dx": rel(got["x"] - c["x"], want["x"] - c["x"])}
    errs.update({f: rel(got[f], want[f]) for f in ("v", "a", "pres")})
    print(f"\nfluid step vs oracle ({len(c['mass'])} particles, 2 FLIP steps): "
          + ", ".join(f"{f} {e:.2e}" for f, e in errs.items()) + f"; {st}")
    assert errs["dx"] < 1e-8 and errs["v"] < 1e-8, errs
    assert errs["a"] < 1e-7 and errs["pres"] < 1e-7, errs
    for f in got:
        assert np.array_equal(got[f], again[f]), f


def test_gpu_ns_step_with_boundary_values_matches_reference():
    """Non-zero boundary values and a load factor of 0.6 (the lid-driven
    cavity of tests/golden/ns_step_lid.npz, 2 FLIP steps of the reference's
    own fluid loop): Particle2Node's nodal fields to 1e-12, the particle state
    to 1e-9."""
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_step_lid.npz")))
    vw = (g["bc_vw_nodes"], np.zeros(len(g["bc_vw_nodes"])))
    bcs = [(g["bc_u_nodes"], g["bc_u_vals"]), vw, vw, (g["bc_p_nodes"], g["bc_p_vals"])]
    first, part, st = _fluid_gpu(g, bcs, g["vel"], g["accel"], 1, int(g["nsteps"]))
    for f, v in first.items():
        assert rel(v, g[f"p2g_{f}"]) < TOL, (f, rel(v, g[f"p2g_{f}"]))
    errs = {"dx": rel(part["x"] - g["x"], g["s_x"] - g["x"])}
    errs.update({f: rel(part[f], g[f"s_{f}"]) for f in ("v", "a", "pres")})
    print("\nlid-driven fluid steps vs reference: " + ", ".join(f"{f} {e:.2e}" for f, e in errs.items()))
    assert max(errs.values()) < 1e-9, errs


def test_gpu_ns_member_calls_on_held_particles_match_the_step():
    """The reference's three member calls on particles the context holds
    (mpm_ns_load_particles, then per step mpm_ns_particle2node,
    mpm_ns_solve_ns, mpm_ns_node2particle; mpm_ns_download_particles) give
    bitwise the particle state of mpm_ns_step on caller arrays, which the
    fixture test pins to the reference; a call out of order is refused."""
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_step.npz")))
    bcs = _box_bcs(g)
    _, want, _ = _fluid_gpu(g, bcs, g["vel"], g["accel"], 1, 3)
    pytest.importorskip("torch")
    s = capi.NsSolver(g["xyelem"], g["xymin"], g["dxy"], *(g[k] for k in KEYS), bcs=bcs)
    s.load_particles(g["x"], g["vel"], g["accel"], g["mass"], g["vol"])
    with pytest.raises(capi.MpmError) as err:
        s.node2particle()
    assert err.value.code == 8   # MPM_ERR_STATE: Node2Particle before Particle2Node
    for _ in range(3):
        s.particle2node(1, g["facl"])
        st = s.solve_ns(rtol=1.0e-10)
        s.node2particle()
    got = s.download_particles()
    s.close()
    assert st["newton_iters"] >= 1
    for f in ("x", "v", "a", "pres"):
        assert np.array_equal(got[f], want[f]), f
    assert rel(got["x"] - g["x"], g["flip_s3_x"] - g["x"]) < 1e-9


def test_gpu_ns_step_reports_particle_outside_grid():
    """A particle beyond the grid's upper x wall: mpm_ns_step returns
    MPM_ERR_PARTICLE_OUT_OF_BOX before writing anything (the reference stops
    on a particle that leaves the domain, module/mpi_data.cpp:31-34)."""
    torch = pytest.importorskip("torch")
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ns_step.npz")))
    x = g["x"].copy()
    x[5, 0] = g["dxy"][0] * (g["xyelem"][0] + 0.3)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
    s = capi.NsSolver(g["xyelem"], g["xymin"], g["dxy"], *(g[k] for k in KEYS), bcs=_box_bcs(g))
    X, V, A = t(x.T.copy()), t(g["vel"].T.copy()), t(g["accel"].T.copy())
    P = t(np.zeros(len(g["mass"])))
    before = X.clone()
    with pytest.raises(capi.MpmError) as err:
        s.step(X, V, A, P, t(g["mass"]), t(g["vol"]), 0, 1.0)
    assert err.value.code == 4   # MPM_ERR_PARTICLE_OUT_OF_BOX
    assert torch.equal(X, before)
    s.close()
