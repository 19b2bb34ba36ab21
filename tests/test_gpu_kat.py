"""Known-answer tests of the CUDA explicit path (through the C ABI).

The reference ships no known-answer tests; these follow from the method
itself for a block that touches no boundary, has no boundary conditions
and runs with particle shifting off:

* free fall: with gravity g and no other load every node's acceleration is
  g, so after n steps of size dt every particle has v = v0 + n g dt and, since
  the position update uses the re-projected (MUSL) velocity of the new step,
  x = x0 + n dt v0 + g dt^2 n (n + 1) / 2 (PIC and FLIP alike);
* uniform translation: without gravity a uniform velocity stays uniform and
  x = x0 + n dt v0;
* in both cases the velocity field is uniform, so the deformation gradient
  stays the identity and the stress zero up to the rounding of the shape
  function gradients (which sum to zero only to the working precision).

Tolerances: FP64 1e-12 relative on v, 1e-12 m on x, 1e-12 on F - I,
1e-10 E on the stress; FP32 2e-5 relative on v (a few roundings per step,
50 steps), 1e-6 m on x, 1e-6 on F - I, 1e-6 E on the stress.
"""
import numpy as np
import pytest

from mpm_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

E = 1.0e6
DT = 1.0e-5
NSTEPS = 50
TOL = {64: dict(v=1e-12, x=1e-12, F=1e-12, s=1e-10), 32: dict(v=2e-5, x=1e-6, F=1e-6, s=1e-6)}


def _block(gravity, v0, scheme):
    s = scenes.elastic_block(grid=(32, 32, 32), cell_lo=(10, 10, 10), cell_hi=(22, 22, 22), npc=2, jitter=0.1,
                             E=E, dt=DT, gravity=gravity, fix_bottom=False, scheme=scheme, name="kat_block")
    s.vel[:] = np.asarray(v0, dtype=np.float64)[None, :]
    return s


def _run(s, precision):
    gpu = capi.GpuSolid(s, precision=precision, shifting=False)
    gpu.steps(NSTEPS)
    p = gpu.particles()
    gpu.sync()
    gpu.close()
    return p


def _check(p, s, v_want, x_want, precision):
    tol = TOL[precision]
    vscale = max(float(np.max(np.abs(v_want))), 1e-300)
    assert np.max(np.abs(p["v"] - v_want[None, :])) <= tol["v"] * vscale
    assert np.max(np.abs(p["x"] - x_want)) <= tol["x"]
    assert np.max(np.abs(p["F"] - np.eye(3)[None, :, :])) <= tol["F"]
    assert np.max(np.abs(p["sigma"])) <= tol["s"] * E


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("scheme", [scenes.PIC, scenes.FLIP])
def test_free_fall(precision, scheme):
    g = np.array([0.0, 0.0, -9.81])
    v0 = np.array([0.05, -0.02, 0.1])
    s = _block(tuple(g), v0, scheme)
    x0 = s.coord.copy()
    p = _run(s, precision)
    n = NSTEPS
    v_want = v0 + n * DT * g
    x_want = x0 + n * DT * v0[None, :] + g[None, :] * DT * DT * n * (n + 1) / 2.0
    _check(p, s, v_want, x_want, precision)


@pytest.mark.parametrize("precision", [64, 32])
def test_uniform_translation(precision):
    v0 = np.array([0.3, -0.1, 0.2])
    s = _block((0.0, 0.0, 0.0), v0, scenes.PIC)
    x0 = s.coord.copy()
    p = _run(s, precision)
    _check(p, s, v0, x0 + NSTEPS * DT * v0[None, :], precision)


@pytest.mark.parametrize("precision", [64, 32])
def test_p_wave_speed(precision):
    """The compression front of the driven bar (tests/kat_pwave.py) travels
    at sqrt((lambda + 2 mu) / rho) within 3 %, FP64 and FP32."""
    import kat_pwave as kp

    s = kp.bar()
    x0 = s.coord.copy()
    gpu = capi.GpuSolid(s, precision=precision, shifting=False)
    c = kp.measured_speed(gpu.steps, lambda: gpu.particles()["v"], x0)
    gpu.sync()
    gpu.close()
    assert abs(c / kp.C_P - 1.0) <= 0.03, (c, kp.C_P)


@pytest.mark.parametrize("scatter", [0, 1])
def test_fp32_particles_on_node_planes(scatter):
    """Particles whose x coordinate sits exactly on an FP32 grid plane
    (x = float(0.01 * i)), where FP32 rounding can put a particle on the far
    node of the cell it is binned in, in a linear velocity field: the shape
    gradients take their sign from the node, not from the sign of
    x - x_node, so the FP32 path stays within 1e-4 (v) and 1e-3 (F - I,
    stress) of the FP64 oracle after 5 steps (per-cell and staging-box
    scatter)."""
    from oracle import port

    s = scenes.elastic_block(grid=(32, 32, 32), cell_lo=(8, 8, 8), cell_hi=(24, 24, 24), npc=2, jitter=0.05,
                             E=E, dt=DT, gravity=(0.0, 0.0, 0.0), fix_bottom=False, scheme=scenes.PIC,
                             name="plane_block")
    planes = np.array([np.float32(np.float32(0.01) * np.float32(i)) for i in (10, 15, 20, 23)], dtype=np.float64)
    idx = np.argmin(np.abs(s.coord[:, 0:1] - planes[None, :]), axis=1)
    near = np.abs(s.coord[:, 0] - planes[idx]) < 0.004
    s.coord[near, 0] = planes[idx[near]]
    # a linear velocity field: the one-sided gradients of the two cells that
    # meet at a plane agree (a particle on a plane may be binned on either
    # side, in FP32 and FP64 differently), while a gradient with the wrong
    # sign would be about -2 v / dx, 16 times the field's gradient here
    L = np.array([[0.5, 0.2, 0.0], [-0.1, -0.3, 0.1], [0.0, 0.2, 0.4]])
    s.vel[:] = (s.coord - s.coord.mean(axis=0)) @ L.T
    o = port.PortSolid(s, shifting=False)
    o.steps(5)
    q = o.particles()
    gpu = capi.GpuSolid(s, precision=32, shifting=False, scatter=scatter)
    gpu.steps(5)
    p = gpu.particles()
    gpu.sync()
    gpu.close()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    H, Hq = p["F"] - np.eye(3)[None], q["F"] - np.eye(3)[None]
    e = {"v": rel(p["v"], q["v"]), "H": rel(H, Hq), "sigma": rel(p["sigma"], q["sigma"])}
    assert int(near.sum()) > 1000
    assert e["v"] <= 1e-4 and e["H"] <= 1e-3 and e["sigma"] <= 1e-3, e
