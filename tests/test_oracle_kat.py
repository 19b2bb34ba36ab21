"""The oracle restatement against the same known answers as the GPU path
(tests/test_gpu_kat.py): free fall and uniform translation of a block that
touches no boundary, shifting off.  FP64: 1e-13 relative on v, 1e-13 m on x,
1e-13 on F - I, 1e-15 E on the stress."""
import numpy as np
import pytest

from mpm_gb300 import scenes
from oracle import port

E, DT, NSTEPS = 1.0e6, 1.0e-5, 50


def _block(gravity, v0, scheme):
    s = scenes.elastic_block(grid=(32, 32, 32), cell_lo=(10, 10, 10), cell_hi=(22, 22, 22), npc=2, jitter=0.1,
                             E=E, dt=DT, gravity=gravity, fix_bottom=False, scheme=scheme, name="kat_block")
    s.vel[:] = np.asarray(v0, dtype=np.float64)[None, :]
    return s


@pytest.mark.parametrize("gravity,scheme", [((0.0, 0.0, -9.81), scenes.PIC), ((0.0, 0.0, -9.81), scenes.FLIP),
                                            ((0.0, 0.0, 0.0), scenes.PIC)])
def test_oracle_known_answers(gravity, scheme):
    g = np.asarray(gravity)
    v0 = np.array([0.05, -0.02, 0.1])
    s = _block(gravity, v0, scheme)
    x0 = s.coord.copy()
    o = port.PortSolid(s, shifting=False)
    o.steps(NSTEPS)
    p = o.particles()
    n = NSTEPS
    v_want = v0 + n * DT * g
    x_want = x0 + n * DT * v0[None, :] + g[None, :] * DT * DT * n * (n + 1) / 2.0
    assert np.max(np.abs(p["v"] - v_want[None, :])) <= 1e-13 * np.max(np.abs(v_want))
    assert np.max(np.abs(p["x"] - x_want)) <= 1e-13
    assert np.max(np.abs(p["F"] - np.eye(3)[None, :, :])) <= 1e-13
    assert np.max(np.abs(p["sigma"])) <= 1e-15 * E


def test_oracle_p_wave_speed():
    """The oracle's compression front travels at sqrt((lambda + 2 mu) / rho)
    within 3 % (tests/kat_pwave.py)."""
    import kat_pwave as kp

    s = kp.bar()
    x0 = s.coord.copy()
    o = port.PortSolid(s, shifting=False)
    c = kp.measured_speed(o.steps, lambda: o.particles()["v"], x0)
    assert abs(c / kp.C_P - 1.0) <= 0.03, (c, kp.C_P)
