"""Shared set-up of the P-wave known-answer tests (oracle and GPU).

A bar of 64 x 4 x 4 cells (8 particles per cell, no jitter) with every grid
node's y and z velocity fixed to zero (one-dimensional strain), its x = 0
face driven at a constant velocity v0 and no gravity: a compression front
runs down the bar at the P-wave speed c_p = sqrt((lambda + 2 mu) / rho).
The front is where the cross-section mean of v_x falls to v0 / 2; its speed
is measured between steps 300 and 600 (so the start-up near the driven face
drops out) and compared with c_p.
"""
import numpy as np

from mpm_gb300 import scenes

E, NU, RHO, DX, DT, V0 = 1.0e6, 0.3, 1000.0, 1.0e-2, 2.0e-5, 0.01
N1, N2 = 300, 600
C_P = float(np.sqrt(E * (1.0 - NU) / ((1.0 + NU) * (1.0 - 2.0 * NU)) / RHO))


def bar():
    s = scenes.elastic_block(grid=(72, 4, 4), dx=DX, cell_lo=(0, 0, 0), cell_hi=(64, 4, 4), npc=2, jitter=0.0, E=E,
                             nu=NU, rho=RHO, dt=DT, gravity=(0.0, 0.0, 0.0), fix_bottom=False, scheme=scenes.PIC,
                             name="pwave_bar")
    alln = np.arange(s.nodec, dtype=np.int32)
    s.bcs.append((scenes.BC_V, alln, np.zeros(s.nodec)))
    s.bcs.append((scenes.BC_W, alln, np.zeros(s.nodec)))
    left = scenes.face_nodes(s.xynodec, 0, 0)
    s.bcs.append((scenes.BC_U, left, np.full(left.shape[0], V0)))
    return s


def front(v, x0):
    """Material x at which the cross-section mean of v_x falls to V0 / 2."""
    xs = np.unique(x0[:, 0])
    prof = np.array([v[x0[:, 0] == x, 0].mean() for x in xs])
    i = int(np.argmax(prof < 0.5 * V0))
    assert i > 0, "no front"
    x1, x2, v1, v2 = xs[i - 1], xs[i], prof[i - 1], prof[i]
    return x1 + (0.5 * V0 - v1) * (x2 - x1) / (v2 - v1)


def measured_speed(run_steps, velocities, x0):
    run_steps(N1)
    f1 = front(velocities(), x0)
    run_steps(N2 - N1)
    f2 = front(velocities(), x0)
    return (f2 - f1) / ((N2 - N1) * DT)
