"""Shared set-up of the angular-momentum tests of the affine transfers
(oracle and GPU).

A free elastic block (no gravity, no boundary condition, shifting off)
spinning rigidly about z at OMEGA.  The affine matrix of TPIC / APIC starts
at zero, so the first step transfers like PIC and loses part of the spin;
from then on the affine transfers carry the particles' velocity gradient to
the grid and the block's angular momentum about its centre of mass stays
constant to the time-integration error, while PIC (no affine term) keeps
losing it step after step.  With linear shape functions APIC's B D^-1 equals
TPIC's velocity gradient (the multilinear basis reproduces affine fields), so
the two schemes give the same state to rounding.
"""
import numpy as np

from mpm_gb300 import scenes

OMEGA, DT = 20.0, 1.0e-5


def block(scheme, cells=12, margin=6):
    n = cells + 2 * margin
    s = scenes.elastic_block(grid=(n, n, n), cell_lo=(margin,) * 3, cell_hi=(margin + cells,) * 3, npc=2,
                             jitter=0.1, E=1.0e6, dt=DT, gravity=(0.0, 0.0, 0.0), fix_bottom=False, scheme=scheme,
                             name="spin_block")
    c = s.coord.mean(axis=0)
    s.vel[:] = OMEGA * np.cross([0.0, 0.0, 1.0], s.coord - c)
    return s


def angular_momentum_z(mass, x, v):
    """L_z about the centre of mass."""
    r = x - (mass[:, None] * x).sum(axis=0) / mass.sum()
    return float(np.sum(mass * (r[:, 0] * v[:, 1] - r[:, 1] * v[:, 0])))
