"""Full-size FP64 fixtures from the reference itself, for the accuracy targets
stated at full size.

Runs the reference's own compiled translation units (oracle/_ref/libmpmref.so,
built by oracle/build_ref.sh from the reference checkout) on the full-size
seeded workloads and stores a seeded subsample of the particles' final state,
so that a GPU test can state the FP32 (and FP64) errors against the
reference's own FP64 path without running it:

    oracle/build_ref.sh <reference checkout> && python tests/golden/make_fullsize.py --spinning

--spinning   the 4,096,000-particle spinning block (80^3 cells on a 128^3 grid,
             dx = 4e-3 m, 8 particles per cell, the top quarter compressed to
             27 per cell, Gaussian velocities plus 10 rad/s about z), PIC,
             shifting on, 1000 steps of dt = 2e-6 s: about an hour on one core.
             Writes tests/golden/fullsize_spinning_block.npz.

--cantilever the 1,728,000-particle Neo-Hookean cantilever (60^3 cells on a
             64^3 grid, dx = 1e-2 m, 8 particles per cell, E = 1e7 Pa,
             nu = 0.3, x = 0 face clamped, dt = 1e-3 s), Newton with the
             implicit solid's own convergence test, 3 steps, each linear
             system solved to ||r||^2 < 1e-20 ||r0||^2 (far below the
             reference's default, so that the result does not depend on the
             Krylov method).  Runs the oracle's C restatement
             (oracle/mpm_oracle.c, which matches the reference's implicit
             solid bit for bit at equal tolerance, tests/test_oracle_golden.py)
             because the reference's GPBiCGSafe stops at its fixed 1e-8.
             Writes tests/golden/fullsize_cantilever.npz.

The fixture holds the sorted ids of 32,768 particles drawn without
replacement (seed 4242), their initial coordinates (a test checks that it
regenerated the same scene), their coordinates, velocities and Voigt stress
after the last step, and the FP64 totals over all particles (mass, momentum,
kinetic energy, first moment of position).
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "hpc-mpm-code_gb300"))

from mpm_gb300 import scenes  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
NSAMPLE = 32768
SAMPLE_SEED = 4242


def sample_ids(n):
    rng = np.random.default_rng(SAMPLE_SEED)
    return np.sort(rng.choice(n, size=NSAMPLE, replace=False)).astype(np.int64)


def totals(mass, x, v):
    return {"tot_mass": np.array(mass.sum()), "tot_momentum": (mass[:, None] * v).sum(axis=0),
            "tot_kinetic": np.array(0.5 * (mass * (v * v).sum(axis=1)).sum()),
            "tot_moment_x": (mass[:, None] * x).sum(axis=0)}


def spinning(nsteps=1000, chunk=50):
    s = scenes.spinning_block()
    ids = sample_ids(s.num)
    r = ref.RefSolid(s)
    t0 = time.time()
    done = 0
    while done < nsteps:
        k = min(chunk, nsteps - done)
        r.steps(k)
        done += k
        print(f"step {done}/{nsteps}  {time.time() - t0:.0f} s", flush=True)
    p = r.particles()
    out = {"ids": ids, "x0": s.coord[ids], "v0": s.vel[ids], "x": p["x"][ids], "v": p["v"][ids],
           "sigma": p["sigma"][ids], "nsteps": np.array(nsteps), "num": np.array(s.num),
           "seconds": np.array(time.time() - t0)}
    out.update(totals(s.mass, p["x"], p["v"]))
    out.update({f"init_{k}": v for k, v in totals(s.mass, s.coord, s.vel).items()})
    path = os.path.join(OUT, "fullsize_spinning_block.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def cantilever(nsteps=3, eps=1.0e-20):
    from oracle import port

    s = scenes.cantilever(iprop=1)
    ids = sample_ids(s.num)
    o = port.PortSolid(s, implicit=True, nr_flag=True)
    t0 = time.time()
    kt = nt = 0
    for k in range(nsteps):
        a, b = o.implicit_steps(1, eps=eps)
        kt += a
        nt += b
        print(f"step {k + 1}/{nsteps}  {time.time() - t0:.0f} s  krylov {a}  newton {b}", flush=True)
    p = o.particles()
    out = {"ids": ids, "x0": s.coord[ids], "x": p["x"][ids], "v": p["v"][ids], "sigma": p["sigma"][ids],
           "F": p["F"][ids], "nsteps": np.array(nsteps), "num": np.array(s.num), "eps": np.array(eps),
           "krylov": np.array(kt), "newton": np.array(nt), "seconds": np.array(time.time() - t0)}
    path = os.path.join(OUT, "fullsize_cantilever.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--spinning", action="store_true")
    ap.add_argument("--cantilever", action="store_true")
    ap.add_argument("--steps", type=int, default=1000)
    a = ap.parse_args()
    if a.cantilever:
        cantilever()
    if a.spinning:
        if not ref.available():
            raise SystemExit("oracle/_ref/libmpmref.so missing: run oracle/build_ref.sh <reference checkout> first")
        spinning(a.steps)
