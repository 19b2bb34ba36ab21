"""Train the learned preconditioner for the implicit cantilever on the GPU.

Training pairs come from the implicit solver's own solves on the
1,728,000-particle cantilever (64^3-cell grid, 65^3 control points) in its
initial state (``trajectory_points`` > 1 spreads the systems over states
along its own motion, 12 implicit steps apart; on the 50-step run that gave
35.2 Krylov iterations per step against 34.4 for the committed parameters):
for moduli E drawn log-uniformly from [1e6, 1e8] and the system's own plus
seeded random loads, each system is solved twice and (residual, error)
pairs are stored along the second solve (mpm_gpu_implicit_harvest); a
second pass stores pairs along the learned solver's own iterations.  The network is then trained with
Adam by the library's own tensor-core forward and backward kernels
(mpm_nn_train).  The result is written as raw FP32 parameters plus a JSON
record of the run; bench.py and the tests load them through
``load_weights``.

    python -m mpm_gb300.train_precond            # 20,000 pairs, default schedule
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import capi, scenes

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "weights")
WEIGHTS = os.path.join(WEIGHTS_DIR, "precond_cantilever64.f32")


def load_weights(path=WEIGHTS):
    """The committed parameters (FP32) or None."""
    if not os.path.exists(path):
        return None
    p = np.fromfile(path, dtype=np.float32)
    return p if p.size == capi.load().mpm_nn_num_params() else None


def _along(gpu, npoints, steps_between, total, fn, log):
    """Calls fn(point, count) at npoints states of the solid's own
    trajectory (steps_between implicit steps apart, Jacobi-PCG), splitting
    `total` systems over them; the solid is advanced in between."""
    done = 0
    for k in range(npoints):
        count = (total - done) // (npoints - k)
        if k > 0 and steps_between > 0:
            gpu.implicit_steps(steps_between, eps=1.0e-16)
        if count > 0:
            fn(k, count)
        done += count


def train(pairs=20000, loads_per_system=8, pairs_per_load=25, epochs=8, batch=8, lr=1.0e-3, seed=0,
          harvest_eps=1.0e-20, learned_pairs=8000, learned_pairs_per_load=16, epochs2=4, scene=None, out=WEIGHTS,
          trajectory_points=1, steps_between=12, log=print):
    """Two passes: pairs along Jacobi-PCG solves, training; then (if
    learned_pairs > 0) pairs along the learned solver's own iterations with
    the first-pass network, and training on all pairs.  The systems are
    taken at `trajectory_points` states of the solid's own motion,
    `steps_between` implicit steps apart (the systems a run meets change as
    the body deforms)."""
    s = scene if scene is not None else scenes.cantilever(iprop=1)
    gpu = capi.GpuImplicitSolid(s, nr_flag=True)
    per_system = loads_per_system * pairs_per_load
    nsystems = max(1, math.ceil(pairs / per_system))
    net = capi.PrecondNet(s.xynodec, max_batch=batch, max_pairs=pairs + learned_pairs, seed=seed)
    t0 = time.perf_counter()
    _along(gpu, trajectory_points, steps_between, nsystems,
           lambda k, n: gpu.harvest(net, n, loads_per_system, pairs_per_load, 1.0e6, 1.0e8, seed=seed + 17 * k,
                                    eps=harvest_eps), log)
    t1 = time.perf_counter()
    n = net.num_pairs()
    log(f"harvested {n} pairs from {nsystems} systems in {t1 - t0:.1f} s")
    losses = net.train(epochs, batch, lr=lr, seed=seed)
    t2 = time.perf_counter()
    log(f"trained {epochs} epochs in {t2 - t1:.1f} s, loss per epoch {[round(float(x), 4) for x in losses]}")
    losses2, nsys2 = [], 0
    if learned_pairs > 0:
        nsys2 = max(1, math.ceil(learned_pairs / (loads_per_system * learned_pairs_per_load)))
        gpu.close()
        gpu = capi.GpuImplicitSolid(s, nr_flag=True)   # back to the initial state

        def harvest2(k, n):
            gpu.set_precond(net)
            gpu.harvest(net, n, loads_per_system, learned_pairs_per_load, 1.0e6, 1.0e8, seed=seed + 1 + 17 * k,
                        eps=harvest_eps)
            gpu.set_precond(None)

        _along(gpu, trajectory_points, steps_between, nsys2, harvest2, log)
        losses2 = net.train(epochs2, batch, lr=lr * 0.5, seed=seed + 1)
        log(f"second pass: {net.num_pairs()} pairs, {epochs2} epochs, loss per epoch "
            f"{[round(float(x), 4) for x in losses2]}")
    t3 = time.perf_counter()
    params = net.params()
    n = net.num_pairs()
    rec = {"scene": s.name, "particles": int(s.num), "nodes": list(s.xynodec), "pairs": int(n),
           "systems": nsystems, "loads_per_system": loads_per_system, "pairs_per_load": pairs_per_load,
           "learned_systems": nsys2, "learned_pairs_per_load": learned_pairs_per_load,
           "trajectory_points": trajectory_points, "steps_between": steps_between,
           "moduli": [1.0e6, 1.0e8], "epochs": epochs, "epochs2": epochs2, "batch": batch, "lr": lr, "seed": seed,
           "harvest_eps": harvest_eps, "loss_per_epoch": [float(x) for x in losses],
           "loss_per_epoch2": [float(x) for x in losses2],
           "harvest_s": t1 - t0, "train_s": t3 - t1}
    if out:
        os.makedirs(os.path.dirname(out), exist_ok=True)
        params.astype(np.float32).tofile(out)
        with open(out + ".json", "w") as f:
            json.dump(rec, f, indent=1)
    net.close()
    gpu.close()
    return params, rec


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1.0e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    train(pairs=a.pairs, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, out=a.out)


if __name__ == "__main__":
    main()
