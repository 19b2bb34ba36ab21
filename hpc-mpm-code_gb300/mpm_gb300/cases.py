"""Focused runs of one workload each, for profiling with ncu.

    python -m mpm_gb300.cases explicit [--cells 64] [--steps 20]
    python -m mpm_gb300.cases implicit [--steps 1] [--precision 32]  # Jacobi-PCG Newton steps, 1.728M-particle cantilever
    python -m mpm_gb300.cases precond  [--steps 1] [--precision 32]  # the same with the learned preconditioner
    python -m mpm_gb300.cases ns       [--reps 3]        # stabilized-fluid Newton solves (SolveNS), filled box
    python -m mpm_gb300.cases ns_assemble [--cells 56] [--reps 3]  # stabilized-fluid systems, cells^3 block at 8 per cell
    python -m mpm_gb300.cases network  [--reps 10]       # network forward passes on the 65^3 grid
    python -m mpm_gb300.cases batched  [--steps 20]      # 256 packed scenes
    python -m mpm_gb300.cases fluid    [--steps 20] [--cells 128]  # Tait dam break, a cells x cells x 3/4 cells column (128: 12.6M particles)
    python -m mpm_gb300.cases apic     [--cells 64] [--steps 20]   # the explicit block with APIC transfers
    python -m mpm_gb300.cases fbar     [--cells 64] [--steps 20]   # the explicit block with the F-bar projection

Each case builds its scene, runs a few warm-up steps, then the requested
steps on a non-default stream, and exits 0.  Nothing is timed here: the
numbers come from the profiler or from bench.py.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import capi, scenes


def _stream():
    import torch

    return torch.cuda.Stream()


def run(case, steps, cells, reps, precision=64):
    st = _stream()
    if case in ("explicit", "apic", "fbar"):
        s = scenes.spinning_block(cells=(cells, cells, cells),
                                  grid=(cells + 48, cells + 48, cells + 48))
        if case == "apic":
            s.scheme = scenes.APIC
        g = capi.GpuSolid(s, precision=32, stream=st.cuda_stream, fbar=(case == "fbar"))
        g.steps(3)
        g.steps(steps)
        g.sync()
    elif case in ("implicit", "precond"):
        s = scenes.cantilever(iprop=1)
        g = capi.GpuImplicitSolid(s, nr_flag=True, stream=st.cuda_stream, precision=precision)
        if case == "precond":
            from . import train_precond

            p = train_precond.load_weights()
            if p is None:
                sys.exit("no committed preconditioner parameters")
            net = capi.PrecondNet(s.xynodec)
            net.set_params(p)
            g.set_precond(net)
        g.implicit_steps(1, eps=1.0e-16)
        g.implicit_steps(steps, eps=1.0e-16)
        g.sync()
    elif case == "network":
        net = capi.PrecondNet((65, 65, 65), seed=1)
        x = np.random.default_rng(0).normal(size=(1, 65 ** 3, 6)).astype(np.float32)
        for _ in range(reps):
            net.forward(x)
    elif case == "ns":
        import os
        import torch

        sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                        "tests", "golden"))
        import make_golden

        c = make_golden.ns_box_inputs(xyelem=(24, 20, 16), seed=9, amp=0.2)
        bcs = [(c["bc_wall"], np.zeros(len(c["bc_wall"])))] * 3 + [(c["bc_top"], np.zeros(len(c["bc_top"])))]
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
        ns = capi.NsSolver(c["xyelem"], c["xymin"], c["dxy"], c["rho"], c["rmu"], c["dt"], c["beta"], c["gamma"],
                           c["gravity"], c["facl"], c["mtol"], bcs=bcs, stream=st.cuda_stream)
        args = [t(c["x"].T.copy()), t(c["mass"]), t(c["vol"]), t(c["nvel"]), t(c["naccel"]), t(c["nmass"])]
        for _ in range(reps):
            ns.solve(*args)
        ns.close()
    elif case == "ns_assemble":
        import torch

        ne = cells + 20
        dx = 1.0 / ne
        rng = np.random.default_rng(9)
        lo = 10
        cl = np.stack(np.meshgrid(*[np.arange(lo, lo + cells)] * 3, indexing="ij"), -1).reshape(-1, 3)
        sub = np.array([(i, j, k) for k in range(2) for j in range(2) for i in range(2)])
        x = ((cl[:, None, :] + (sub[None] + 0.5) / 2.0).reshape(-1, 3) +
             rng.uniform(-0.2, 0.2, (len(cl) * 8, 3)) / 2) * dx
        n, N = len(x), (ne + 1) ** 3
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda:0")
        vol = np.full(n, dx ** 3 / 8)
        args = [t(x.T.copy()), t(1000.0 * vol), t(vol), t(rng.normal(0, 0.5, 3 * N)), t(rng.normal(0, 2, 3 * N)),
                t(rng.normal(0, 1e-3 * dx, 3 * N)), t(rng.normal(0, 50, N)), t(rng.uniform(0, 0.2, N))]
        with torch.cuda.stream(st):
            for _ in range(reps):
                capi.ns_assemble((ne,) * 3, (0.0,) * 3, (dx,) * 3, 1000.0, 0.05, 1e-3, 0.25, 0.5, (0.0, 0.0, -9.8),
                                 1.0, 1e-12, *args, stream=st.cuda_stream)
        torch.cuda.synchronize()
    elif case == "batched":
        b = scenes.pack_scenes(scenes.batch_scenes())
        g = capi.GpuSolid(b.scene, precision=32, shifting=False, stream=st.cuda_stream)
        g.steps(3)
        g.steps(steps)
        g.sync()
    elif case == "fluid":
        scene = scenes.dam_break() if cells >= 128 else scenes.dam_break(
            grid=(2 * cells, cells, cells), cells=(cells, cells, 3 * cells // 4))
        g = capi.GpuSolid(scene, precision=32, stream=st.cuda_stream)
        g.steps(3)
        g.steps(steps)
        g.sync()
    else:
        sys.exit(f"unknown case {case}")


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--cells", type=int, default=None,
                    help="block edge in cells (explicit / apic / fbar: 64; fluid: 128, the full dam break)")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--precision", type=int, default=64, choices=[32, 64])
    a = ap.parse_args()
    cells = a.cells if a.cells is not None else (128 if a.case == "fluid" else 64)
    run(a.case, a.steps, cells, a.reps, a.precision)


if __name__ == "__main__":
    main()
