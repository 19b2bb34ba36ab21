"""Benchmark of the GB300 MPM transfer path: explicit solid MPM, particle-steps/s.

Workload (default): the 4,096,000-particle spinning elastic block on a 128^3
grid (dx = 4e-3 m, 80^3 cells at 8 particles per cell, the top quarter
squeezed to 27 per cell, Gaussian + rigid-rotation velocities), FP32, PIC,
dt = 2e-6 s.  Seeded synthetic data; the reference publishes no dataset.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

* value      K fused explicit steps (mpm_gpu_step_explicit) with the particle
             state resident in HBM, timed with CUDA events on the library's
             stream between a barrier + synchronize on both sides; the
             particle state (393 MB) is larger than L2.
* e2e        the same steps through the reference-facing C ABI with host
             buffers: per step the FP64 particle state is uploaded from
             pinned host memory (mpm_gpu_upload_particles), one step runs,
             and the state is downloaded (mpm_gpu_download_particles).
* roofline   the whole explicit step against the measured HBM copy
             bandwidth, with the algorithmic bytes N_p*176 + N_n*56 per step.
* accuracy   the FP32 path's x, v and sigma after the workload's 1000 steps
             against the reference's own FP64 run of the same seeded
             workload (a committed 32,768-particle subsample), relative L2.
* cpu_baseline / --impl reference: the CPU restatement of the reference's
             algorithm (oracle/mpm_oracle.c, pinned bit-exact to the
             reference's own compiled code) on a bounded sample.
N > 1: independent replicas, one per GPU (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "hpc-mpm-code_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s"
WORKLOAD = "explicit solid MPM, spinning elastic block, 4,096,000 particles, 128^3 grid, FP32, PIC"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false",
                    help="skip the 1000-step FP32 run checked against the reference's full-size fixture")
    ap.add_argument("--batched-steps", type=int, default=100,
                    help="steps of the 256-scene batched workload (0 skips)")
    ap.add_argument("--fluid-steps", type=int, default=100,
                    help="steps of the 12.6M-particle Tait dam break (0 skips)")
    ap.add_argument("--apic-steps", type=int, default=100,
                    help="steps of the headline workload with APIC transfers (0 skips)")
    ap.add_argument("--fbar-steps", type=int, default=100,
                    help="steps of the headline workload with the F-bar projection (0 skips)")
    ap.add_argument("--train-pairs", type=int, default=2000,
                    help="training pairs when no committed preconditioner parameters exist")
    ap.add_argument("--implicit-steps", type=int, default=50,
                    help="implicit cantilever steps timed per solver after the explicit run (50: the mean over 50 steps; 0 skips)")
    ap.add_argument("--cells", type=int, default=80,
                    help="block edge in cells (80 = the 4,096,000-particle workload; smaller for profiling)")
    return ap.parse_args()


def workload(cells):
    from mpm_gb300 import scenes

    if cells == 80:
        return scenes.spinning_block()
    return scenes.spinning_block(grid=(cells + 48,) * 3, cell_lo=(24, 24, 24), cells=(cells,) * 3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def max_over_ranks(value, world, device="cpu"):
    """Largest value over the ranks (the slowest replica's time); identity at N = 1."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(num, steps, ms_max, world):
    """Whole-job particle-steps/s of `world` independent replicas timed by the slowest one."""
    return world * num * steps / (ms_max * 1e-3)


def algorithmic_bytes(num, nodec):
    # per explicit step, FP32: 23 words read + 21 written per particle, 7 nodal words written + read
    return num * 176 + nodec * 56


def cpu_baseline(scene, steps):
    """The oracle restatement on this host, one core, a bounded sample of the same workload."""
    from oracle import port

    o = port.PortSolid(scene)
    o.steps(1)   # warm-up (page-in, first linked list)
    t0 = time.perf_counter()
    o.steps(steps)
    dt = time.perf_counter() - t0
    value = scene.num * steps / dt
    return {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"{steps} FP64 steps of the full {scene.num}-particle workload ({dt:.1f} s)"}


def _reference_worker(cells, W, K, start, out):
    """One process of the reference arm: W untimed and K timed FP64 explicit
    steps of its own block of the workload; waits on `start` so that all
    processes time the same interval."""
    from oracle import port

    s = workload(cells)
    o = port.PortSolid(s)
    o.steps(W)
    start.wait()
    t0 = time.perf_counter()
    o.steps(K)
    out.put((s.num, time.perf_counter() - t0))


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's algorithm on
    all of this host's cores.

    The reference parallelises its explicit solid by MPI ranks, each owning a
    slab of the domain (one core each; its MPI+PETSc build cannot be
    produced on this host).  Here each core runs one process with its own
    block of the workload (same dx, dt, particle density, velocity field and
    compressed quarter) through the oracle restatement, FP64, with the block
    edge chosen so that W + K steps take about a minute of one core; the value is all
    processes' particle-steps over the slowest process's time, an upper bound
    for the MPI build (no halo exchange between the blocks).
    """
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import port

    K, W = max(1, args.steps), max(0, args.warmup)
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    probe = workload(24)
    o = port.PortSolid(probe)
    o.steps(1)
    t0 = time.perf_counter()
    o.steps(2)
    rate = probe.num * 2 / (time.perf_counter() - t0)
    del o
    budget = 60.0   # seconds of one core; the processes share the memory bandwidth, so allow about 2x
    cells = int(((budget * rate) / (8.0 * (K + W))) ** (1.0 / 3.0))
    cells = max(8, min(args.cells, cells - cells % 4))
    ctx = mp.get_context("spawn")
    start, out = ctx.Event(), ctx.Queue()
    procs = [ctx.Process(target=_reference_worker, args=(cells, W, K, start, out)) for _ in range(cores)]
    for pr in procs:
        pr.start()
    time.sleep(1.0)
    # every process finishes its warm-up before the clock starts: each has
    # built its block and run W steps when it reaches start.wait()
    start.set()
    res = [out.get() for _ in procs]
    for pr in procs:
        pr.join()
    total = sum(n for n, _ in res)
    dt = max(t for _, t in res)
    v = total * K / dt
    per = res[0][0]
    sample = (f"{K} FP64 explicit steps of a {cells}^3-cell block ({per} particles) of the workload in each of "
              f"{cores} processes, one per core ({dt:.1f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles_per_step_sample": total, "grid": list(workload(cells).xyelem),
                       "processes": cores},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_implicit(args, torch, stream):
    """The implicit solid: 1,728,000-particle Neo-Hookean cantilever on a 64^3 grid,
    E = 1e7 Pa, nu = 0.3, dt = 1e-3 s, Newton + Krylov solved to a relative
    residual of 1e-8 (eps = 1e-16 on squared norms).  For the FP32 operator (the
    record's top level) and the FP64 one ("fp64"), two solids each from the same
    initial state: Jacobi-PCG, and flexible GCR with the learned preconditioner
    (committed parameters trained by mpm_gb300.train_precond, else a short
    on-the-spot training run, stated in the record)."""
    from mpm_gb300 import capi, scenes, train_precond

    s = scenes.cantilever(iprop=1)

    def timed(gpu):
        gpu.implicit_steps(1, eps=1.0e-16)           # warm-up step
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t0 = time.perf_counter()
        st = gpu.implicit_steps(args.implicit_steps, eps=1.0e-16, full=True)
        ev1.record(stream)
        ev1.synchronize()
        ms = max(ev0.elapsed_time(ev1), (time.perf_counter() - t0) * 1e3) / args.implicit_steps
        return ms, st

    def timed_solve(gpu, reps=3):
        """The linear solve alone: the system of the solid's current state, assembled
        once, solved from x = 0 to the same tolerance `reps` times."""
        gpu.assemble()
        gpu.solve(eps=1.0e-16, download=False)       # warm-up (graphs captured)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t0 = time.perf_counter()
        its = [gpu.solve(eps=1.0e-16, download=False)[1] for _ in range(reps)]
        ev1.record(stream)
        ev1.synchronize()
        return max(ev0.elapsed_time(ev1), (time.perf_counter() - t0) * 1e3) / reps, its[-1]

    params = train_precond.load_weights()
    training = "committed parameters (" + os.path.basename(train_precond.WEIGHTS) + ")"
    if params is None:
        params, rec = train_precond.train(pairs=args.train_pairs, epochs=2, out=None, log=lambda *_: None)
        training = (f"trained in this run: {rec['pairs']} pairs, {rec['epochs']} epochs, "
                    f"{rec['harvest_s'] + rec['train_s']:.0f} s")
    # algorithmic FLOPs of one network application: sum over the five 3x3x3
    # convolutions of output nodes x 2 x 27 x C_in x C_out (real channels)
    n0 = list(s.xynodec)
    n1 = [m // 2 + 1 for m in n0]
    n2 = [m // 2 + 1 for m in n1]
    v0, v1, v2 = (int(np.prod(v)) for v in (n0, n1, n2))
    flops = 2 * 27 * (v0 * 6 * 16 + v1 * 16 * 32 + v2 * 32 * 64 + v2 * 64 * 32 + v1 * 32 * 16)
    tc_peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            tc_peak = json.load(f).get("bf16_tflops")
    except (OSError, ValueError):
        pass

    def arms(prec):
        """Jacobi-PCG and the learned solver from the same initial state, for the
        FP32 operator (prec 32) or the FP64 one (prec 64)."""
        gpu = capi.GpuImplicitSolid(s, nr_flag=True, stream=stream.cuda_stream, precision=prec)
        jac_ms, jac = timed(gpu)
        gpu.enable_kernel_timing(True)
        gpu.implicit_steps(1, eps=1.0e-16)
        kt_j = gpu.kernel_times()   # per-kernel-class time of one more step (timers run without graphs)
        gpu.enable_kernel_timing(False)
        jac_solve_ms, jac_solve_it = timed_solve(gpu)
        gpu.close()
        net = capi.PrecondNet(s.xynodec)
        net.set_params(params)
        gpu = capi.GpuImplicitSolid(s, nr_flag=True, stream=stream.cuda_stream, precision=prec)
        gpu.set_precond(net)
        nn_ms, nn = timed(gpu)
        nn_solve_ms, nn_solve_it = timed_solve(gpu)
        # one application of the network: CUDA-event kernel timers over one more
        # solve (timers run the solve without graphs; the per-class time is the
        # network's kernels, from the input scaling to the output layer)
        gpu.enable_kernel_timing(True)
        gpu.solve(eps=1.0e-16, download=False)
        kt = gpu.kernel_times()
        gpu.enable_kernel_timing(False)
        gpu.sync()
        nn_app_ms = kt["precond_nn"][0] / max(kt["precond_nn"][1], 1) if "precond_nn" in kt else None
        gpu.close()
        net.close()
        out = {"metric": "implicit step time", "value": jac_ms, "unit": "ms/step", "higher_is_better": False,
               "steps": args.implicit_steps, "particles": s.num, "grid": list(s.xyelem),
               "dtype": "f32" if prec == 32 else "f64",
               "operator": ("FP32 particles, assembly, matrix and Krylov matvecs; FP64 Krylov dots and norms, "
                            "true residual (FP32 matrix in FP64 arithmetic) and Newton check") if prec == 32
               else "FP64 throughout",
               "solver": "Newton + Jacobi (symmetric diagonal scaling) CG to a true ||r||/||r0|| <= 1e-8",
               "krylov_iters_per_step": jac["krylov_iters"] / args.implicit_steps,
               "newton_iters_per_step": jac["newton_iters"] / args.implicit_steps,
               "kernel_ms_one_jacobi_step": {k: round(v[0], 4) for k, v in kt_j.items()}}
        out["learned"] = {"value": nn_ms, "unit": "ms/step",
                          "solver": "Newton + flexible GCR(4) with the learned right preconditioner (linear BF16 "
                                    "tcgen05 conv encoder-decoder, z = r + N r) while each 8-iteration window "
                                    "halves the residual, then CG with Jacobi; true FP64 residual <= 1e-8",
                          "krylov_iters_per_step": nn["krylov_iters"] / args.implicit_steps,
                          "newton_iters_per_step": nn["newton_iters"] / args.implicit_steps,
                          "fallbacks": nn["precond_fallbacks"], "network_applications": nn["nn_applications"],
                          "training": training,
                          "speedup_vs_jacobi": jac_ms / nn_ms if nn_ms > 0 else None,
                          "target_speedup": 2.0}
        if nn_app_ms:
            ach = flops / (nn_app_ms * 1e-3) / 1e12
            out["learned"]["network"] = {
                "us_per_application": nn_app_ms * 1e3, "flops_per_application": flops,
                "roofline": {"bound": "tensor", "achieved": ach, "peak": tc_peak, "unit": "TFLOP/s",
                             "frac": ach / tc_peak if tc_peak else None,
                             "note": "latency-bound: the five convolutions run on 65^3, 33^3 and 17^3 grids "
                                     "out of L2; the tensor pipe is 7-13 % busy (ncu)"}}
        out["solve"] = {"what": "one linear solve of the assembled system after the timed steps, from x = 0 to "
                                "||r||/||r0|| <= 1e-8, solution left on the device",
                        "jacobi_ms": jac_solve_ms, "jacobi_iters": jac_solve_it,
                        "learned_ms": nn_solve_ms, "learned_iters": nn_solve_it,
                        "speedup": jac_solve_ms / nn_solve_ms if nn_solve_ms > 0 else None}
        return out

    out = arms(32)
    out["fp64"] = arms(64)
    return out


def timed_steps(torch, stream, gpu, steps):
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gpu.steps(steps)
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1)


def run_batched(args, torch, stream, hbm_peak):
    """256 independent elastic scenes (log-uniform 1e3..1e5 particles, grids 32^3..64^3,
    E log-uniform 1e5..1e7) packed into one grid and advanced by one context: one
    launch per kernel and step for all scenes, blocks of steps replayed from a CUDA
    graph, launch variants picked by the autotuner.  FP32, shifting off."""
    from mpm_gb300 import capi, scenes

    b = scenes.pack_scenes(scenes.batch_scenes())
    s = b.scene
    gpu = capi.GpuSolid(s, precision=32, shifting=False, stream=stream.cuda_stream)
    tune = gpu.autotune(3)
    gpu.steps(args.warmup)
    gpu.sync()
    ms = timed_steps(torch, stream, gpu, args.batched_steps)
    gpu.sync()
    gpu.close()
    ms_step = ms / args.batched_steps
    nodes = int(sum(sc.nodec for sc in b.scenes))
    alg = algorithmic_bytes(s.num, nodes)
    return {"metric": METRIC, "value": s.num * args.batched_steps / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms_step, "steps": args.batched_steps, "scenes": len(b.scenes), "particles": s.num,
            "scene_nodes": nodes, "packed_grid": list(s.xyelem), "dtype": "f32", "tuning": tune,
            "roofline": {"bound": "hbm", "achieved": alg / (ms_step * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": alg / (ms_step * 1e-3) / 1e9 / hbm_peak,
                         "algorithmic_bytes_per_step": alg}}


def run_fluid(args, torch, stream, hbm_peak):
    """Tait-fluid dam break: 12,582,912 particles (128x128x96-cell column at 8 per cell)
    in a 256x128x128-cell box, dx = 4e-3 m, c0 = 30 m/s, gamma = 7, mu = 1e-3 Pa s,
    slip walls, dt = 5e-6 s, FP32."""
    from mpm_gb300 import capi, scenes

    s = scenes.dam_break()
    gpu = capi.GpuSolid(s, precision=32, stream=stream.cuda_stream)
    gpu.steps(args.warmup)
    gpu.sync()
    ms = timed_steps(torch, stream, gpu, args.fluid_steps)
    gpu.sync()
    gpu.close()
    ms_step = ms / args.fluid_steps
    alg = s.num * 64 + s.nodec * 56    # read x3 v3 m V0 J, write x3 v3 J; 7 nodal words written + read
    return {"metric": METRIC, "value": s.num * args.fluid_steps / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms_step, "steps": args.fluid_steps, "particles": s.num, "grid": list(s.xyelem),
            "dtype": "f32",
            "roofline": {"bound": "hbm", "achieved": alg / (ms_step * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": alg / (ms_step * 1e-3) / 1e9 / hbm_peak, "algorithmic_bytes_per_step": alg,
                         "note": "fluid formula N_p*64 + N_n*56; the fluid keeps J - 1 in place of the 9-field deformation gradient, and the stress (6 fields) that the P2G reads"}}


def run_apic(args, torch, stream, hbm_peak):
    """The headline spinning block with APIC transfers (MapScheme APIC): each
    particle also carries its 3x3 affine velocity matrix; the transfers run on
    the generic brick kernels (affine P2G; gather, scale and MUSL launches).
    FP32."""
    from mpm_gb300 import capi, scenes

    s = workload(args.cells)
    s.scheme = scenes.APIC
    gpu = capi.GpuSolid(s, precision=32, stream=stream.cuda_stream)
    gpu.steps(args.warmup)
    gpu.sync()
    ms = timed_steps(torch, stream, gpu, args.apic_steps)
    gpu.sync()
    gpu.close()
    ms_step = ms / args.apic_steps
    alg = algorithmic_bytes(s.num, s.nodec) + s.num * 72   # + the affine matrix read and written (9 + 9 words)
    return {"metric": METRIC, "value": s.num * args.apic_steps / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms_step, "steps": args.apic_steps, "particles": s.num, "scheme": "APIC", "dtype": "f32",
            "roofline": {"bound": "hbm", "achieved": alg / (ms_step * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": alg / (ms_step * 1e-3) / 1e9 / hbm_peak, "algorithmic_bytes_per_step": alg,
                         "note": "N_p*(176 + 72) + N_n*56: the solid formula plus the affine matrix"}}


def run_fbar(args, torch, stream, hbm_peak):
    """The headline spinning block with the F-bar projection on (Fbar_flag):
    per step a trial-J pass, the nodal projection of J vol, and the generic
    particle update with the J-bar gather.  FP32."""
    from mpm_gb300 import capi

    s = workload(args.cells)
    gpu = capi.GpuSolid(s, precision=32, stream=stream.cuda_stream, fbar=True)
    gpu.steps(args.warmup)
    gpu.sync()
    ms = timed_steps(torch, stream, gpu, args.fbar_steps)
    gpu.sync()
    gpu.close()
    ms_step = ms / args.fbar_steps
    alg = algorithmic_bytes(s.num, s.nodec) + s.num * 40   # + def_grad_bar and J-bar read and written (10 + 10 words)
    return {"metric": METRIC, "value": s.num * args.fbar_steps / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms_step, "steps": args.fbar_steps, "particles": s.num, "fbar": True, "dtype": "f32",
            "roofline": {"bound": "hbm", "achieved": alg / (ms_step * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": alg / (ms_step * 1e-3) / 1e9 / hbm_peak, "algorithmic_bytes_per_step": alg,
                         "note": "N_p*(176 + 40) + N_n*56: the solid formula plus def_grad_bar and J-bar"}}


def fullsize_accuracy(capi, stream, path):
    """Relative L2 errors of x, v and sigma of the FP32 path after the
    workload's full step count, on the fixture's particle subsample, against
    the reference's FP64 run."""
    g = np.load(path)
    s = workload(80)
    ids = g["ids"]
    if s.num != int(g["num"]) or not np.array_equal(s.coord[ids], g["x0"]):
        return {"error": "the fixture was made from a different scene"}
    gpu = capi.GpuSolid(s, precision=32, stream=stream.cuda_stream)
    nsteps = int(g["nsteps"])
    gpu.steps(nsteps)
    p = gpu.particles()
    gpu.sync()
    gpu.close()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out = {"vs": "the reference's FP64 run of the same workload (tests/golden/fullsize_spinning_block.npz)",
           "metric": "relative L2 over the subsample", "steps": nsteps, "sample": int(ids.size)}
    out.update({k: rel(p[k][ids], g[k]) for k in ("x", "v", "sigma")})
    return out


def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from mpm_gb300 import build, capi

    build.build()
    s = workload(args.cells)
    stream = torch.cuda.Stream()
    gpu = capi.GpuSolid(s, precision=32, stream=stream.cuda_stream)
    hbm_peak, peak_kind = measured_peaks()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # warm-up
    gpu.steps(args.warmup)
    gpu.sync()
    launches0 = gpu.stats()["kernel_launches"]
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        gpu.steps(args.steps)
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    gpu.sync()
    ms = ev0.elapsed_time(ev1)
    launches = gpu.stats()["kernel_launches"] - launches0
    ms = max_over_ranks(ms, world, "cuda")
    ms_step = ms / args.steps
    value = replica_throughput(s.num, args.steps, ms, world)

    # per-kernel device time over a second timed window (events around every kernel)
    gpu.enable_kernel_timing(True)
    ksteps = min(args.steps, 100)
    gpu.steps(ksteps)
    kt = gpu.kernel_times()
    gpu.enable_kernel_timing(False)
    gpu.sync()
    kernels = {k: {"ms_per_step": v[0] / ksteps, "launches": v[1]} for k, v in kt.items() if v[1]}
    ktot = sum(k["ms_per_step"] for k in kernels.values())
    for k in kernels.values():
        k["share"] = k["ms_per_step"] / ktot if ktot else None

    alg = algorithmic_bytes(s.num, s.nodec)
    achieved = alg / (ms_step * 1e-3) / 1e9
    # DRAM bytes per step of this workload from the full-size ncu capture
    # summarised in profiles/ (dram__bytes_read.sum + dram__bytes_write.sum of
    # every kernel of the step, the re-sort over its period)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "explicit_step_traffic_spinning_block_4M.json")
    if args.cells == 80 and os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("dram_bytes_per_step")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "kernel": "one explicit step (p2g, grid1, g2p_musl, grid2, g2p_update, amortised re-sort)",
                "algorithmic_bytes_per_step": alg, "peak_source": peak_kind}

    # end to end through the C ABI with host buffers
    n = s.num
    pin = lambda *shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hx, hv, hF, hs, hvol = pin(n, 3), pin(n, 3), pin(n, 9), pin(n, 6), pin(n)
    gpu.download_into(hx, hv, hF, hs, hvol)
    e_steps = max(1, args.e2e_steps)
    gpu.upload_state(hx, hv, hF, hs, hvol)
    gpu.steps(1)
    gpu.download_into(hx, hv, hF, hs, hvol)
    barrier()
    t0 = time.perf_counter()
    ev0.record(stream)
    gpu.steps_host(e_steps, hx, hv, hF, hs, hvol)   # every step: state in from and out to the host arrays
    ev1.record(stream)
    ev1.synchronize()
    e_ms = max(ev0.elapsed_time(ev1), (time.perf_counter() - t0) * 1e3)
    barrier()
    e_ms = max_over_ranks(e_ms, world, "cuda")
    state_bytes = n * 8 * (3 + 3 + 9 + 6 + 1)
    e2e = {"value": replica_throughput(n, e_steps, e_ms, world), "unit": METRIC, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": e_steps,
           "call": "mpm_gpu_steps_host: per step the particle state uploaded from and downloaded into FP64 host "
                   "arrays in pinned memory, the copies pipelined piece by piece on two copy streams"}
    gpu.sync()

    # accuracy of the FP32 path after the workload's 1000 steps against the
    # reference's own FP64 run of the same seeded workload, stored as a fixture
    # (a subsample of the particles; tests/golden/make_fullsize.py)
    accuracy = None
    fx_path = os.path.join(ROOT, "tests", "golden", "fullsize_spinning_block.npz")
    if args.cells == 80 and rank == 0 and args.accuracy and os.path.exists(fx_path):
        try:
            accuracy = fullsize_accuracy(capi, stream, fx_path)
        except Exception as exc:   # reported, never required
            accuracy = {"error": str(exc)}

    implicit = None
    if args.implicit_steps > 0:
        try:
            implicit = run_implicit(args, torch, stream)
        except Exception as exc:   # reported, never required
            implicit = {"metric": "implicit step time", "value": None, "error": str(exc)}

    batched = fluid = apic = fbar = None
    if args.fbar_steps > 0:
        try:
            fbar = run_fbar(args, torch, stream, hbm_peak)
        except Exception as exc:
            fbar = {"metric": METRIC, "value": None, "error": str(exc)}
    if args.apic_steps > 0:
        try:
            apic = run_apic(args, torch, stream, hbm_peak)
        except Exception as exc:
            apic = {"metric": METRIC, "value": None, "error": str(exc)}
    if args.batched_steps > 0:
        try:
            batched = run_batched(args, torch, stream, hbm_peak)
        except Exception as exc:
            batched = {"metric": METRIC, "value": None, "error": str(exc)}
    if args.fluid_steps > 0:
        try:
            fluid = run_fluid(args, torch, stream, hbm_peak)
        except Exception as exc:
            fluid = {"metric": METRIC, "value": None, "error": str(exc)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(s, args.cpu_steps)
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": METRIC, "cores": 1, "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD if args.cells == 80 else f"{WORKLOAD} (block of {args.cells}^3 cells)",
                           "particles": s.num, "grid": list(s.xyelem), "nodes": s.nodec,
                           "dt": s.dt, "scheme": "PIC", "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2: 393 MB particle state per step, no flush"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks.summary(),
                "gpu_launches": int(launches), "kernels": kernels, "implicit": implicit,
                "batched": batched, "fluid": fluid, "apic": apic, "fbar": fbar, "accuracy": accuracy}
        print(json.dumps(line), flush=True)
    gpu.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
