"""ctypes binding of the C ABI in include/mpm_gpu.h (libmpm_gb300.so).

This is the binding a Python caller of the reference-facing API uses; the
tests and bench.py call the CUDA path through it.  There is no CPU fallback:
if the library is missing or a call fails, an exception is raised.

``GpuSolid`` keeps the reference's operator names (module/material_point.h,
module/solid/solid_material_point.h): ``MeshPointLinklist`` +
``Particle2Node`` -> ``p2g``, ``SolveSolid`` -> ``grid_update``,
``Node2Particle`` -> ``g2p``; ``steps`` runs the fused explicit step.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

MPM_PIC, MPM_FLIP = 0, 1
STATUS = {0: "ok", 1: "bad argument", 2: "out of device memory", 3: "non-finite particle state",
          4: "particle outside the grid", 5: "Krylov iteration limit", 6: "device wait timed out", 7: "CUDA error",
          8: "call out of order", 9: "unsupported configuration", 10: "Newton iteration did not converge"}


class MpmError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where}: {STATUS.get(code, code)} (status {code})")
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [("xyelem", C.c_int * 3), ("xymin", C.c_double * 3), ("dxy", C.c_double * 3),
                ("idimc", C.c_int * 3), ("npxye", C.c_int * 3)]


class NsParams(C.Structure):
    """mpm_ns_params: constants of the stabilized fluid (StabilizedMPM)."""
    _fields_ = [("rho", C.c_double), ("rmu", C.c_double), ("dt", C.c_double), ("beta_nb", C.c_double),
                ("gamma_nb", C.c_double), ("gravity", C.c_double * 3), ("facl", C.c_double), ("mtol", C.c_double)]


class MaterialDesc(C.Structure):
    _fields_ = [("nmat", C.c_int), ("iprop", C.POINTER(C.c_int)), ("mat_prop", C.POINTER(C.c_double))]


class Config(C.Structure):
    _fields_ = [("dt", C.c_double), ("mtol", C.c_double), ("gravity", C.c_double * 3), ("scheme", C.c_int),
                ("precision", C.c_int), ("shifting", C.c_int), ("resort_period", C.c_int), ("scatter", C.c_int),
                ("implicit", C.c_int), ("fbar", C.c_int), ("reserved", C.c_int * 5)]


class SolveStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int), ("krylov_iters", C.c_int), ("last_rel_residual", C.c_double),
                ("precond_fallbacks", C.c_int), ("nn_applications", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("num", C.c_int64), ("nodec", C.c_int64), ("steps", C.c_int64), ("resorts", C.c_int64),
                ("kernel_launches", C.c_int64), ("out_of_box", C.c_int64), ("tile_misses", C.c_int64),
                ("ntiles", C.c_int32), ("nwork", C.c_int32)]


_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

EXPORTS = ["mpm_gpu_create", "mpm_gpu_destroy", "mpm_gpu_set_stream", "mpm_gpu_status_string",
           "mpm_gpu_load_particles", "mpm_gpu_set_bc", "mpm_gpu_p2g", "mpm_gpu_grid_update", "mpm_gpu_g2p",
           "mpm_gpu_step_explicit", "mpm_gpu_download_nodal", "mpm_gpu_download_particles",
           "mpm_gpu_download_affine", "mpm_gpu_upload_affine", "mpm_gpu_download_fbar",
           "mpm_gpu_upload_particles", "mpm_gpu_steps_host", "mpm_gpu_sync",
           "mpm_gpu_get_stats", "mpm_gpu_enable_kernel_timing", "mpm_gpu_kernel_times", "mpm_gpu_implicit_setup",
           "mpm_gpu_implicit_step", "mpm_gpu_implicit_assemble", "mpm_gpu_implicit_get_system",
           "mpm_gpu_implicit_matvec", "mpm_gpu_implicit_solve", "mpm_gpu_p2g_noalloc", "mpm_gpu_ns_assemble", "mpm_gpu_autotune",
           "mpm_gpu_get_tuning", "mpm_nn_num_params", "mpm_nn_create", "mpm_nn_destroy", "mpm_nn_set_stream",
           "mpm_nn_init_params", "mpm_nn_set_linear", "mpm_nn_set_additive", "mpm_nn_set_symmetric", "mpm_nn_set_params", "mpm_nn_get_params", "mpm_nn_forward", "mpm_nn_backward",
           "mpm_nn_num_pairs", "mpm_nn_train", "mpm_gpu_implicit_set_precond", "mpm_gpu_implicit_harvest", "mpm_gpu_implicit_apply_precond",
           "mpm_gpu_set_graph", "mpm_gpu_set_tuning", "mpm_gpu_selftest_wait", "mpm_ns_create", "mpm_ns_destroy",
           "mpm_ns_set_stream", "mpm_ns_set_bc", "mpm_ns_solve", "mpm_ns_p2g", "mpm_ns_step", "mpm_ns_get_nodal",
           "mpm_ns_load_particles", "mpm_ns_particle2node", "mpm_ns_solve_ns", "mpm_ns_node2particle",
           "mpm_ns_download_particles"]


def load(path: str | None = None):
    """Load libmpm_gb300.so (building it in-tree first if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        _build.build()
    lib = C.CDLL(path)
    lib.mpm_gpu_create.argtypes = [C.POINTER(GridDesc), C.POINTER(MaterialDesc), C.POINTER(Config),
                                   C.POINTER(C.c_void_p)]
    lib.mpm_gpu_destroy.argtypes = [C.c_void_p]
    lib.mpm_gpu_destroy.restype = None
    lib.mpm_gpu_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.mpm_gpu_status_string.restype = C.c_char_p
    lib.mpm_gpu_status_string.argtypes = [C.c_int]
    lib.mpm_gpu_load_particles.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    lib.mpm_gpu_set_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, _ip, _dp]
    lib.mpm_gpu_p2g.argtypes = [C.c_void_p, C.c_double]
    lib.mpm_gpu_grid_update.argtypes = [C.c_void_p]
    lib.mpm_gpu_g2p.argtypes = [C.c_void_p]
    lib.mpm_gpu_step_explicit.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.mpm_gpu_download_nodal.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.mpm_gpu_download_particles.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
    lib.mpm_gpu_download_affine.argtypes = [C.c_void_p, _dp]
    lib.mpm_gpu_upload_affine.argtypes = [C.c_void_p, _dp]
    lib.mpm_gpu_download_fbar.argtypes = [C.c_void_p, _dp, _dp]
    lib.mpm_gpu_upload_particles.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
    lib.mpm_gpu_steps_host.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp]
    lib.mpm_gpu_sync.argtypes = [C.c_void_p]
    lib.mpm_gpu_selftest_wait.argtypes = [C.c_void_p, C.c_double]
    lib.mpm_gpu_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    lib.mpm_gpu_enable_kernel_timing.argtypes = [C.c_void_p, C.c_int]
    lib.mpm_gpu_autotune.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.mpm_gpu_set_graph.argtypes = [C.c_void_p, C.c_int]
    lib.mpm_gpu_set_tuning.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    lib.mpm_gpu_get_tuning.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.mpm_gpu_implicit_setup.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.mpm_gpu_implicit_step.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                                          C.POINTER(SolveStats)]
    lib.mpm_gpu_implicit_assemble.argtypes = [C.c_void_p, C.c_double]
    lib.mpm_gpu_implicit_get_system.argtypes = [C.c_void_p, _dp, _dp, _dp]
    lib.mpm_gpu_implicit_matvec.argtypes = [C.c_void_p, _dp, _dp]
    lib.mpm_gpu_implicit_solve.argtypes = [C.c_void_p, C.c_double, C.c_int, _dp, C.POINTER(C.c_int)]
    lib.mpm_gpu_kernel_times.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_char_p), _dp,
                                         C.POINTER(C.c_int64)]
    _fp = C.POINTER(C.c_float)
    lib.mpm_nn_num_params.restype = C.c_int64
    lib.mpm_nn_num_params.argtypes = []
    lib.mpm_nn_create.argtypes = [_ip, C.c_int, C.c_int64, C.POINTER(C.c_void_p)]
    lib.mpm_nn_destroy.argtypes = [C.c_void_p]
    lib.mpm_nn_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.mpm_nn_set_linear.argtypes = [C.c_void_p, C.c_int]
    lib.mpm_nn_set_additive.argtypes = [C.c_void_p, C.c_int]
    lib.mpm_nn_set_symmetric.argtypes = [C.c_void_p, C.c_int]
    lib.mpm_nn_init_params.argtypes = [C.c_void_p, C.c_uint64]
    lib.mpm_nn_set_params.argtypes = [C.c_void_p, _fp]
    lib.mpm_nn_get_params.argtypes = [C.c_void_p, _fp]
    lib.mpm_nn_forward.argtypes = [C.c_void_p, C.c_int, _fp, _fp]
    lib.mpm_nn_backward.argtypes = [C.c_void_p, C.c_int, _fp, _fp, _fp]
    lib.mpm_nn_num_pairs.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.mpm_nn_train.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_uint64, _fp]
    lib.mpm_gpu_implicit_set_precond.argtypes = [C.c_void_p, C.c_void_p]
    lib.mpm_gpu_implicit_apply_precond.argtypes = [C.c_void_p, _dp, _dp]
    lib.mpm_gpu_implicit_harvest.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                             C.c_double, C.c_uint64, C.c_double, C.c_int]
    _lib = lib
    return lib


def _chk(code, where):
    if code != 0:
        raise MpmError(code, where)


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, ty=_dp):
    return None if a is None else a.ctypes.data_as(ty)


NODAL = {"nmass": (0, 1), "nvof": (1, 1), "nmome": (2, 3), "nforce": (3, 3), "nvel": (4, 3), "naccel": (5, 3),
         "nvol": (6, 1)}


class GpuSolid:
    """One explicit solid on the GPU, built from a scene (mpm_gb300.scenes.Scene)."""

    def __init__(self, scene, precision=32, shifting=True, resort_period=0, scatter=0, stream=None, implicit=False,
                 fbar=False):
        self.lib = lib = load()
        self.scene = s = scene
        g = GridDesc((C.c_int * 3)(*s.xyelem), (C.c_double * 3)(*s.xymin), (C.c_double * 3)(*s.dxy),
                     (C.c_int * 3)(*s.idimc), (C.c_int * 3)(*s.npxye))
        self._iprop = np.ascontiguousarray(s.iprop, dtype=np.int32)
        self._mat = np.ascontiguousarray(s.mat_prop, dtype=np.float64).ravel()
        m = MaterialDesc(len(self._iprop), self._iprop.ctypes.data_as(_ip), self._mat.ctypes.data_as(_dp))
        cfg = Config(s.dt, s.mtol, (C.c_double * 3)(*s.gravity), s.scheme, precision, int(shifting),
                     int(resort_period), int(scatter), int(implicit), int(fbar), (C.c_int * 5)())
        h = C.c_void_p()
        _chk(lib.mpm_gpu_create(C.byref(g), C.byref(m), C.byref(cfg), C.byref(h)), "mpm_gpu_create")
        self.ctx = h
        self.nodec = s.nodec
        self.precision = precision
        if stream is not None:
            _chk(lib.mpm_gpu_set_stream(self.ctx, C.c_void_p(stream)), "mpm_gpu_set_stream")
        self.load(s.coord, s.vel, s.mass, s.vol0, matid=s.matid)
        for comp, nodes, vals in s.bcs:
            self.set_bc(comp, nodes, vals)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.mpm_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ---------------------------------------------------------------
    def load(self, coord, vel, mass, vol0, F=None, stress=None, matid=None):
        coord, vel, mass, vol0, F, stress = map(_d, (coord, vel, mass, vol0, F, stress))
        matid = None if matid is None else np.ascontiguousarray(matid, dtype=np.int32)
        n = mass.shape[0]
        self.num = n
        _chk(self.lib.mpm_gpu_load_particles(self.ctx, n, _ptr(coord), _ptr(vel), _ptr(mass), _ptr(vol0), _ptr(F),
                                             _ptr(stress), _ptr(matid, _ip)), "mpm_gpu_load_particles")

    def set_bc(self, comp, nodes, vals):
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        vals = _d(vals)
        _chk(self.lib.mpm_gpu_set_bc(self.ctx, comp, len(nodes), _ptr(nodes, _ip), _ptr(vals)), "mpm_gpu_set_bc")

    def set_stream(self, stream_handle):
        _chk(self.lib.mpm_gpu_set_stream(self.ctx, C.c_void_p(stream_handle)), "mpm_gpu_set_stream")

    # -- reference operator names -------------------------------------------
    def p2g(self, facl=1.0):
        _chk(self.lib.mpm_gpu_p2g(self.ctx, facl), "mpm_gpu_p2g")

    def grid_update(self):
        _chk(self.lib.mpm_gpu_grid_update(self.ctx), "mpm_gpu_grid_update")

    def g2p(self):
        _chk(self.lib.mpm_gpu_g2p(self.ctx), "mpm_gpu_g2p")

    Particle2Node = p2g
    SolveSolid = grid_update
    Node2Particle = g2p

    def steps(self, n, facl=1.0):
        _chk(self.lib.mpm_gpu_step_explicit(self.ctx, n, facl), "mpm_gpu_step_explicit")

    def sync(self):
        _chk(self.lib.mpm_gpu_sync(self.ctx), "mpm_gpu_sync")

    def sync_status(self):
        """mpm_gpu_sync's status code (0 ok) without raising."""
        return self.lib.mpm_gpu_sync(self.ctx)

    def selftest_wait(self, seconds):
        """Test hook: a bounded device wait that runs out after `seconds` (see mpm_gpu_selftest_wait)."""
        _chk(self.lib.mpm_gpu_selftest_wait(self.ctx, float(seconds)), "mpm_gpu_selftest_wait")

    # -- results ----------------------------------------------------------------
    def nodal(self, name):
        fid, ncomp = NODAL[name]
        out = np.zeros(self.nodec * ncomp)
        _chk(self.lib.mpm_gpu_download_nodal(self.ctx, fid, _ptr(out)), "mpm_gpu_download_nodal")
        return out.reshape(ncomp, self.nodec) if ncomp == 3 else out

    def particles(self):
        n = self.num
        x, v, F, sig, vol = (np.zeros(n * 3), np.zeros(n * 3), np.zeros(n * 9), np.zeros(n * 6), np.zeros(n))
        _chk(self.lib.mpm_gpu_download_particles(self.ctx, _ptr(x), _ptr(v), _ptr(F), _ptr(sig), _ptr(vol)),
             "mpm_gpu_download_particles")
        return {"x": x.reshape(n, 3), "v": v.reshape(n, 3), "F": F.reshape(n, 3, 3), "sigma": sig.reshape(n, 6),
                "vol": vol}

    def affine(self):
        """TPIC / APIC: the affine velocity matrix per particle (n, 3, 3), load order."""
        out = np.zeros(self.num * 9)
        _chk(self.lib.mpm_gpu_download_affine(self.ctx, _ptr(out)), "mpm_gpu_download_affine")
        return out.reshape(self.num, 3, 3)

    def fbar(self):
        """F-bar contexts: def_grad_bar (n, 3, 3) and det_def_grad_bar (n,), load order."""
        F, J = np.zeros(self.num * 9), np.zeros(self.num)
        _chk(self.lib.mpm_gpu_download_fbar(self.ctx, _ptr(F), _ptr(J)), "mpm_gpu_download_fbar")
        return F.reshape(self.num, 3, 3), J

    def upload_affine(self, affine):
        """TPIC / APIC: overwrite the affine matrices ((n, 3, 3) float64, load order)."""
        a = np.ascontiguousarray(affine, dtype=np.float64)
        _chk(self.lib.mpm_gpu_upload_affine(self.ctx, _ptr(a)), "mpm_gpu_upload_affine")

    def download_into(self, coord=None, vel=None, F=None, stress=None, vol=None):
        """Download into caller-provided C-contiguous float64 arrays (pinned for full speed)."""
        _chk(self.lib.mpm_gpu_download_particles(self.ctx, _ptr(coord), _ptr(vel), _ptr(F), _ptr(stress), _ptr(vol)),
             "mpm_gpu_download_particles")

    def steps_host(self, n, coord=None, vel=None, F=None, stress=None, vol=None, facl=1.0):
        """n explicit steps, each reading the state from and writing it back to
        the given C-contiguous float64 arrays (pinned for full speed)."""
        _chk(self.lib.mpm_gpu_steps_host(self.ctx, int(n), float(facl), _ptr(coord), _ptr(vel), _ptr(F), _ptr(stress),
                                         _ptr(vol)), "mpm_gpu_steps_host")

    def upload_state(self, coord=None, vel=None, F=None, stress=None, vol=None):
        """Overwrite particle state from float64 host arrays in load order."""
        _chk(self.lib.mpm_gpu_upload_particles(self.ctx, _ptr(coord), _ptr(vel), _ptr(F), _ptr(stress), _ptr(vol)),
             "mpm_gpu_upload_particles")

    def stats(self):
        st = Stats()
        _chk(self.lib.mpm_gpu_get_stats(self.ctx, C.byref(st)), "mpm_gpu_get_stats")
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def set_tuning(self, p2g_minb, musl_minb, update_ctas_per_sm):
        """Launch variants (0 = shared-memory staged kernel); see mpm_gpu_set_tuning."""
        _chk(self.lib.mpm_gpu_set_tuning(self.ctx, p2g_minb, musl_minb, update_ctas_per_sm), "mpm_gpu_set_tuning")

    def set_graph(self, on=True):
        """Replay blocks of fused steps from a captured CUDA graph (default on)."""
        _chk(self.lib.mpm_gpu_set_graph(self.ctx, int(on)), "mpm_gpu_set_graph")

    def autotune(self, steps_per_trial=5, facl=1.0):
        """Runs 3 x steps_per_trial explicit steps and keeps the fastest launch variants."""
        _chk(self.lib.mpm_gpu_autotune(self.ctx, steps_per_trial, facl), "mpm_gpu_autotune")
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _chk(self.lib.mpm_gpu_get_tuning(self.ctx, C.byref(a), C.byref(b), C.byref(c)), "mpm_gpu_get_tuning")
        return {"p2g_minb": a.value, "musl_minb": b.value, "update_ctas_per_sm": c.value}

    def enable_kernel_timing(self, on=True):
        _chk(self.lib.mpm_gpu_enable_kernel_timing(self.ctx, int(on)), "mpm_gpu_enable_kernel_timing")

    def kernel_times(self):
        cap = 16
        cnt = C.c_int(cap)
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        launches = (C.c_int64 * cap)()
        _chk(self.lib.mpm_gpu_kernel_times(self.ctx, C.byref(cnt), names, ms, launches), "mpm_gpu_kernel_times")
        return {names[i].decode(): (ms[i], launches[i]) for i in range(cnt.value)}


class GpuImplicitSolid(GpuSolid):
    """The implicit solid on the GPU; operator names of implicitmpm::SolidMaterialPoint.

    precision 64 (default): the FP64 operator (parity mode); 32: FP32
    particles, assembly, matrix and Krylov matvecs, with FP64 inner products,
    norms, true residual and Newton check."""

    def __init__(self, scene, nr_flag=False, spec_rad=1.0, shifting=True, stream=None, precision=64):
        super().__init__(scene, precision=precision, shifting=shifting, stream=stream, implicit=True)
        self.radius = tuple(int(o) for o in scene.idimc)
        self.nslots = int(np.prod([2 * r + 1 for r in self.radius]))
        _chk(self.lib.mpm_gpu_implicit_setup(self.ctx, int(nr_flag), float(spec_rad)), "mpm_gpu_implicit_setup")

    def implicit_steps(self, n, facl=1.0, eps=1.0e-8, kmax=10000, full=False):
        st = SolveStats()
        _chk(self.lib.mpm_gpu_implicit_step(self.ctx, n, facl, eps, kmax, C.byref(st)), "mpm_gpu_implicit_step")
        if full:
            return {k: getattr(st, k) for k, _ in SolveStats._fields_}
        return st.krylov_iters, st.newton_iters, st.last_rel_residual

    def set_precond(self, net):
        """Use a PrecondNet (or None: Jacobi) for the linear solves."""
        _chk(self.lib.mpm_gpu_implicit_set_precond(self.ctx, net.net if net is not None else None),
             "mpm_gpu_implicit_set_precond")
        self._net = net

    def apply_precond(self, r):
        """z = M(r) with the preconditioner set by set_precond (scaled system)."""
        r = _d(r)
        z = np.zeros(3 * self.nodec)
        _chk(self.lib.mpm_gpu_implicit_apply_precond(self.ctx, _ptr(r), _ptr(z)), "mpm_gpu_implicit_apply_precond")
        return z

    def harvest(self, net, nsystems, loads_per_system, pairs_per_load, e_min, e_max, seed=0, eps=1.0e-16,
                kmax=20000):
        """Training pairs for `net` from this solid's own Jacobi-PCG solves."""
        _chk(self.lib.mpm_gpu_implicit_harvest(self.ctx, net.net, nsystems, loads_per_system, pairs_per_load,
                                                 e_min, e_max, seed, eps, kmax), "mpm_gpu_implicit_harvest")

    def assemble(self, facl=1.0):
        _chk(self.lib.mpm_gpu_implicit_assemble(self.ctx, facl), "mpm_gpu_implicit_assemble")

    def system(self):
        """(stencil [ns][9][nodec], D^-1/2, RHS) of the last assembled system."""
        n = self.nodec
        A = np.zeros(self.nslots * 9 * n)
        d = np.zeros(3 * n)
        b = np.zeros(3 * n)
        _chk(self.lib.mpm_gpu_implicit_get_system(self.ctx, _ptr(A), _ptr(d), _ptr(b)), "mpm_gpu_implicit_get_system")
        return A.reshape(self.nslots, 9, n), d, b

    def matvec(self, x):
        x = _d(x)
        y = np.zeros(3 * self.nodec)
        _chk(self.lib.mpm_gpu_implicit_matvec(self.ctx, _ptr(x), _ptr(y)), "mpm_gpu_implicit_matvec")
        return y

    def solve(self, eps=1.0e-8, kmax=10000, download=True):
        """One linear solve of the assembled system from x = 0; returns (x, iterations),
        x None with download=False (the solution stays on the device)."""
        x = np.zeros(3 * self.nodec) if download else None
        it = C.c_int(0)
        _chk(self.lib.mpm_gpu_implicit_solve(self.ctx, eps, kmax, _ptr(x) if download else None, C.byref(it)),
             "mpm_gpu_implicit_solve")
        return x, it.value


def stencil_to_csr(stencil, xynodec, matrow, matcolid, radius=(1, 1, 1)):
    """Reorder [ns][E][nodec] stencil values (E = 9 for the solid's 3x3
    blocks, 16 for the fluid's 4x4 blocks; ns = prod(2 r + 1) slots for the
    stencil radius r per axis, the shape order: 27 for linear shape
    functions, 125 for quadratic B-splines, 75 for idimc 2 1 2) into the
    reference's CSR block-major layout amat[e][j] for the graph (matrow,
    matcolid) of CrsMat::BuildCrsMat."""
    nx, ny, nz = xynodec
    rx, ry, rz = radius
    sx, sy = 2 * rx + 1, 2 * ry + 1
    nodec = nx * ny * nz
    ne = stencil.shape[1]
    amat = np.zeros((ne, len(matcolid)))
    rows = np.repeat(np.arange(nodec), np.diff(matrow))
    cols = np.asarray(matcolid)
    ri, rj, rk = rows % nx, (rows // nx) % ny, rows // (nx * ny)
    ci, cj, ck = cols % nx, (cols // nx) % ny, cols // (nx * ny)
    slot = (ci - ri + rx) + sx * (cj - rj + ry) + sx * sy * (ck - rk + rz)
    for e in range(ne):
        amat[e] = stencil[slot, e, rows]
    return amat


_fp32 = C.POINTER(C.c_float)


class PrecondNet:
    """The learned preconditioner network (mpm_nn_*) on a grid of `nodes` control points."""

    def __init__(self, nodes, max_batch=1, max_pairs=0, seed=None, linear=True, additive=True, symmetric=False):
        self.lib = load()
        self.nodes = tuple(int(n) for n in nodes)
        n3 = (C.c_int * 3)(*self.nodes)
        h = C.c_void_p()
        _chk(self.lib.mpm_nn_create(n3, int(max_batch), int(max_pairs), C.byref(h)), "mpm_nn_create")
        self.net = h
        _chk(self.lib.mpm_nn_set_linear(self.net, int(linear)), "mpm_nn_set_linear")
        _chk(self.lib.mpm_nn_set_additive(self.net, int(additive)), "mpm_nn_set_additive")
        _chk(self.lib.mpm_nn_set_symmetric(self.net, int(symmetric)), "mpm_nn_set_symmetric")
        self.nvox = self.nodes[0] * self.nodes[1] * self.nodes[2]
        self.nparams = int(self.lib.mpm_nn_num_params())
        if seed is not None:
            _chk(self.lib.mpm_nn_init_params(self.net, int(seed)), "mpm_nn_init_params")

    def close(self):
        if getattr(self, "net", None):
            self.lib.mpm_nn_destroy(self.net)
            self.net = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _chk(self.lib.mpm_nn_set_params(self.net, p.ctypes.data_as(_fp32)), "mpm_nn_set_params")

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        _chk(self.lib.mpm_nn_get_params(self.net, p.ctypes.data_as(_fp32)), "mpm_nn_get_params")
        return p

    def forward(self, x):
        """x: [batch][nodes][6] float32 (residual, features) -> [batch][nodes][3]."""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.nvox, 6)
        out = np.zeros(x.shape[:2] + (3,), dtype=np.float32)
        _chk(self.lib.mpm_nn_forward(self.net, x.shape[0], x.ctypes.data_as(_fp32), out.ctypes.data_as(_fp32)),
             "mpm_nn_forward")
        return out

    def backward(self, x, gout):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.nvox, 6)
        g = np.ascontiguousarray(gout, dtype=np.float32).reshape(x.shape[:2] + (3,))
        grad = np.zeros(self.nparams, dtype=np.float32)
        _chk(self.lib.mpm_nn_backward(self.net, x.shape[0], x.ctypes.data_as(_fp32), g.ctypes.data_as(_fp32),
                                      grad.ctypes.data_as(_fp32)), "mpm_nn_backward")
        return grad

    def num_pairs(self):
        n = C.c_int64(0)
        _chk(self.lib.mpm_nn_num_pairs(self.net, C.byref(n)), "mpm_nn_num_pairs")
        return n.value

    def train(self, epochs, batch, lr=1.0e-3, seed=0):
        losses = np.zeros(epochs, dtype=np.float32)
        _chk(self.lib.mpm_nn_train(self.net, epochs, batch, lr, seed, losses.ctypes.data_as(_fp32)), "mpm_nn_train")
        return losses


def ns_assemble(xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol,
                x, mass, vol, nvel, naccel, ndispl, npres, nmass, stream=None):
    """One Newton system of StabilizedMPM::SolveNS (module/fluid/MPM/solve_ns_mpm.cpp:28-62)
    through mpm_gpu_ns_assemble.  Inputs are FP64 CUDA tensors: x (3, n) or
    (3*n,), mass and vol (n), nvel / naccel / ndispl (3*nodec, component-major),
    npres and nmass (nodec).  Returns (tau1, tau2, stencil [27][16][nodec],
    b_rhs [4*nodec]) as CUDA tensors; raises when a particle lies outside the
    grid or the call fails.  Waits for the stream before it returns."""
    import torch

    lib = load()
    lib.mpm_gpu_ns_assemble.argtypes = [C.POINTER(GridDesc), C.POINTER(NsParams), C.c_int64] + \
        [C.c_void_p] * 13 + [C.c_void_p]
    lib.mpm_gpu_ns_assemble.restype = C.c_int
    g = GridDesc()
    for d in range(3):
        g.xyelem[d] = int(xyelem[d])
        g.xymin[d] = float(xymin[d])
        g.dxy[d] = float(dxy[d])
        g.idimc[d] = 1
        g.npxye[d] = 2
    p = NsParams(rho, rmu, dt, beta, gamma, (C.c_double * 3)(*[float(v) for v in gravity]), facl, mtol)
    n = int(mass.numel())
    nodec = int(np.prod(np.asarray(xyelem) + 1))
    for t in (x, mass, vol, nvel, naccel, ndispl, npres, nmass):
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise ValueError("ns_assemble: inputs must be contiguous FP64 CUDA tensors")
    dev = mass.device
    tau1 = torch.empty(n, dtype=torch.float64, device=dev)
    tau2 = torch.empty(n, dtype=torch.float64, device=dev)
    st = torch.empty(27 * 16 * nodec, dtype=torch.float64, device=dev)
    b = torch.empty(4 * nodec, dtype=torch.float64, device=dev)
    status = torch.empty(1, dtype=torch.int32, device=dev)
    strm = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    rc = lib.mpm_gpu_ns_assemble(C.byref(g), C.byref(p), n, x.data_ptr(), mass.data_ptr(), vol.data_ptr(),
                                 nvel.data_ptr(), naccel.data_ptr(), ndispl.data_ptr(), npres.data_ptr(),
                                 nmass.data_ptr(), tau1.data_ptr(), tau2.data_ptr(), st.data_ptr(), b.data_ptr(),
                                 status.data_ptr(), C.c_void_p(strm))
    if rc != 0:
        raise RuntimeError("mpm_gpu_ns_assemble failed: " + lib.mpm_gpu_status_string(rc).decode())
    if int(status.item()) != 0:
        raise RuntimeError("mpm_gpu_ns_assemble: a particle lies outside the grid")
    return tau1, tau2, st.view(27, 16, nodec), b


class NsStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int), ("krylov_iters", C.c_int), ("r0r", C.c_double),
                ("last_residual", C.c_double), ("last_abs_residual", C.c_double)]


class NsSolver:
    """The stabilized fluid MPM of module/fluid/MPM/ on the GPU: SolveNS
    (solve_ns_mpm.cpp:28-62, mpm_ns_solve), Particle2Node (mpm_ns_p2g) and whole
    time steps Particle2Node + SolveNS + Node2Particle (var_trans_fluid.cpp,
    mpm_ns_step), through mpm_ns_create / mpm_ns_set_bc.  bcs: four
    (nodes, values) pairs for u, v, w, p (ubc, vbc, wbc, pbc)."""

    def __init__(self, xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol, bcs=None,
                 stream=None, npxye=(2, 2, 2)):
        import torch

        self.lib = lib = load()
        lib.mpm_ns_create.argtypes = [C.POINTER(GridDesc), C.POINTER(NsParams), C.POINTER(C.c_void_p)]
        lib.mpm_ns_destroy.argtypes = [C.c_void_p]
        lib.mpm_ns_destroy.restype = None
        lib.mpm_ns_set_stream.argtypes = [C.c_void_p, C.c_void_p]
        lib.mpm_ns_set_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, _ip, _dp]
        lib.mpm_ns_solve.argtypes = [C.c_void_p, C.c_int64] + [C.c_void_p] * 10 + [C.c_double, C.c_int,
                                                                                    C.POINTER(NsStats)]
        g = GridDesc()
        for d in range(3):
            g.xyelem[d] = int(xyelem[d])
            g.xymin[d] = float(xymin[d])
            g.dxy[d] = float(dxy[d])
            g.idimc[d] = 1
            g.npxye[d] = int(npxye[d])
        p = NsParams(rho, rmu, dt, beta, gamma, (C.c_double * 3)(*[float(v) for v in gravity]), facl, mtol)
        h = C.c_void_p()
        _chk(lib.mpm_ns_create(C.byref(g), C.byref(p), C.byref(h)), "mpm_ns_create")
        self.ns = h
        self.nodec = int(np.prod(np.asarray(xyelem) + 1))
        self.stream = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _chk(lib.mpm_ns_set_stream(self.ns, C.c_void_p(self.stream)), "mpm_ns_set_stream")
        for comp, (nodes, vals) in enumerate(bcs or []):
            self.set_bc(comp, nodes, vals)

    def set_bc(self, comp, nodes, vals):
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        _chk(self.lib.mpm_ns_set_bc(self.ns, comp, len(nodes), _ptr(nodes, _ip), _ptr(vals)), "mpm_ns_set_bc")

    def solve(self, x, mass, vol, nvel, naccel, nmass, rtol=1.0e-10, kmax=10000):
        """FP64 CUDA tensors as ns_assemble (x (3, n) or (3*n,)); returns
        (ndispl, npres, tau1, tau2) as CUDA tensors and the stats dict."""
        import torch

        for t in (x, mass, vol, nvel, naccel, nmass):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("NsSolver.solve: inputs must be contiguous FP64 CUDA tensors")
        dev = mass.device
        n = int(mass.numel())
        f = lambda k: torch.empty(k, dtype=torch.float64, device=dev)
        nd, npres, t1, t2 = f(3 * self.nodec), f(self.nodec), f(max(n, 1)), f(max(n, 1))
        st = NsStats()
        rc = self.lib.mpm_ns_solve(self.ns, n, x.data_ptr(), mass.data_ptr(), vol.data_ptr(), nvel.data_ptr(),
                                   naccel.data_ptr(), nmass.data_ptr(), nd.data_ptr(), npres.data_ptr(),
                                   t1.data_ptr(), t2.data_ptr(), float(rtol), int(kmax), C.byref(st))
        _chk(rc, "mpm_ns_solve")
        return (nd, npres, t1[:n], t2[:n]), {k: getattr(st, k) for k, _ in NsStats._fields_}

    def _step_args(self, x, vel, accel, mass, vol):
        import torch

        for t in (x, vel, accel, mass, vol):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("NsSolver: particle arrays must be contiguous FP64 CUDA tensors")
        n = int(mass.numel())
        for t in (x, vel, accel):
            if t.numel() != 3 * n:
                raise ValueError("NsSolver: x, vel, accel hold three blocks of n values")
        return n

    def p2g(self, x, vel, accel, mass, vol, scheme=0, facl=1.0):
        """StabilizedMPM::Particle2Node (mpm_ns_p2g) into the context's nodal
        state; x, vel, accel (3, n) FP64 CUDA tensors, mass, vol (n)."""
        lib = self.lib
        lib.mpm_ns_p2g.argtypes = [C.c_void_p, C.c_int64] + [C.c_void_p] * 5 + [C.c_int, C.c_double]
        n = self._step_args(x, vel, accel, mass, vol)
        _chk(lib.mpm_ns_p2g(self.ns, n, x.data_ptr(), vel.data_ptr(), accel.data_ptr(), mass.data_ptr(),
                            vol.data_ptr(), int(scheme), float(facl)), "mpm_ns_p2g")

    def step(self, x, vel, accel, pres, mass, vol, scheme=0, facl=1.0, rtol=1.0e-10, kmax=10000):
        """One fluid time step (mpm_ns_step: Particle2Node, SolveNS,
        Node2Particle) updating x, vel, accel (3, n) and pres (n) in place;
        returns the stats dict of its Newton loop."""
        lib = self.lib
        lib.mpm_ns_step.argtypes = [C.c_void_p, C.c_int64] + [C.c_void_p] * 6 + [C.c_int, C.c_double, C.c_double,
                                                                                  C.c_int, C.POINTER(NsStats)]
        n = self._step_args(x, vel, accel, mass, vol)
        st = NsStats()
        _chk(lib.mpm_ns_step(self.ns, n, x.data_ptr(), vel.data_ptr(), accel.data_ptr(), pres.data_ptr(),
                             mass.data_ptr(), vol.data_ptr(), int(scheme), float(facl), float(rtol), int(kmax),
                             C.byref(st)), "mpm_ns_step")
        return {k: getattr(st, k) for k, _ in NsStats._fields_}

    # --- the reference's three member calls on particles the context holds
    def load_particles(self, coord, vel, accel, mass, vol):
        """mpm_ns_load_particles from host arrays (coord, vel, accel (n, 3); mass, vol (n))."""
        self.lib.mpm_ns_load_particles.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp]
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._host = [f(coord), f(vel), f(accel), f(mass), f(vol)]
        _chk(self.lib.mpm_ns_load_particles(self.ns, len(self._host[3]), *[_ptr(a) for a in self._host]),
             "mpm_ns_load_particles")
        self.np = len(self._host[3])

    def particle2node(self, scheme=0, facl=1.0):
        self.lib.mpm_ns_particle2node.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _chk(self.lib.mpm_ns_particle2node(self.ns, int(scheme), float(facl)), "mpm_ns_particle2node")

    def solve_ns(self, rtol=1.0e-10, kmax=10000):
        self.lib.mpm_ns_solve_ns.argtypes = [C.c_void_p, C.c_double, C.c_int, C.POINTER(NsStats)]
        st = NsStats()
        _chk(self.lib.mpm_ns_solve_ns(self.ns, float(rtol), int(kmax), C.byref(st)), "mpm_ns_solve_ns")
        return {k: getattr(st, k) for k, _ in NsStats._fields_}

    def node2particle(self):
        self.lib.mpm_ns_node2particle.argtypes = [C.c_void_p]
        _chk(self.lib.mpm_ns_node2particle(self.ns), "mpm_ns_node2particle")

    def download_particles(self):
        """x, v, a (n, 3) and pres (n) of the particles the context holds."""
        self.lib.mpm_ns_download_particles.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        n = self.np
        x, v, a, p = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        _chk(self.lib.mpm_ns_download_particles(self.ns, _ptr(x), _ptr(v), _ptr(a), _ptr(p)),
             "mpm_ns_download_particles")
        return dict(x=x, v=v, a=a, pres=p)

    NODAL = {"nmass": (0, 1), "nvof": (1, 1), "nvel": (2, 3), "naccel": (3, 3), "ndispl": (4, 3), "npres": (5, 1),
             "nvol": (6, 1)}

    def nodal(self, name):
        """The context's nodal field after p2g / step (mpm_ns_get_nodal) as a host array."""
        field, comps = self.NODAL[name]
        out = np.zeros(comps * self.nodec)
        self.lib.mpm_ns_get_nodal.argtypes = [C.c_void_p, C.c_int, _dp]
        _chk(self.lib.mpm_ns_get_nodal(self.ns, field, _ptr(out)), "mpm_ns_get_nodal")
        return out

    def close(self):
        if getattr(self, "ns", None):
            self.lib.mpm_ns_destroy(self.ns)
            self.ns = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
