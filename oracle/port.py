"""ORACLE (test infrastructure only): ctypes driver for the plain-C FP64
restatement oracle/mpm_oracle.c (built to oracle/lib/libmpmoracle.so).

Only tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py may
use it, and only as the reference results are compared with / the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmpmoracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib_cache = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _lib():
    global _lib_cache
    if _lib_cache is not None:
        return _lib_cache
    if not os.path.exists(LIB_PATH):
        build()
    lib = C.CDLL(LIB_PATH)
    lib.mo_create.restype = C.c_void_p
    lib.mo_create.argtypes = [_ip, _dp, _dp, _ip, _ip, C.c_double, C.c_double, _dp, C.c_int, _ip, _dp]
    lib.mo_destroy.argtypes = [C.c_void_p]
    lib.mo_nodec.argtypes = [C.c_void_p]
    lib.mo_load.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _ip, C.c_int, C.c_int]
    lib.mo_set_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, _ip, _dp]
    lib.mo_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mo_explicit_p2g.argtypes = [C.c_void_p, C.c_double]
    lib.mo_explicit_steps.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.mo_get_nodal.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.mo_get_particles.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
    lib.mo_get_affine.argtypes = [C.c_void_p, _dp]
    lib.mo_set_fbar.argtypes = [C.c_void_p, C.c_int]
    lib.mo_get_fbar.argtypes = [C.c_void_p, _dp, _dp]
    lib.mo_shape.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _dp, _dp]
    lib.mo_implicit_setup.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.mo_implicit_nnzb.argtypes = [C.c_void_p]
    lib.mo_implicit_assemble.argtypes = [C.c_void_p, C.c_double]
    lib.mo_implicit_get_matrix.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp, _dp]
    lib.mo_implicit_matvec.argtypes = [C.c_void_p, _dp, _dp]
    lib.mo_implicit_solve.argtypes = [C.c_void_p, C.c_double, C.c_int, _dp]
    lib.mo_implicit_steps.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]
    _lib_cache = lib
    return lib


NODAL_FIELDS = {"nmass": (0, 1), "nvof": (1, 1), "nmome": (2, 3), "nforce": (3, 3), "nvel": (4, 3),
                "naccel": (5, 3), "nvol": (6, 1), "ndispl": (7, 3)}


class PortSolid:
    """Same interface as oracle.ref.RefSolid, on the C restatement."""

    def __init__(self, scene, implicit=False, shifting=True, nr_flag=False, spec_rad=1.0, fbar=False):
        self.lib = lib = _lib()
        self.scene = s = scene
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.ctx = lib.mo_create(i32(s.xyelem), f64(s.xymin), f64(s.dxy), i32(s.idimc), i32(s.npxye), s.dt, s.mtol,
                                 f64(s.gravity), len(s.iprop), i32(s.iprop), f64(s.mat_prop).ravel())
        self.nodec = lib.mo_nodec(self.ctx)
        lib.mo_load(self.ctx, s.num, f64(s.coord).ravel(), f64(s.vel).ravel(), f64(s.mass), f64(s.vol0),
                    i32(s.matid), s.scheme, int(shifting))
        for comp, nodes, vals in s.bcs:
            lib.mo_set_bc(self.ctx, comp, len(nodes), i32(nodes), f64(vals))
        if fbar:
            lib.mo_set_fbar(self.ctx, 1)
        if implicit:
            self.nmat = lib.mo_implicit_setup(self.ctx, int(nr_flag), float(spec_rad))

    def __del__(self):
        if getattr(self, "ctx", None):
            self.lib.mo_destroy(self.ctx)
            self.ctx = None

    def set_state(self, F=None, stress=None, vol=None):
        """Overwrite F (n, 3, 3), the Voigt stress (n, 6) and vol (n) of the loaded particles."""
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (F, stress, vol)]
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
        self.lib.mo_set_state(self.ctx, *(ptr(a) for a in keep))

    def steps(self, n, facl=1.0):
        self.lib.mo_explicit_steps(self.ctx, n, facl)

    def p2g(self, facl=1.0):
        self.lib.mo_explicit_p2g(self.ctx, facl)

    def implicit_steps(self, n, facl=1.0, eps=1.0e-8):
        kt, nt = C.c_int(0), C.c_int(0)
        self.lib.mo_implicit_steps(self.ctx, n, facl, eps, C.byref(kt), C.byref(nt))
        return kt.value, nt.value

    def nodal(self, name):
        fid, ncomp = NODAL_FIELDS[name]
        out = np.zeros(self.nodec * ncomp)
        self.lib.mo_get_nodal(self.ctx, fid, out)
        return out.reshape(ncomp, self.nodec) if ncomp == 3 else out

    def particles(self):
        n = self.scene.num
        x, v, F, sig, vol = (np.zeros(n * 3), np.zeros(n * 3), np.zeros(n * 9), np.zeros(n * 6), np.zeros(n))
        self.lib.mo_get_particles(self.ctx, x, v, F, sig, vol)
        return {"x": x.reshape(n, 3), "v": v.reshape(n, 3), "F": F.reshape(n, 3, 3), "sigma": sig.reshape(n, 6),
                "vol": vol}

    def fbar(self):
        """F-bar runs: def_grad_bar (n, 3, 3) and det_def_grad_bar (n,)."""
        n = self.scene.num
        F, J = np.zeros(n * 9), np.zeros(n)
        self.lib.mo_get_fbar(self.ctx, F, J)
        return F.reshape(n, 3, 3), J

    def affine(self):
        """TPIC / APIC: the affine velocity matrix per particle (n, 3, 3)."""
        n = self.scene.num
        out = np.zeros(n * 9)
        self.lib.mo_get_affine(self.ctx, out)
        return out.reshape(n, 3, 3)

    def shape(self, m, x):
        nc = np.zeros(27, dtype=np.int32)
        sf = np.zeros(27)
        dsf = np.zeros(81)
        ne = self.lib.mo_shape(self.ctx, m, np.ascontiguousarray(x, dtype=np.float64), nc, sf, dsf)
        return nc[:ne], sf[:ne], dsf[:3 * ne].reshape(ne, 3)

    # --- implicit -------------------------------------------------------------
    def assemble(self, facl=1.0):
        return self.lib.mo_implicit_assemble(self.ctx, facl)

    def matrix(self):
        nodec, nmat = self.nodec, self.nmat
        matrow = np.zeros(nodec + 1, dtype=np.int32)
        matcol = np.zeros(nmat, dtype=np.int32)
        amat = np.zeros(nmat * 9)
        adiag = np.zeros(nodec * 3)
        b = np.zeros(nodec * 3)
        self.lib.mo_implicit_get_matrix(self.ctx, matrow, matcol, amat, adiag, b)
        return matrow, matcol, amat.reshape(9, nmat), adiag, b

    def matvec(self, x):
        y = np.zeros(self.nodec * 3)
        self.lib.mo_implicit_matvec(self.ctx, np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def solve(self, eps=1.0e-8, kmax=10000):
        x = np.zeros(self.nodec * 3)
        it = self.lib.mo_implicit_solve(self.ctx, eps, kmax, x)
        return x, it
