"""ORACLE (test infrastructure only): ctypes driver for oracle/_ref/libmpmref.so.

libmpmref.so is the reference's own compiled C++ (module/*.cpp of
HPC-MPM-Code) plus oracle/ref_harness.cpp, built by oracle/build_ref.sh in
the development container only (the reference checkout is not present
anywhere else).  It is used to generate the committed golden fixtures
(tests/golden/make_golden.py) and, where present, as the CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libmpmref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def available() -> bool:
    return os.path.exists(LIB_PATH)


def _lib():
    lib = C.CDLL(LIB_PATH)
    lib.ref_setup.argtypes = [_ip, _dp, _dp, _ip, _ip, C.c_double, C.c_double, _dp, C.c_int, _ip, _dp]
    lib.ref_explicit_init.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _ip, C.c_int, C.c_int]
    lib.ref_set_bc.argtypes = [C.c_int, C.c_int, _ip, _dp]
    lib.ref_explicit_steps.argtypes = [C.c_int, C.c_double]
    lib.ref_explicit_p2g.argtypes = [C.c_double]
    lib.ref_get_nodal.argtypes = [C.c_int, _dp]
    lib.ref_get_particles.argtypes = [_dp, _dp, _dp, _dp, _dp]
    lib.ref_get_affine.argtypes = [_dp]
    lib.ref_io_read.argtypes = [C.c_char_p, C.c_char_p, _ip, _dp]
    lib.ref_io_bc.argtypes = [C.c_int, _ip, _dp]
    lib.ref_io_particles.argtypes = [_ip, _ip, _ip, _dp, _dp]
    lib.ref_restart_output.argtypes = [C.c_char_p]
    lib.ref_restart_input.argtypes = [C.c_char_p]
    lib.ref_set_fbar.argtypes = [C.c_int]
    lib.ref_get_fbar.argtypes = [_dp, _dp]
    lib.ref_implicit_init.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _ip, C.c_int, C.c_int, C.c_double]
    lib.ref_implicit_steps.argtypes = [C.c_int, C.c_double]
    lib.ref_implicit_assemble.argtypes = [C.c_double]
    lib.ref_implicit_get_matrix.argtypes = [_ip, _ip, _dp, _dp, _dp]
    lib.ref_implicit_matvec.argtypes = [_dp, _dp]
    lib.ref_implicit_solve.argtypes = [_dp]
    return lib


NODAL_FIELDS = {"nmass": (0, 1), "nvof": (1, 1), "nmome": (2, 3), "nforce": (3, 3), "nvel": (4, 3),
                "naccel": (5, 3), "nvol": (6, 1), "ndispl": (7, 3)}


def read_decks(grid_path, point_path):
    """The reference's own readers (InputParaGriddata + BCInput x3 +
    InputPointData) on a grid and a particle deck: what they parsed."""
    lib = _lib()
    ints = np.zeros(20, dtype=np.int32)
    dbl = np.zeros(12)
    assert lib.ref_io_read(grid_path.encode(), point_path.encode(), ints, dbl) == 0
    out = {"ints": ints.copy(), "dbl": dbl.copy()}
    for k in range(3):
        n = int(ints[16 + k])
        nodes, vals = np.zeros(max(n, 1), dtype=np.int32), np.zeros(max(n, 1))
        lib.ref_io_bc(k, nodes, vals)
        out[f"bc{k}_nodes"], out[f"bc{k}_vals"] = nodes[:n], vals[:n]
    n = int(ints[19])
    idv, mat, surf = (np.zeros(n, dtype=np.int32) for _ in range(3))
    mass, vol0 = np.zeros(n), np.zeros(n)
    lib.ref_io_particles(idv, mat, surf, mass, vol0)
    x = np.zeros(3 * n)
    lib.ref_get_particles(x, np.zeros(3 * n), np.zeros(9 * n), np.zeros(6 * n), np.zeros(n))
    out.update({"coord": x.reshape(n, 3), "id": idv, "matid": mat, "surf": surf, "mass": mass, "vol0": vol0})
    return out


class RefSolid:
    """One reference solid (explicit restated driver or implicit as-is)."""

    def __init__(self, scene, implicit=False, shifting=True, nr_flag=False, spec_rad=1.0, fbar=False):
        self.lib = _lib()
        self.lib.ref_set_fbar(int(fbar))
        self.scene = s = scene
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.nodec = self.lib.ref_setup(i32(s.xyelem), f64(s.xymin), f64(s.dxy), i32(s.idimc), i32(s.npxye),
                                        s.dt, s.mtol, f64(s.gravity), len(s.iprop), i32(s.iprop),
                                        f64(s.mat_prop).ravel())
        args = (s.num, f64(s.coord).ravel(), f64(s.vel).ravel(), f64(s.mass), f64(s.vol0), i32(s.matid), s.scheme)
        if implicit:
            self.nmat = self.lib.ref_implicit_init(*args, int(nr_flag), float(spec_rad))
        else:
            self.lib.ref_explicit_init(*args, int(shifting))
        for comp, nodes, vals in s.bcs:
            self.lib.ref_set_bc(comp, len(nodes), i32(nodes), f64(vals))

    def steps(self, n, facl=1.0):
        assert self.lib.ref_explicit_steps(n, facl) == 0

    def p2g(self, facl=1.0):
        assert self.lib.ref_explicit_p2g(facl) == 0

    def implicit_steps(self, n, facl=1.0):
        assert self.lib.ref_implicit_steps(n, facl) == 0

    def nodal(self, name):
        fid, ncomp = NODAL_FIELDS[name]
        out = np.zeros(self.nodec * ncomp)
        self.lib.ref_get_nodal(fid, out)
        return out.reshape(ncomp, self.nodec) if ncomp == 3 else out

    def particles(self):
        n = self.scene.num
        x, v, F, sig, vol = (np.zeros(n * 3), np.zeros(n * 3), np.zeros(n * 9), np.zeros(n * 6), np.zeros(n))
        self.lib.ref_get_particles(x, v, F, sig, vol)
        return {"x": x.reshape(n, 3), "v": v.reshape(n, 3), "F": F.reshape(n, 3, 3), "sigma": sig.reshape(n, 6),
                "vol": vol}

    def fbar(self):
        """F-bar runs: def_grad_bar (n, 3, 3) and det_def_grad_bar (n,)."""
        n = self.scene.num
        F, J = np.zeros(n * 9), np.zeros(n)
        assert self.lib.ref_get_fbar(F, J) == n
        return F.reshape(n, 3, 3), J

    def restart_output(self, prefix):
        """SolidMaterialPointBase::RestartOutput to prefix + "0_re.txt"."""
        assert self.lib.ref_restart_output(prefix.encode()) == 0

    def restart_input(self, prefix):
        """SolidMaterialPointBase::RestartInput from prefix + "0_re.txt"."""
        assert self.lib.ref_restart_input(prefix.encode()) == self.scene.num

    def affine(self):
        """TPIC / APIC: the affine velocity matrix per particle (n, 3, 3)."""
        n = self.scene.num
        out = np.zeros(n * 9)
        assert self.lib.ref_get_affine(out) == n
        return out.reshape(n, 3, 3)

    # --- implicit solid hooks -------------------------------------------------
    def assemble(self, facl=1.0):
        return self.lib.ref_implicit_assemble(facl)

    def matrix(self):
        nodec, nmat = self.nodec, self.nmat
        matrow = np.zeros(nodec + 1, dtype=np.int32)
        matcol = np.zeros(nmat, dtype=np.int32)
        amat = np.zeros(nmat * 9)
        adiag = np.zeros(nodec * 3)
        b = np.zeros(nodec * 3)
        self.lib.ref_implicit_get_matrix(matrow, matcol, amat, adiag, b)
        return matrow, matcol, amat.reshape(9, nmat), adiag, b

    def matvec(self, x):
        y = np.zeros(self.nodec * 3)
        self.lib.ref_implicit_matvec(np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def solve(self):
        x = np.zeros(self.nodec * 3)
        it = self.lib.ref_implicit_solve(x)
        return x, it


class RefFluid:
    """The reference's stabilizedmpm::StabilizedMPM (module/fluid/MPM/) on one
    rank, through oracle/_ref: one Newton system of SolveNS on a given nodal
    state (MakNSStabCoeff, PredictNewmarkBetaVelAndAccel, AssembleNSSystem)."""

    def __init__(self, xyelem, xymin, dxy, dt, mtol, gravity, x, mass, vol, rho, rmu, beta, gamma):
        lib = self.lib = _lib()
        lib.ref_ns_init.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double]
        lib.ref_ns_assemble.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp]
        lib.ref_ns_get_matrix.argtypes = [_ip, _ip, _dp, _dp]
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.nodec = lib.ref_setup(i32(xyelem), f64(xymin), f64(dxy), i32([1, 1, 1]), i32([2, 2, 2]), float(dt),
                                   float(mtol), f64(gravity), 1, i32([0]), f64([0.0, 0.0, 0.0]))
        self.num = len(mass)
        self.nmat = lib.ref_ns_init(self.num, f64(x), f64(mass), f64(vol), rho, rmu, beta, gamma)

    def assemble(self, nvel, naccel, ndispl, npres, nmass, facl):
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        tau1 = np.zeros(self.num)
        tau2 = np.zeros(self.num)
        assert self.lib.ref_ns_assemble(f64(nvel), f64(naccel), f64(ndispl), f64(npres), f64(nmass), facl,
                                        tau1, tau2) == 0
        matrow = np.zeros(self.nodec + 1, dtype=np.int32)
        matcolid = np.zeros(self.nmat, dtype=np.int32)
        amat = np.zeros(16 * self.nmat)
        b = np.zeros(4 * self.nodec)
        self.lib.ref_ns_get_matrix(matrow, matcolid, amat, b)
        return dict(tau1=tau1, tau2=tau2, matrow=matrow, matcolid=matcolid, amat=amat.reshape(16, self.nmat),
                    b_rhs=b)

    def solve(self, nvel, naccel, nmass, facl, bcs, rtol=1.0e-10, max_newton=50):
        """SolveNS: the Newton loop of one time step on the nodal state, each
        linear system solved to ||b - A x|| <= rtol ||b||.  bcs: four
        (nodes, values) pairs for u, v, w, p.  Returns ndispl, npres, Newton
        iterations and Krylov iterations; self.rkr_hist holds the residual of
        each Newton iteration."""
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        lib = self.lib
        lib.ref_ns_solve.restype = C.c_int
        lib.ref_ns_solve.argtypes = [_dp, _dp, _dp, C.c_double, _ip] + [_ip, _dp] * 4 + [
            C.c_double, C.c_int, _dp, _dp, C.POINTER(C.c_int), _dp]
        nodes = [i32(n) if len(n) else np.zeros(1, dtype=np.int32) for n, _ in bcs]
        vals = [f64(v) if len(v) else np.zeros(1) for _, v in bcs]
        counts = i32([len(n) for n, _ in bcs])
        nd = np.zeros(3 * self.nodec)
        npr = np.zeros(self.nodec)
        kry = C.c_int(0)
        args = []
        for k in range(4):
            args += [nodes[k], vals[k]]
        hist = np.zeros(max_newton)
        it = lib.ref_ns_solve(f64(nvel), f64(naccel), f64(nmass), float(facl), counts, *args, float(rtol),
                              int(max_newton), nd, npr, C.byref(kry), hist)
        assert it > 0
        self.rkr_hist = hist[:it]
        return nd, npr, it, kry.value

    def run(self, vel, accel, scheme, facl, bcs, nsteps, rtol=1.0e-10):
        """nsteps time steps of the fluid loop (work/src_fluid/MPM/main.cpp:45-68):
        MeshPointLinklist, Particle2Node, SolveNS (each linear system solved to
        ||b - A x|| <= rtol ||b||), Node2Particle, from particle velocities and
        accelerations (n, 3); scheme 0 PIC, 1 FLIP.  Returns the nodal fields of
        the first Particle2Node (nmass, nvof, nvel, naccel), the particle state
        after the last step (x, v, a as (n, 3), pres), and the Newton and Krylov
        iteration counts."""
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        lib = self.lib
        lib.ref_ns_run.restype = C.c_int
        lib.ref_ns_run.argtypes = [_dp, _dp, C.c_int, C.c_double, _ip] + [_ip, _dp] * 4 + [
            C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, C.POINTER(C.c_int)]
        nodes = [i32(n) if len(n) else np.zeros(1, dtype=np.int32) for n, _ in bcs]
        vals = [f64(v) if len(v) else np.zeros(1) for _, v in bcs]
        counts = i32([len(n) for n, _ in bcs])
        args = []
        for k in range(4):
            args += [nodes[k], vals[k]]
        N = self.nodec
        nodal = np.zeros(8 * N)
        x = np.zeros((self.num, 3))
        v = np.zeros((self.num, 3))
        a = np.zeros((self.num, 3))
        pres = np.zeros(self.num)
        kry = C.c_int(0)
        it = lib.ref_ns_run(f64(vel), f64(accel), int(scheme), float(facl), counts, *args, float(rtol), int(nsteps),
                            nodal, x, v, a, pres, C.byref(kry))
        assert it > 0
        out = dict(nmass=nodal[:N], nvof=nodal[N:2 * N], nvel=nodal[2 * N:5 * N], naccel=nodal[5 * N:])
        return out, dict(x=x, v=v, a=a, pres=pres), it, kry.value
