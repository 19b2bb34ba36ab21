"""mpm_gpu_p2g_noalloc: the P2G scatter for callers that cannot let a library
allocate device memory (a host program that owns every allocation, or a time
loop that must not hit cudaMalloc's device-wide synchronisation).  Its only
scratch is a static device array; the test checks, through the C ABI, that
two calls in a row reproduce the nodal sums of the regular entry point
(mpm_gpu_p2g) to the FP32 P2G tolerance used elsewhere (1e-5 relative L2).
It also checks the caller-visible status word: a particle outside the grid
and a particle with a non-finite value are skipped and reported, an empty
particle set gives all-zero nodal fields, and a grid of exactly 64^3 control
points (the scratch limit) is accepted while 65^3 is refused.
Collected last so that a failure here cannot stop the rest of a run.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _bind(lib):
    fp = C.POINTER(C.c_float)
    lib.mpm_gpu_p2g_noalloc.restype = C.c_int
    lib.mpm_gpu_p2g_noalloc.argtypes = [C.POINTER(capi.GridDesc), C.POINTER(C.c_double), C.c_double, C.c_double,
                                        C.c_int64, fp, fp, fp, fp, fp, fp, fp, fp, fp, C.c_void_p, C.c_void_p]
    return fp


def _grid(s):
    return capi.GridDesc((C.c_int * 3)(*s.xyelem), (C.c_double * 3)(*s.xymin), (C.c_double * 3)(*s.dxy),
                         (C.c_int * 3)(*s.idimc), (C.c_int * 3)(*s.npxye))


def _noalloc(torch, s, facl, x, v, sig, m, vol, fill=123.0):
    """One call through the C ABI on torch device arrays (SoA FP32); returns
    the nodal outputs and the status word."""
    dev = torch.device("cuda:0")
    lib = capi.load()
    fp = _bind(lib)
    out = {k: torch.full((s.nodec * c,), fill, dtype=torch.float32, device=dev)
           for k, c in (("nmass", 1), ("nvof", 1), ("nmome", 3), ("nforce", 3))}
    status = torch.full((1,), -7, dtype=torch.int32, device=dev)
    ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), fp)
    g = _grid(s)
    grav = (C.c_double * 3)(*s.gravity)
    n = int(m.numel())
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mpm_gpu_p2g_noalloc(C.byref(g), grav, facl, s.mtol, n, ptr(x), ptr(v), ptr(sig), ptr(m), ptr(vol),
                                 ptr(out["nmass"]), ptr(out["nvof"]), ptr(out["nmome"]), ptr(out["nforce"]),
                                 C.c_void_p(status.data_ptr()), C.c_void_p(stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return {k: t.cpu().numpy().astype(np.float64) for k, t in out.items()}, int(status.item())


def _soa(torch, s, p):
    dev = torch.device("cuda:0")
    f32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=dev)
    return (f32(p["x"].T.copy()), f32(p["v"].T.copy()), f32(p["sigma"].T.copy()), f32(s.mass), f32(p["vol"]))


def _regular(s, p, facl):
    """The regular entry point's nodal fields for the particle state p."""
    gpu = capi.GpuSolid(s, precision=32)
    gpu.load(p["x"], p["v"], s.mass, s.vol0, F=p["F"], stress=p["sigma"], matid=s.matid)
    gpu.upload_state(vol=np.ascontiguousarray(p["vol"]))
    gpu.p2g(facl)
    gpu.grid_update()
    want = {k: gpu.nodal(k) for k in ("nmass", "nvof", "nmome", "nforce")}
    gpu.sync()
    gpu.close()
    return want


def _stressed_block():
    s = scenes.elastic_block(grid=(40, 40, 40), cell_lo=(6, 6, 0), cell_hi=(34, 34, 24), npc=2)
    s.vel[:] = np.random.default_rng(5).normal(0.0, 0.4, size=s.vel.shape)
    gpu = capi.GpuSolid(s, precision=32)
    gpu.steps(3, 0.75)
    p = gpu.particles()
    gpu.sync()
    gpu.close()
    return s, p


def test_noalloc_p2g_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    facl = 0.75
    s, p = _stressed_block()   # a non-zero stress state
    want = _regular(s, p, facl)
    arrays = _soa(torch, s, p)
    for call in range(2):
        # stale output must be overwritten and stale scratch cleared
        got, status = _noalloc(torch, s, facl, *arrays)
        assert status == 0, (call, status)
        for k, ref in want.items():
            err = rel_l2(got[k].reshape(ref.shape), ref)
            assert err <= 1e-5, (call, k, err)


def test_noalloc_skips_and_reports_bad_particles():
    """One particle just outside the grid and one with a NaN velocity: both
    are skipped (the nodal fields equal those of the other particles alone)
    and reported in the status word (bit 0 outside, bit 1 non-finite)."""
    torch = pytest.importorskip("torch")
    facl = 1.0
    s, p = _stressed_block()
    n = s.num
    keep = np.ones(n, dtype=bool)
    keep[[17, 4242]] = False
    q = {k: np.array(v, copy=True) for k, v in p.items()}
    q["x"][17, 0] = s.xymin[0] + s.dxy[0] * s.xyelem[0] + 0.25 * s.dxy[0]   # beyond the last cell
    q["v"][4242, 1] = np.nan
    sub = scenes.Scene(xyelem=s.xyelem, xymin=s.xymin, dxy=s.dxy, idimc=s.idimc, npxye=s.npxye, dt=s.dt, mtol=s.mtol,
                       gravity=s.gravity, iprop=s.iprop, mat_prop=s.mat_prop, coord=p["x"][keep], vel=p["v"][keep],
                       mass=s.mass[keep], vol0=s.vol0[keep], matid=s.matid[keep], scheme=s.scheme)
    want = _regular(sub, {k: v[keep] for k, v in p.items()}, facl)
    got, status = _noalloc(torch, s, facl, *_soa(torch, s, q))
    assert status == 3, status
    for k, ref in want.items():
        err = rel_l2(got[k].reshape(ref.shape), ref)
        assert err <= 1e-5, (k, err)
    # only the outside particle: bit 0 alone
    q["v"][4242, 1] = p["v"][4242, 1]
    _, status = _noalloc(torch, s, facl, *_soa(torch, s, q))
    assert status == 1, status


def test_noalloc_empty_set_and_largest_grid():
    """n = 0 gives all-zero nodal fields (only the clear and finish kernels
    run) on a grid of exactly 64^3 control points, the scratch limit."""
    torch = pytest.importorskip("torch")
    s = scenes.elastic_block(grid=(63, 63, 63), cell_lo=(0, 0, 0), cell_hi=(1, 1, 1), npc=1, fix_bottom=False)
    assert s.nodec == 64 ** 3
    dev = torch.device("cuda:0")
    e = torch.zeros(16, dtype=torch.float32, device=dev)   # never read with n = 0
    got, status = _noalloc(torch, s, 1.0, e, e, e, e[:0], e)
    assert status == 0
    for k, a in got.items():
        assert a.shape[0] in (s.nodec, 3 * s.nodec) and not np.any(a), k


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = capi.load()
    _bind(lib)
    g = capi.GridDesc((C.c_int * 3)(64, 64, 64), (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1),
                      (C.c_int * 3)(1, 1, 1), (C.c_int * 3)(2, 2, 2))
    grav = (C.c_double * 3)(0, 0, 0)
    dummy = C.cast(C.c_void_p(16), C.POINTER(C.c_float))   # never dereferenced: the size check comes first
    rc = lib.mpm_gpu_p2g_noalloc(C.byref(g), grav, C.c_double(1.0), C.c_double(1e-12), C.c_int64(0), dummy, dummy,
                                 dummy, dummy, dummy, dummy, dummy, dummy, dummy, C.c_void_p(16), None)
    assert rc == 1   # MPM_ERR_BAD_ARG: 65^3 control points exceed 64^3
    g = capi.GridDesc((C.c_int * 3)(8, 8, 8), (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1),
                      (C.c_int * 3)(1, 1, 1), (C.c_int * 3)(2, 2, 2))
    rc = lib.mpm_gpu_p2g_noalloc(C.byref(g), grav, C.c_double(1.0), C.c_double(1e-12), C.c_int64((1 << 30) + 1),
                                 dummy, dummy, dummy, dummy, dummy, dummy, dummy, dummy, dummy, C.c_void_p(16), None)
    assert rc == 1   # more particles than the 2^30 the entry point takes
