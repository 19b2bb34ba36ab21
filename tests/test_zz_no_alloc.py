"""mpm_gpu_p2g_noalloc: the P2G scatter for callers that cannot let a library
allocate device memory (a host program that owns every allocation, or a time
loop that must not hit cudaMalloc's device-wide synchronisation).  Its only
scratch is a static device array; the test checks, through the C ABI, that
two calls in a row reproduce the nodal sums of the regular entry point
(mpm_gpu_p2g) to the FP32 P2G tolerance used elsewhere (1e-5 relative L2).
Collected last so that a failure here cannot stop the rest of a run.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def test_noalloc_p2g_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    s = scenes.elastic_block(grid=(40, 40, 40), cell_lo=(6, 6, 0), cell_hi=(34, 34, 24), npc=2)
    s.vel[:] = np.random.default_rng(5).normal(0.0, 0.4, size=s.vel.shape)
    facl = 0.75
    # reference values from the regular entry point, with a non-zero stress state
    gpu = capi.GpuSolid(s, precision=32)
    gpu.steps(3, facl)
    p = gpu.particles()
    gpu.load(p["x"], p["v"], s.mass, s.vol0, F=p["F"], stress=p["sigma"], matid=s.matid)
    gpu.upload_state(vol=np.ascontiguousarray(p["vol"]))
    gpu.p2g(facl)
    gpu.grid_update()
    want = {k: gpu.nodal(k) for k in ("nmass", "nvof", "nmome", "nforce")}
    gpu.sync()
    gpu.close()

    dev = torch.device("cuda:0")
    f32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=dev)
    x = f32(p["x"].T.copy())
    v = f32(p["v"].T.copy())
    sig = f32(p["sigma"].T.copy())
    m = f32(s.mass)
    vol = f32(p["vol"])
    nodec = s.nodec
    out = {k: torch.zeros(nodec * c, dtype=torch.float32, device=dev)
           for k, c in (("nmass", 1), ("nvof", 1), ("nmome", 3), ("nforce", 3))}
    lib = capi.load()
    fp = C.POINTER(C.c_float)
    lib.mpm_gpu_p2g_noalloc.argtypes = [C.POINTER(capi.GridDesc), C.POINTER(C.c_double), C.c_double, C.c_double,
                                        C.c_int64, fp, fp, fp, fp, fp, fp, fp, fp, fp, C.c_void_p]
    g = capi.GridDesc((C.c_int * 3)(*s.xyelem), (C.c_double * 3)(*s.xymin), (C.c_double * 3)(*s.dxy),
                      (C.c_int * 3)(*s.idimc), (C.c_int * 3)(*s.npxye))
    grav = (C.c_double * 3)(*s.gravity)
    ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), fp)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for t in out.values():
            t.fill_(123.0)   # stale output must be overwritten, stale scratch must be cleared
        rc = lib.mpm_gpu_p2g_noalloc(C.byref(g), grav, facl, s.mtol, s.num, ptr(x), ptr(v), ptr(sig), ptr(m),
                                     ptr(vol), ptr(out["nmass"]), ptr(out["nvof"]), ptr(out["nmome"]),
                                     ptr(out["nforce"]), C.c_void_p(stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        for k, ref in want.items():
            got = out[k].cpu().numpy().astype(np.float64).reshape(ref.shape)
            assert rel_l2(got, ref) <= 1e-5, (call, k, rel_l2(got, ref))


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = capi.load()
    lib.mpm_gpu_p2g_noalloc.restype = C.c_int
    g = capi.GridDesc((C.c_int * 3)(64, 64, 64), (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1),
                      (C.c_int * 3)(1, 1, 1), (C.c_int * 3)(2, 2, 2))
    grav = (C.c_double * 3)(0, 0, 0)
    dummy = C.cast(C.c_void_p(16), C.POINTER(C.c_float))   # never dereferenced: the size check comes first
    rc = lib.mpm_gpu_p2g_noalloc(C.byref(g), grav, C.c_double(1.0), C.c_double(1e-12), C.c_int64(0), dummy, dummy,
                                 dummy, dummy, dummy, dummy, dummy, dummy, dummy, None)
    assert rc == 1   # MPM_ERR_BAD_ARG: 65^3 control points exceed 64^3
