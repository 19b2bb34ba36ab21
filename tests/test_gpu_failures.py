"""Failure paths of the C ABI, made on the host or with a bounded device wait.

The reference stops the run where these are detected: GPBiCGSafe aborts at
its iteration limit (module/solver/solver.cpp:135), the Newton loop at its
limit (module/solver/solver.cpp:586-589) and a particle that leaves every
rank's domain aborts the job (module/mpi_data.cpp:31-34).  Here each one is
a status code returned by the next synchronising call, after which the
context stays usable:

* a NaN written into a host particle array and uploaded -> MPM_ERR_NONFINITE
* a particle placed outside the grid -> MPM_ERR_PARTICLE_OUT_OF_BOX, counted
  in mpm_stats.out_of_box
* an implicit solve capped at kmax = 2 -> MPM_ERR_KRYLOV_MAXIT
* a bounded device wait that runs out (mpm_gpu_selftest_wait: an mbarrier
  that nothing completes, limit 50 ms) -> MPM_ERR_DEVICE_TIMEOUT

No test here faults, traps or hangs the GPU: every failure is made on the
host (a bad value in an input array, an iteration cap) or is a wait with a
wall-time limit.
"""
import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

OK, NONFINITE, OUT_OF_BOX, KRYLOV_MAXIT, DEVICE_TIMEOUT = 0, 3, 4, 5, 6


def _block(**kw):
    s = scenes.elastic_block(grid=(16, 16, 16), cell_lo=(4, 4, 0), cell_hi=(12, 12, 8), npc=2, **kw)
    s.vel[:] = np.random.default_rng(11).normal(0.0, 0.2, size=s.vel.shape)
    return s


def _reload(gpu, s):
    gpu.load(s.coord, s.vel, s.mass, s.vol0, matid=s.matid)


@pytest.mark.parametrize("precision", [64, 32])
def test_nan_upload_reports_nonfinite_then_recovers(precision):
    s = _block()
    gpu = capi.GpuSolid(s, precision=precision)
    gpu.steps(2)
    p = gpu.particles()
    assert gpu.sync_status() == OK
    v = np.ascontiguousarray(p["v"])
    v[123, 2] = np.nan
    gpu.upload_state(vel=v)
    gpu.steps(1)
    assert gpu.sync_status() == NONFINITE
    # a load with a non-finite value is refused outright
    bad = np.array(s.coord, copy=True)
    bad[5, 1] = np.inf
    with pytest.raises(capi.MpmError) as e:
        gpu.load(bad, s.vel, s.mass, s.vol0, matid=s.matid)
    assert e.value.code == NONFINITE
    # the context is still usable: a fresh load runs as a new context does
    _reload(gpu, s)
    gpu.steps(3)
    assert gpu.sync_status() == OK
    ref = capi.GpuSolid(s, precision=precision)
    ref.steps(3)
    want = ref.particles()
    got = gpu.particles()
    ref.close()
    gpu.close()
    assert rel_l2(got["v"], want["v"]) <= 1e-12 and rel_l2(got["x"], want["x"]) <= 1e-12


def test_particle_outside_grid_reports_out_of_box():
    s = _block(fix_bottom=False)
    s.coord[7] = (s.xyelem[0] + 0.25) * s.dxy[0], 0.5 * s.xyelem[1] * s.dxy[1], 0.5 * s.xyelem[2] * s.dxy[2]
    gpu = capi.GpuSolid(s, precision=32)
    gpu.steps(1)
    st = gpu.stats()
    assert gpu.sync_status() == OUT_OF_BOX
    assert st["out_of_box"] >= 1
    # with the particle back inside the grid the next steps are clean
    s.coord[7] = 0.5 * np.array(s.xyelem) * np.array(s.dxy)
    _reload(gpu, s)
    gpu.steps(2)
    assert gpu.sync_status() == OK
    gpu.close()


def test_krylov_iteration_cap_reports_maxit():
    s = scenes.cantilever(grid=(12, 8, 8), cell_lo=(0, 2, 2), cells=(10, 4, 4))
    gpu = capi.GpuImplicitSolid(s)
    with pytest.raises(capi.MpmError) as e:
        gpu.implicit_steps(1, eps=1.0e-20, kmax=2)
    assert e.value.code == KRYLOV_MAXIT
    gpu.sync_status()
    # a fresh context with the normal limits solves the same step
    ok = capi.GpuImplicitSolid(s)
    kt, nt, _ = ok.implicit_steps(1, eps=1.0e-16)
    assert kt > 2 and nt >= 1
    ok.close()
    gpu.close()


def test_device_wait_timeout_reports_and_context_stays_usable():
    s = _block()
    gpu = capi.GpuSolid(s, precision=32)
    gpu.steps(2)
    assert gpu.sync_status() == OK
    gpu.selftest_wait(0.05)
    assert gpu.sync_status() == DEVICE_TIMEOUT
    assert gpu.sync_status() == OK   # the latched error was cleared by the call that returned it
    gpu.steps(2)
    got = gpu.particles()
    assert gpu.sync_status() == OK
    ref = capi.GpuSolid(s, precision=32)
    ref.steps(4)
    want = ref.particles()
    ref.close()
    gpu.close()
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["v"], want["v"])


def test_selftest_wait_rejects_unbounded_limits():
    s = _block()
    gpu = capi.GpuSolid(s, precision=32)
    for bad in (0.0, -1.0, 2.0, float("nan")):
        with pytest.raises(capi.MpmError) as e:
            gpu.selftest_wait(bad)
        assert e.value.code == 1
    gpu.close()
