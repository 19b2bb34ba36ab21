"""The learned preconditioner inside the implicit solver (through the C ABI).

A small clamped cantilever (16^3-cell grid, 12^3-cell block, 13,824
particles, linear elastic).  Training pairs are harvested from the
solver's own Jacobi-PCG solves (moduli log-uniform in [1e6, 1e8], seeded
random loads), the network is trained on the GPU by its own forward and
backward kernels, and the assembled system of the cantilever is then solved
to ||r|| / ||r0|| <= 1e-8 by flexible CG with the network and by Jacobi-PCG.

* Training reduces the loss.
* Both solves reach the tolerance on the true FP64 residual and agree to
  relative L2 <= 1e-5 (the network cannot change the solution).
* The trained network needs fewer Krylov iterations than Jacobi-PCG, the
  gain this test records (printed with -s).
* An untrained (random) network still converges: the solve falls back to
  Jacobi when the network stops reducing the residual.
"""
import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

EPS = 1.0e-16   # on squared norms: ||r|| / ||r0|| <= 1e-8


def _cantilever():
    return scenes.cantilever(grid=(16, 16, 16), dx=1.0 / 16, cell_lo=(0, 2, 2), cells=(12, 12, 12), npc=2, E=1.0e7)


def test_learned_preconditioner_gain():
    s = _cantilever()
    gpu = capi.GpuImplicitSolid(s, nr_flag=False)
    nodes = s.xynodec
    net = capi.PrecondNet(nodes, max_batch=8, max_pairs=800, seed=5)
    gpu.harvest(net, nsystems=8, loads_per_system=4, pairs_per_load=25, e_min=1.0e6, e_max=1.0e8, seed=1)
    npairs = net.num_pairs()
    assert npairs >= 400
    losses = net.train(epochs=30, batch=8, lr=2.0e-3, seed=3)
    assert losses[-1] < 0.7 * losses[0], losses

    gpu.assemble()
    xj, itj = gpu.solve(eps=EPS)
    gpu.set_precond(net)
    xn, itn = gpu.solve(eps=EPS)
    gpu.set_precond(None)
    gpu.sync()
    print(f"\nJacobi-PCG {itj} iterations, learned FCG {itn} iterations, pairs {npairs}, "
          f"loss {losses[0]:.3f} -> {losses[-1]:.3f}")
    assert rel_l2(xn, xj) <= 1e-5
    assert itn < itj


def test_untrained_network_falls_back_and_converges():
    s = _cantilever()
    gpu = capi.GpuImplicitSolid(s, nr_flag=False)
    net = capi.PrecondNet(s.xynodec, seed=9)
    gpu.assemble()
    xj, itj = gpu.solve(eps=EPS)
    gpu.set_precond(net)
    xn, itn = gpu.solve(eps=EPS)
    gpu.set_precond(None)
    gpu.sync()
    assert rel_l2(xn, xj) <= 1e-5
    assert itn > 0


def test_symmetric_preconditioner_is_symmetric():
    """The applied preconditioner r + (N r + N^T r) / 2 is symmetric:
    <M a, b> = <a, M b> up to BF16 rounding (the transposed convolutions are
    the exact adjoints of the forward ones)."""
    s = _cantilever()
    gpu = capi.GpuImplicitSolid(s, nr_flag=False)
    gpu.assemble()
    _, d, _ = gpu.system()
    act = np.abs(d) > 0
    rng = np.random.default_rng(4)
    net = capi.PrecondNet(s.xynodec, seed=21, symmetric=True)
    gpu.set_precond(net)
    bcmask = np.ones(3 * s.nodec, dtype=bool)
    for comp, nodes, _v in s.bcs:
        bcmask[comp * s.nodec + nodes] = False
    a = rng.normal(size=3 * s.nodec) * act * bcmask
    b = rng.normal(size=3 * s.nodec) * act * bcmask
    scale = np.linalg.norm(a) / np.linalg.norm(b)
    b *= scale   # same RMS, so both applications use the same input scaling
    ma, mb = gpu.apply_precond(a), gpu.apply_precond(b)
    lhs, rhs = float(ma @ b), float(a @ mb)
    gpu.set_precond(None)
    gpu.sync()
    assert abs(lhs - rhs) <= 3e-2 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("precision", [64, 32])
def test_committed_network_on_the_full_cantilever(precision):
    """The committed parameters (weights/precond_cantilever64.f32, trained by
    mpm_gb300.train_precond) on the 1,728,000-particle cantilever they were
    trained for: the system after one implicit step is solved to
    ||r|| / ||r0|| <= 1e-8 on the true FP64 residual by both solvers; the
    learned solver needs at most 36 % of Jacobi-PCG's iterations (FP64
    operator: measured 34 against 100 with the default GCR window of 4
    directions, 32 with 8) and the two solutions agree to 1e-5; a following
    implicit step with the network falls back to Jacobi nowhere.  With the
    FP32 operator the learned GCR keeps its directions and their images in
    FP32 (x, r and the true residual stay FP64)."""
    from mpm_gb300 import train_precond

    params = train_precond.load_weights()
    if params is None:
        pytest.skip("no committed preconditioner parameters")
    s = scenes.cantilever(iprop=1)
    gpu = capi.GpuImplicitSolid(s, nr_flag=True, precision=precision)
    gpu.implicit_steps(1, eps=EPS)
    gpu.assemble()
    xj, itj = gpu.solve(eps=EPS)
    net = capi.PrecondNet(s.xynodec)
    net.set_params(params)
    gpu.set_precond(net)
    xn, itn = gpu.solve(eps=EPS)
    st = gpu.implicit_steps(1, eps=EPS, full=True)   # a whole step with the network: its statistics
    gpu.set_precond(None)
    gpu.sync()
    print(f"\nfull cantilever, FP{precision} operator: Jacobi-PCG {itj} iterations, learned GCR {itn} iterations; "
          f"solutions {rel_l2(xn, xj):.1e} apart; next step {st}")
    assert rel_l2(xn, xj) <= 1e-5
    assert itn <= 0.36 * itj, (itn, itj)
    assert st["precond_fallbacks"] == 0 and st["nn_applications"] > 0, st
