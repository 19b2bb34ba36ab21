"""Tensor-core network kernels (hpc-mpm-code_gb300/csrc/mpm_nn.cu) against the
FP64 oracle (oracle/nn_oracle.py), through the C ABI.

* Forward: relative L2 <= 1e-2 against the oracle with BF16 rounding at the
  places the GPU stores BF16, and <= 5e-2 against the exact FP64 network.
* Backward (weight and bias gradients, which exercise the forward
  convolutions, the transposed data-gradient convolutions, the
  weight-gradient GEMMs, prolongation/restriction and the 1x1 layer):
  relative L2 per parameter block <= 3e-2 against the BF16-rounded oracle.
* Grids with odd and even node counts, batch 2, so that zero padding,
  stride-2 parity and batch boundaries inside a 128-row tile all occur.
"""
import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import capi
from oracle import nn_oracle as O

pytestmark = pytest.mark.gpu

NODES = (17, 12, 10)   # x, y, z control points


def _inputs(seed, batch=2):
    rng = np.random.default_rng(seed)
    shape = (batch, NODES[2], NODES[1], NODES[0])
    x = np.concatenate([rng.normal(size=shape + (3,)), rng.uniform(0.0, 1.0, size=shape + (3,))], axis=-1)
    return x.astype(np.float32), rng.normal(size=shape + (3,)).astype(np.float32)


@pytest.mark.parametrize("linear", [True, False])
def test_forward_matches_oracle(linear):
    p = O.init_params(11)
    net = capi.PrecondNet(NODES, max_batch=2, linear=linear)
    net.set_params(p)
    x, _ = _inputs(1)
    z = net.forward(x.reshape(2, -1, 6)).reshape(x.shape[:-1] + (3,))
    zq, _ = O.forward(p.astype(np.float64), x.astype(np.float64), bf16=True, linear=linear)
    ze, _ = O.forward(p.astype(np.float64), x.astype(np.float64), bf16=False, linear=linear)
    net.close()
    assert rel_l2(z, zq) <= 1e-2, rel_l2(z, zq)
    assert rel_l2(z, ze) <= 5e-2, rel_l2(z, ze)


@pytest.mark.parametrize("linear", [True, False])
def test_backward_matches_oracle(linear):
    p = O.init_params(12)
    net = capi.PrecondNet(NODES, max_batch=2, linear=linear)
    net.set_params(p)
    x, g = _inputs(2)
    grad = net.backward(x.reshape(2, -1, 6), g.reshape(2, -1, 3))
    _, go = O.backward(p.astype(np.float64), x.astype(np.float64), g.astype(np.float64), bf16=True, linear=linear)
    net.close()
    gb, ob = O.unpack(grad), O.unpack(go)
    for k in gb:
        if linear and k.startswith("b"):
            assert np.all(gb[k] == 0.0), k
            continue
        assert rel_l2(gb[k], ob[k]) <= 3e-2, (k, rel_l2(gb[k], ob[k]))


def test_single_sample_equals_batch():
    p = O.init_params(13)
    net = capi.PrecondNet(NODES, max_batch=2)
    net.set_params(p)
    x, _ = _inputs(3)
    zb = net.forward(x.reshape(2, -1, 6))
    z1 = net.forward(x[1].reshape(1, -1, 6))
    net.close()
    assert np.array_equal(zb[1], z1[0])
