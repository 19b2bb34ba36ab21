"""The FP64 network oracle (oracle/nn_oracle.py) against finite differences.

The oracle is what the tensor-core forward and backward kernels are checked
against, so its own gradients are pinned here first: for each parameter
block, the directional derivative of sum(z * g) along a random direction
must match a central difference to 1e-3.  The step is small (1e-8) so that
no ReLU kink falls inside the difference interval.
"""
import numpy as np
import pytest

from oracle import nn_oracle as O


def test_parameter_layout():
    assert O.num_params() == 139747 + 27 * 3 * 16
    p = O.init_params(0)
    assert np.array_equal(O.pack(O.unpack(p)).astype(np.float32), p)


@pytest.mark.parametrize("linear", [False, True])
def test_gradients_match_finite_differences(linear):
    rng = np.random.default_rng(7)
    p = O.init_params(3).astype(np.float64)
    r = np.concatenate([rng.normal(size=(1, 6, 7, 9, 3)), rng.uniform(size=(1, 6, 7, 9, 3))], axis=-1)
    gz = rng.normal(size=(1, 6, 7, 9, 3))
    _, g = O.backward(p, r, gz, linear=linear)

    def loss(pp):
        return float((O.forward(pp, r, linear=linear)[0] * gz).sum())

    eps = 1e-8
    base = O.unpack(np.zeros_like(p))
    for name in base:
        d = {k: np.zeros_like(v) for k, v in base.items()}
        d[name] = rng.normal(size=d[name].shape)
        v = O.pack(d)
        fd = (loss(p + eps * v) - loss(p - eps * v)) / (2 * eps)
        an = float(g @ v)
        if linear and name.startswith("b"):
            assert an == 0.0
            continue
        assert abs(fd - an) <= 1e-3 * max(abs(fd), 1e-6), (name, fd, an)


def test_transposed_conv_is_adjoint():
    rng = np.random.default_rng(8)
    for stride, nin in ((1, (5, 6, 7)), (2, (5, 6, 7)), (2, (4, 8, 9))):
        x = rng.normal(size=(2,) + nin + (4,))
        W = rng.normal(size=(27, 4, 8))
        y = O.conv(x, W, None, stride)
        g = rng.normal(size=y.shape)
        lhs = float((y * g).sum())
        rhs = float((x * O.conv_t(g, W, stride, nin)).sum())
        assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_restriction_is_adjoint_of_prolongation():
    rng = np.random.default_rng(9)
    nf = (9, 8, 7)
    nc = O.coarse_dims(nf)
    c = rng.normal(size=(1,) + nc + (3,))
    f = rng.normal(size=(1,) + nf + (3,))
    assert abs(float((O.up(c, nf) * f).sum()) - float((c * O.restrict(f, nc)).sum())) <= 1e-10 * abs(
        float((O.up(c, nf) * f).sum()))
