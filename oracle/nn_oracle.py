"""FP64 numpy restatement of the learned-preconditioner network (test oracle).

Test infrastructure only: the tests use it to check the tensor-core forward,
data-gradient and weight-gradient kernels of hpc-mpm-code_gb300/csrc/mpm_nn.cu.
The network has no counterpart in the reference (its solid solves use
GPBiCGSafe, module/solver/solver.cpp:19-141); the definition followed here is
the one documented in include/mpm_gpu.h and csrc/mpm_nn.cuh:

    x0 = [r (3 channels), phi (3 channels)]
    e0 = relu(conv3(x0; 6->16))          e1 = relu(conv3/2(e0; 16->32))
    e2 = relu(conv3/2(e1; 32->64))       c2 = conv3(e2; 64->32)
    d1 = relu(up(c2) + e1)               c1 = conv3(d1; 32->16)
    d0 = relu(up(c1) + e0)               z  = d0 W5 + b5

Arrays are (batch, nz, ny, nx, channels) so that flattening gives the
control-point order i + nx (j + ny k).  With ``bf16=True`` the values the GPU
stores in BF16 (input, conv weights, activations, activation gradients) are
rounded to BF16 at the same places, so that the comparison measures the
kernels rather than the number format.
"""
from __future__ import annotations

import numpy as np

CIN = (6, 16, 32, 64, 32)
COUT = (16, 32, 64, 32, 16)
TAPS = [((t % 3) - 1, ((t // 3) % 3) - 1, (t // 9) - 1) for t in range(27)]   # (dx, dy, dz)


def num_params():
    return sum(27 * ci * co + co for ci, co in zip(CIN, COUT)) + 48 + 3


def unpack(p):
    """FP32 parameter vector -> dict of arrays (layout of include/mpm_gpu.h)."""
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for l, (ci, co) in enumerate(zip(CIN, COUT)):
        out[f"W{l}"] = p[o:o + 27 * ci * co].reshape(27, ci, co)
        o += 27 * ci * co
        out[f"b{l}"] = p[o:o + co]
        o += co
    out["W5"] = p[o:o + 48].reshape(16, 3)
    o += 48
    out["b5"] = p[o:o + 3]
    return out


def pack(d):
    parts = []
    for l in range(5):
        parts += [d[f"W{l}"].ravel(), d[f"b{l}"].ravel()]
    parts += [d["W5"].ravel(), d["b5"].ravel()]
    return np.concatenate(parts)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    d = {}
    for l, (ci, co) in enumerate(zip(CIN, COUT)):
        d[f"W{l}"] = rng.normal(0.0, np.sqrt(2.0 / (27 * ci)), (27, ci, co))
        d[f"b{l}"] = rng.normal(0.0, 0.05, co)
    d["W5"] = rng.normal(0.0, 0.25, (16, 3))
    d["b5"] = rng.normal(0.0, 0.05, 3)
    return pack(d).astype(np.float32)


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def coarse_dims(n):
    return tuple(m // 2 + 1 for m in n)


def _pad(x, stride, nout):
    """Zero-pad the spatial axes so that every tap slice of the output exists."""
    pads = [(0, 0)]
    for ax in range(3):
        nin = x.shape[1 + ax]
        last = stride * (nout[ax] - 1) + 1
        pads.append((1, max(0, last - (nin - 1))))
    pads.append((0, 0))
    return np.pad(x, pads)


def _tap_slice(t, stride, nout):
    dx, dy, dz = TAPS[t]
    sl = [slice(None)]
    for d, n in zip((dz, dy, dx), nout):
        s0 = 1 + d
        sl.append(slice(s0, s0 + stride * (n - 1) + 1, stride))
    sl.append(slice(None))
    return tuple(sl)


def conv(x, W, b, stride):
    """x (B, nz, ny, nx, cin) -> (B, nz', ny', nx', cout); nout per axis from stride."""
    nin = x.shape[1:4]
    nout = nin if stride == 1 else coarse_dims(nin)
    xp = _pad(x, stride, nout)
    out = np.zeros(x.shape[:1] + tuple(nout) + (W.shape[2],))
    for t in range(27):
        out += xp[_tap_slice(t, stride, nout)] @ W[t]
    if b is not None:
        out += b
    return out


def conv_t(g, W, stride, nin):
    """Adjoint of conv with respect to its input: g (B, nout.., cout) -> (B, nin.., cin)."""
    nout = g.shape[1:4]
    shape = (g.shape[0],) + tuple(nin) + (W.shape[1],)
    xp = _pad(np.zeros(shape), stride, nout)
    for t in range(27):
        xp[_tap_slice(t, stride, nout)] += g @ W[t].T
    return xp[:, 1:1 + nin[0], 1:1 + nin[1], 1:1 + nin[2], :]


def conv_dw(x, g, stride):
    """dW[t] = sum over output nodes of x[gather(o, t)]^T g[o]."""
    nout = g.shape[1:4]
    xp = _pad(x, stride, nout)
    dw = np.zeros((27, x.shape[-1], g.shape[-1]))
    for t in range(27):
        xs = xp[_tap_slice(t, stride, nout)]
        dw[t] = xs.reshape(-1, xs.shape[-1]).T @ g.reshape(-1, g.shape[-1])
    return dw


def _prolong(nf, nc):
    P = np.zeros((nf, nc))
    for i in range(nf):
        if i % 2 == 0:
            P[i, i // 2] = 1.0
        else:
            P[i, i // 2] = 0.5
            P[i, i // 2 + 1] = 0.5
    return P


def up(c, nf):
    nc = c.shape[1:4]
    Pz, Py, Px = (_prolong(nf[a], nc[a]) for a in range(3))
    return np.einsum("zZ,yY,xX,bZYXc->bzyxc", Pz, Py, Px, c)


def restrict(g, nc):
    nf = g.shape[1:4]
    Pz, Py, Px = (_prolong(nf[a], nc[a]) for a in range(3))
    return np.einsum("zZ,yY,xX,bzyxc->bZYXc", Pz, Py, Px, g)


def relu(a):
    return np.maximum(a, 0.0)


def forward(params, r, bf16=False, linear=False):
    """r (B, nz, ny, nx, 6): input channels -> (z (..., 3), cache).  linear:
    no activations and no biases (the network's default mode on the GPU)."""
    P = unpack(params)
    q = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W = [q(P[f"W{l}"]) for l in range(5)]
    b = [0.0 * P[f"b{l}"] if linear else P[f"b{l}"] for l in range(5)]
    relu = (lambda a: a) if linear else globals()["relu"]
    x0 = q(r)
    n0 = x0.shape[1:4]
    n1 = coarse_dims(n0)
    e0 = q(relu(conv(x0, W[0], b[0], 1)))
    e1 = q(relu(conv(e0, W[1], b[1], 2)))
    e2 = q(relu(conv(e1, W[2], b[2], 2)))
    c2 = q(conv(e2, W[3], b[3], 1))
    d1 = q(relu(up(c2, n1) + e1))
    c1 = q(conv(d1, W[4], b[4], 1))
    d0 = q(relu(up(c1, n0) + e0))
    z = d0 @ P["W5"] + (0.0 if linear else P["b5"])
    cache = dict(x0=x0, e0=e0, e1=e1, e2=e2, c2=c2, d1=d1, c1=c1, d0=d0, W=W, P=P, q=q, linear=linear)
    return z, cache


def backward(params, r, gz, bf16=False, linear=False):
    """Gradient of sum(z * gz) with respect to the parameters (packed like params)."""
    z, C = forward(params, r, bf16, linear)
    q, W, P = C["q"], C["W"], C["P"]
    act = (lambda a: np.ones_like(a)) if linear else (lambda a: a > 0)
    x0, e0, e1, e2, c2, d1, c1, d0 = (C[k] for k in ("x0", "e0", "e1", "e2", "c2", "d1", "c1", "d0"))
    n0, n1, n2 = x0.shape[1:4], e1.shape[1:4], e2.shape[1:4]
    G = {}
    G["W5"] = d0.reshape(-1, 16).T @ gz.reshape(-1, 3)
    G["b5"] = gz.reshape(-1, 3).sum(0)
    gd0 = q((gz @ P["W5"].T) * act(d0))
    gc1 = q(restrict(gd0, n1))
    G["b4"] = gc1.reshape(-1, 16).sum(0)
    G["W4"] = conv_dw(d1, gc1, 1)
    gd1 = q(conv_t(gc1, W[4], 1, n1) * act(d1))
    gc2 = q(restrict(gd1, n2))
    G["b3"] = gc2.reshape(-1, 32).sum(0)
    G["W3"] = conv_dw(e2, gc2, 1)
    ge2 = q(conv_t(gc2, W[3], 1, n2) * act(e2))
    G["b2"] = ge2.reshape(-1, 64).sum(0)
    G["W2"] = conv_dw(e1, ge2, 2)
    ge1 = q((conv_t(ge2, W[2], 2, n1) + gd1) * act(e1))
    G["b1"] = ge1.reshape(-1, 32).sum(0)
    G["W1"] = conv_dw(e0, ge1, 2)
    ge0 = q((conv_t(ge1, W[1], 2, n0) + gd0) * act(e0))
    G["b0"] = ge0.reshape(-1, 16).sum(0)
    G["W0"] = conv_dw(x0, ge0, 1)
    if linear:
        for l in range(5):
            G[f"b{l}"] = 0.0 * G[f"b{l}"]
        G["b5"] = 0.0 * G["b5"]
    return z, pack(G)


def blocks(vec):
    """Split a packed parameter-sized vector into named blocks."""
    return unpack(vec)
