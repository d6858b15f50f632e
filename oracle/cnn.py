"""CPU oracle of the learned reconstruction network (float64 numpy).

TEST INFRASTRUCTURE ONLY: the tests check the GPU kernels' forward outputs and
gradients against these definitions.  The reference has no such network (it
replaces the reference's progressive reduced-quality frames), so this module
defines the mathematics the kernels implement:

* activations NHWC; a 3x3 convolution with zero padding 1, weights
  [tap = ky * 3 + kx][cout][cin], y[p][co] = b[co] + sum_tap sum_ci
  x[p + (ky - 1, kx - 1)][ci] * w[tap][co][ci] (cross-correlation), then
  LeakyReLU(slope) where slope >= 0;
* 2x2 average pooling, 2x nearest upsampling, concatenation along channels;
* the head: out[2y + dy][2x + dx][c] = base[...] + h[y][x][c * 4 + dy * 2 + dx];
* the loss: mean squared error over all elements.

The backward passes are written out by hand; `numerical_grad` checks them by
central differences.
"""
from __future__ import annotations

import numpy as np

# the fixed U-Net (name, c1, c2, cout, LeakyReLU slope or -1)
UNET = [("e0a", 16, 0, 32, 0.1), ("e0b", 32, 0, 32, 0.1), ("e1a", 32, 0, 48, 0.1),
        ("e1b", 48, 0, 48, 0.1), ("e2a", 48, 0, 64, 0.1), ("e2b", 64, 0, 64, 0.1),
        ("b", 64, 0, 64, 0.1), ("d2", 64, 64, 64, 0.1), ("d1", 64, 48, 48, 0.1),
        ("d0", 48, 32, 32, 0.1), ("head", 32, 0, 16, -1.0)]


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """x[p + (dy, dx)] with zeros outside (NHWC)."""
    n, h, w, c = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(h, h - dy)
    xs, xe = max(0, -dx), min(w, w - dx)
    out[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv3x3(x, w, b=None, slope=-1.0):
    """Pre-activation z and output y of a 3x3 convolution (float64)."""
    n, h, wd, cin = x.shape
    cout = w.shape[1]
    z = np.zeros((n, h, wd, cout))
    for tap in range(9):
        ky, kx = tap // 3 - 1, tap % 3 - 1
        z += _shift(x, ky, kx) @ w[tap].T
    if b is not None:
        z += b
    y = np.where(z < 0, z * slope, z) if slope >= 0 else z
    return z, y


def conv3x3_backward(x, w, z, dy, slope=-1.0):
    """dx, dw, db of conv3x3 given the upstream gradient dy at the output."""
    g = np.where(z < 0, dy * slope, dy) if slope >= 0 else dy
    dx = np.zeros_like(x)
    dw = np.zeros_like(w)
    for tap in range(9):
        ky, kx = tap // 3 - 1, tap % 3 - 1
        xs = _shift(x, ky, kx)
        dw[tap] = np.einsum("nhwo,nhwi->oi", g, xs)
        dx += _shift(g @ w[tap], -ky, -kx)
    db = g.sum(axis=(0, 1, 2))
    return dx, dw, db, g


def avgpool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def avgpool2_backward(dy):
    return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_backward(dy):
    n, h, w, c = dy.shape
    return dy.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def head(hh, base):
    n, h, w, _ = hh.shape
    sub = hh.reshape(n, h, w, 4, 2, 2)          # [c][dy][dx]
    up = sub.transpose(0, 1, 4, 2, 5, 3).reshape(n, 2 * h, 2 * w, 4)
    return base + up


def head_backward(dout):
    n, h2, w2, _ = dout.shape
    d = dout.reshape(n, h2 // 2, 2, w2 // 2, 2, 4).transpose(0, 1, 3, 5, 2, 4)
    return d.reshape(n, h2 // 2, w2 // 2, 16)


def mse(out, target):
    d = out - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def unet_forward(params, x, base, round_bf16=False):
    """params: {name: (w, b)}; returns (out, cache).  round_bf16 rounds every
    stored activation and the weights to bfloat16 as the GPU keeps them (the
    head's output stays FP32)."""
    c = {"round": round_bf16}
    rnd = bf16 if round_bf16 else (lambda a: a)

    def conv(name, *inp):
        _, _, _, _, slope = next(l for l in UNET if l[0] == name)
        xin = np.concatenate(inp, axis=3) if len(inp) > 1 else inp[0]
        w, b = params[name]
        z, y = conv3x3(xin, rnd(w), b, slope)
        if name != "head":
            y = rnd(y)
        c[name] = (xin, z, slope, [a.shape[3] for a in inp])
        return y

    a0 = conv("e0a", x)
    s0 = conv("e0b", a0)
    a1 = conv("e1a", rnd(avgpool2(s0)))
    s1 = conv("e1b", a1)
    a2 = conv("e2a", rnd(avgpool2(s1)))
    s2 = conv("e2b", a2)
    bt = conv("b", rnd(avgpool2(s2)))
    d2 = conv("d2", upsample2(bt), s2)
    d1 = conv("d1", upsample2(d2), s1)
    d0 = conv("d0", upsample2(d1), s0)
    hh = conv("head", d0)
    return head(hh, base), c


def unet_backward(params, cache, dout):
    """Gradients {name: (dw, db)} of the loss whose output gradient is dout."""
    grads = {}

    rnd = bf16 if cache.get("round") else (lambda a: a)

    def back(name, dy):
        xin, z, slope, parts = cache[name]
        # the GPU multiplies the BF16 gradient G = dy * act'(z) by BF16 weights
        g = np.where(z < 0, dy * slope, dy) if slope >= 0 else dy
        dx, dw, db, _ = conv3x3_backward(xin, rnd(params[name][0]), z, rnd(g), -1.0)
        grads[name] = (dw, db)
        out, o = [], 0
        for p in parts:
            out.append(dx[..., o:o + p])
            o += p
        return out

    (dd0,) = back("head", head_backward(dout))
    du0, ds0 = back("d0", dd0)
    du1, ds1 = back("d1", upsample2_backward(du0))
    du2, ds2 = back("d2", upsample2_backward(du1))
    (dp2,) = back("b", upsample2_backward(du2))
    (da2,) = back("e2b", ds2 + avgpool2_backward(dp2))
    (dp1,) = back("e2a", da2)
    (da1,) = back("e1b", ds1 + avgpool2_backward(dp1))
    (dp0,) = back("e1a", da1)
    (da0,) = back("e0b", ds0 + avgpool2_backward(dp0))
    back("e0a", da0)
    return grads


def init_params(seed=0, head_zero=False):
    """He-uniform weights, zero biases (float64); head zero if asked."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, c1, c2, cout, _ in UNET:
        cin = c1 + c2
        lim = np.sqrt(6.0 / (9 * cin))
        w = rng.uniform(-lim, lim, size=(9, cout, cin))
        if head_zero and name == "head":
            w[:] = 0
        p[name] = (w, np.zeros(cout))
    return p


def numerical_grad(f, a, idx, eps=1e-6):
    """Central difference of scalar f() w.r.t. a[idx] (a modified in place)."""
    old = a[idx]
    a[idx] = old + eps
    fp = f()
    a[idx] = old - eps
    fm = f()
    a[idx] = old
    return (fp - fm) / (2 * eps)
