"""Tensor-core CNN kernels against the CPU oracle (oracle/cnn.py).

Inputs and weights are drawn as BF16-exact values, so the GPU's products are
exact and the only differences are FP32 (GPU) vs FP64 (oracle) accumulation and
the BF16 rounding of stored outputs.  Whole-network gradients are checked with
the oracle emulating the GPU's BF16 storage of activations and weights.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import cnn as K
from tuvok_gb300 import _native as N
from tuvok_gb300._native import check, lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda").contiguous()


def p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def host(t):
    return t.float().cpu().numpy().astype(np.float64)


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def weights_bf16(w32, cout, cin):
    wf = torch.empty((9, cout, cin), dtype=torch.bfloat16, device="cuda")
    wb = torch.empty((9, cin, cout), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_weights_bf16(p(w32), cout, cin, p(wf), p(wb), stream()))
    return wf, wb


CASES = [  # n, h, w, c1, c2, cout, slope
    # channel counts that are multiples of 16 run on tcgen05 (16x8-pixel
    # patches, TMEM accumulators), the others on mma.sync
    (2, 13, 21, 16, 0, 32, 0.1),
    (1, 40, 24, 4, 12, 32, 0.1),      # c1 = 4: forward on mma.sync
    (1, 290, 300, 4, 12, 32, 0.1),    # the same with 16x16 patches
    (1, 16, 16, 32, 0, 48, 0.1),
    (2, 9, 8, 48, 0, 64, -1.0),
    (1, 12, 20, 64, 64, 64, 0.1),
    (1, 8, 24, 48, 32, 32, 0.1),
    (2, 10, 10, 32, 0, 16, -1.0),
    # large images take the 16x16-patch kernel: all taps' weights staged at
    # once, and (128 input channels) one tap at a time
    (1, 290, 300, 32, 0, 32, 0.1),
    (1, 300, 288, 64, 64, 64, 0.1),
    (2, 200, 248, 48, 32, 32, 0.1),
    (1, 300, 300, 32, 16, 32, 0.1),   # data gradient split over the concatenation
]


@pytest.mark.parametrize("case", CASES, ids=[str(c) for c in CASES])
def test_gpu_conv3x3_forward_and_gradients(cuda_ok, case):
    n, h, w, c1, c2, cout, slope = case
    rng = np.random.default_rng(sum(case[:6]))
    cin = c1 + c2
    x = K.bf16(rng.normal(size=(n, h, w, cin)))
    wt = K.bf16(rng.normal(size=(9, cout, cin)) * (1.0 / np.sqrt(9 * cin)))
    b = rng.normal(size=cout) * 0.1
    x1 = dev(x[..., :c1], torch.bfloat16)
    x2 = dev(x[..., c1:], torch.bfloat16) if c2 else None
    w32 = dev(wt, torch.float32)
    b32 = dev(b, torch.float32)
    wf, wb = weights_bf16(w32, cout, cin)
    assert np.array_equal(host(wf), wt)
    np.testing.assert_array_equal(host(wb), wt[::-1].transpose(0, 2, 1))

    # forward, BF16 output with bias and activation, and FP32 output
    y = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    yf = torch.empty((n, h, w, cout), dtype=torch.float32, device="cuda")
    a = N.CnnConv(x1=p(x1), x2=p(x2), c1=c1, c2=c2, n=n, h=h, w=w, weights=p(wf), bias=p(b32),
                  cout=cout, slope=slope, y_bf16=p(y), y_f32=p(yf), y2_f32=None, split=cout,
                  accumulate=0)
    check(lib().tvk_cnn_conv3x3(C.byref(a), stream()))
    check(lib().tvk_cnn_check(stream()))
    z, yref = K.conv3x3(x, wt, b, slope)
    np.testing.assert_allclose(host(yf), yref, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(host(y), K.bf16(yref), rtol=1e-2, atol=1e-2)

    # backward: G = dY * act'(Y) in BF16, data gradient through the flipped
    # weights (split at c1 for a concatenated input), weight and bias gradients
    dy = rng.normal(size=(n, h, w, cout))
    dy_t = dev(dy, torch.float32)
    g = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_act_grad(p(dy_t), p(y) if slope >= 0 else None, slope, p(g), dy.size,
                                 stream()))
    # the GPU multiplies the FP32 gradient by the FP32 slope, then rounds to BF16
    dy32 = dy.astype(np.float32)
    gref = K.bf16(np.where(host(y) > 0, dy32, dy32 * np.float32(slope)) if slope >= 0 else dy32)
    np.testing.assert_array_equal(host(g), gref)
    dx1 = torch.zeros((n, h, w, c1), dtype=torch.float32, device="cuda")
    dx2 = torch.zeros((n, h, w, c2), dtype=torch.float32, device="cuda") if c2 else None
    bwd = N.CnnConv(x1=p(g), x2=None, c1=cout, c2=0, n=n, h=h, w=w, weights=p(wb), bias=None,
                    cout=cin, slope=-1.0, y_bf16=None, y_f32=p(dx1), y2_f32=p(dx2),
                    split=c1 if c2 else cin, accumulate=0)
    check(lib().tvk_cnn_conv3x3(C.byref(bwd), stream()))
    check(lib().tvk_cnn_check(stream()))
    dxr, dwr, dbr, _ = K.conv3x3_backward(x, wt, z, gref, -1.0)
    got = host(dx1) if not c2 else np.concatenate([host(dx1), host(dx2)], axis=3)
    np.testing.assert_allclose(got, dxr, rtol=1e-4, atol=1e-4)
    dw = torch.zeros((9, cout, cin), dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    wg = N.CnnWgrad(x1=p(x1), x2=p(x2), c1=c1, c2=c2, gy=p(g), n=n, h=h, w=w, cout=cout,
                    dw=p(dw), db=p(db))
    check(lib().tvk_cnn_conv3x3_wgrad(C.byref(wg), stream()))
    scale = np.abs(dwr).max()
    np.testing.assert_allclose(host(dw), dwr, rtol=1e-4, atol=1e-5 * scale)
    np.testing.assert_allclose(host(db), dbr, rtol=1e-4, atol=1e-4)


UP_CASES = [  # h, w (output), c1 (read upsampled from h // 2 x w // 2), c2, cout
    (15, 21, 16, 16, 32),     # tcgen05
    (15, 21, 4, 12, 32),      # mma.sync (c1 not a multiple of 8)
    (300, 290, 32, 16, 32),   # tcgen05, many patches
    (301, 289, 4, 12, 32),    # mma.sync, 16x16 patches
]


@pytest.mark.parametrize("case", UP_CASES, ids=[str(c) for c in UP_CASES])
def test_gpu_conv3x3_upsampled_input(cuda_ok, case):
    """A decoder layer reads the coarser level through the convolution's own
    2x nearest upsampling, clamped at the coarse tensor's last row and column
    when the output size is odd."""
    h, w, c1, c2, cout = case
    h1, w1 = h // 2, w // 2
    rng = np.random.default_rng(h + w + c1)
    x1 = K.bf16(rng.normal(size=(1, h1, w1, c1)))
    x2 = K.bf16(rng.normal(size=(1, h, w, c2)))
    wt = K.bf16(rng.normal(size=(9, cout, c1 + c2)) * (1.0 / np.sqrt(9 * (c1 + c2))))
    b = rng.normal(size=cout) * 0.1
    rows = np.minimum(np.arange(h) // 2, h1 - 1)
    cols = np.minimum(np.arange(w) // 2, w1 - 1)
    x = np.concatenate([x1[:, rows][:, :, cols], x2], axis=3)
    yf = torch.empty((1, h, w, cout), dtype=torch.float32, device="cuda")
    x1_t, x2_t = dev(x1, torch.bfloat16), dev(x2, torch.bfloat16)
    wf, b32 = dev(wt, torch.bfloat16), dev(b, torch.float32)
    a = N.CnnConv(x1=p(x1_t), x2=p(x2_t), c1=c1, c2=c2, n=1, h=h, w=w, weights=p(wf),
                  bias=p(b32), cout=cout, slope=0.1, y_bf16=None, y_f32=p(yf), y2_f32=None,
                  split=cout, accumulate=0, upsample1=1, h1=h1, w1=w1)
    check(lib().tvk_cnn_conv3x3(C.byref(a), stream()))
    check(lib().tvk_cnn_check(stream()))
    _, yref = K.conv3x3(x, wt, b, 0.1)
    np.testing.assert_allclose(host(yf), yref, rtol=1e-5, atol=1e-5)


def test_gpu_pool_upsample_head(cuda_ok):
    rng = np.random.default_rng(5)
    x = K.bf16(rng.normal(size=(2, 6, 10, 32)))
    xt = dev(x, torch.bfloat16)
    y = torch.empty((2, 3, 5, 32), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_avgpool2(p(xt), 2, 6, 10, 32, p(y), stream()))
    np.testing.assert_array_equal(host(y), K.bf16(K.avgpool2(x)))
    # channel counts that are not a multiple of 8 take the one-value-per-thread path
    x6 = K.bf16(rng.normal(size=(1, 6, 10, 6)))
    x6t = dev(x6, torch.bfloat16)
    y6 = torch.empty((1, 3, 5, 6), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_avgpool2(p(x6t), 1, 6, 10, 6, p(y6), stream()))
    np.testing.assert_array_equal(host(y6), K.bf16(K.avgpool2(x6)))
    u = torch.empty((2, 12, 20, 32), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_upsample2(p(xt), 2, 6, 10, 32, p(u), stream()))
    np.testing.assert_array_equal(host(u), K.upsample2(x))
    # (every device tensor is held by a name: a temporary's memory could be
    # reused by the allocator before the kernel reads it)
    d = rng.normal(size=(2, 3, 5, 32))
    d_t = dev(d, torch.float32)
    dx = torch.zeros((2, 6, 10, 32), dtype=torch.float32, device="cuda")
    check(lib().tvk_cnn_avgpool2_backward(p(d_t), 2, 6, 10, 32, p(dx), 1, stream()))
    np.testing.assert_allclose(host(dx), K.avgpool2_backward(d), rtol=1e-6)
    du = rng.normal(size=(2, 12, 20, 32))
    du_t = dev(du, torch.float32)
    o = torch.empty((2, 6, 10, 32), dtype=torch.float32, device="cuda")
    check(lib().tvk_cnn_upsample2_backward(p(du_t), 2, 6, 10, 32, p(o), stream()))
    np.testing.assert_allclose(host(o), K.upsample2_backward(du), rtol=1e-5, atol=1e-6)
    hh = rng.normal(size=(1, 4, 6, 16))
    base = rng.normal(size=(1, 8, 12, 4))
    hh_t, base_t = dev(hh, torch.float32), dev(base, torch.float32)
    out = torch.empty((1, 8, 12, 4), dtype=torch.float32, device="cuda")
    check(lib().tvk_cnn_head(p(hh_t), p(base_t), 1, 4, 6, p(out), stream()))
    np.testing.assert_allclose(host(out), K.head(hh, base), rtol=1e-6, atol=1e-6)
    dh = torch.empty((1, 4, 6, 16), dtype=torch.float32, device="cuda")
    check(lib().tvk_cnn_head_backward(p(base_t), 1, 4, 6, p(dh), stream()))
    np.testing.assert_array_equal(host(dh), K.head_backward(base.astype(np.float32)))


def test_gpu_unet_gradients_match_oracle(cuda_ok):
    """Forward and every layer's weight/bias gradients of the whole U-Net."""
    from tuvok_gb300.learned import UNet
    rng = np.random.default_rng(8)
    params = K.init_params(seed=4)
    params["head"] = (params["head"][0] * 0.3, params["head"][1])
    fparams = {k: (v[0].astype(np.float32), v[1].astype(np.float32)) for k, v in params.items()}
    net = UNet(torch, params=fparams)
    x = K.bf16(rng.normal(size=(2, 16, 24, 16)))
    base = rng.normal(size=(2, 32, 48, 4))
    target = rng.normal(size=(2, 32, 48, 4))
    out = net.forward(dev(x, torch.bfloat16), dev(base, torch.float32))
    oref, cache = K.unet_forward({k: (v[0].astype(np.float64), v[1].astype(np.float64))
                                  for k, v in fparams.items()}, x, base, round_bf16=True)
    rel = np.linalg.norm(host(out) - oref) / np.linalg.norm(oref - base)
    assert rel < 2e-2, rel
    net.zero_grad()
    loss, dout = net.loss(out, dev(target, torch.float32))
    lref, doref = K.mse(oref, target)
    assert abs(loss.item() - lref) < 1e-3 * lref
    net.backward(dout)
    grads = K.unet_backward({k: (v[0].astype(np.float64), v[1].astype(np.float64))
                             for k, v in fparams.items()}, cache, doref)
    for name, (dwr, dbr) in grads.items():
        L = net.layers[name]
        dw, db = host(L["dw"]), host(L["db"])
        ew = np.linalg.norm(dw - dwr) / max(np.linalg.norm(dwr), 1e-30)
        eb = np.linalg.norm(db - dbr) / max(np.linalg.norm(dbr), 1e-30)
        cos = float(np.sum(dw * dwr) / (np.linalg.norm(dw) * np.linalg.norm(dwr)))
        assert ew < 5e-2 and eb < 5e-2 and cos > 0.998, (name, ew, eb, cos)


def test_gpu_adam_matches_formula(cuda_ok):
    rng = np.random.default_rng(3)
    w = rng.normal(size=1000).astype(np.float32)
    g = rng.normal(size=1000).astype(np.float32)
    wt, gt = dev(w, torch.float32), dev(g, torch.float32)
    m = torch.zeros_like(wt)
    v = torch.zeros_like(wt)
    for step in (1, 2):
        check(lib().tvk_cnn_adam(p(wt), p(gt), p(m), p(v), 1000, 1e-2, 0.9, 0.999, 1e-8, step,
                                 stream()))
    mr = 0.9 * (0.1 * g) + 0.1 * g
    vr = 0.999 * (0.001 * g * g) + 0.001 * g * g
    w1 = w - 1e-2 * (0.1 * g / 0.1) / (np.sqrt(0.001 * g * g / 0.001) + 1e-8)
    w2 = w1 - 1e-2 * (mr / (1 - 0.81)) / (np.sqrt(vr / (1 - 0.999 ** 2)) + 1e-8)
    np.testing.assert_allclose(host(wt), w2, rtol=1e-4, atol=1e-6)
