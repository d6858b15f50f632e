"""The CPU oracle of the reconstruction network checks itself: its hand-written
backward passes against central differences of its forward pass."""
import numpy as np

from oracle import cnn as K


def test_conv3x3_backward_by_central_differences():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 5, 7, 16))
    w = rng.normal(size=(9, 8, 16)) * 0.2
    b = rng.normal(size=8)
    t = rng.normal(size=(2, 5, 7, 8))
    for slope in (0.1, -1.0):
        def f():
            return 0.5 * np.sum((K.conv3x3(x, w, b, slope)[1] - t) ** 2)
        z, y = K.conv3x3(x, w, b, slope)
        dx, dw, db, _ = K.conv3x3_backward(x, w, z, y - t, slope)
        for idx in [(0, 0, 0, 0), (1, 4, 6, 15), (0, 2, 3, 7)]:
            assert np.isclose(K.numerical_grad(f, x, idx), dx[idx], rtol=1e-5, atol=1e-7)
        for idx in [(0, 0, 0), (4, 7, 15), (8, 3, 9)]:
            assert np.isclose(K.numerical_grad(f, w, idx), dw[idx], rtol=1e-5, atol=1e-7)
        for idx in [(0,), (7,)]:
            assert np.isclose(K.numerical_grad(f, b, idx), db[idx], rtol=1e-5, atol=1e-7)


def test_pool_upsample_head_adjoints():
    rng = np.random.default_rng(1)
    a = rng.normal(size=(2, 4, 6, 3))
    d = rng.normal(size=(2, 2, 3, 3))
    assert np.isclose(np.sum(K.avgpool2(a) * d), np.sum(a * K.avgpool2_backward(d)))
    u = rng.normal(size=(2, 8, 12, 3))
    assert np.isclose(np.sum(K.upsample2(d) * u[:, :4, :6]), np.sum(d * K.upsample2_backward(
        u[:, :4, :6])))
    h = rng.normal(size=(1, 3, 5, 16))
    o = rng.normal(size=(1, 6, 10, 4))
    assert np.isclose(np.sum((K.head(h, np.zeros((1, 6, 10, 4)))) * o),
                      np.sum(h * K.head_backward(o)))


def test_unet_backward_by_central_differences():
    rng = np.random.default_rng(2)
    params = K.init_params(seed=3)
    x = rng.normal(size=(1, 8, 8, 16))
    base = rng.normal(size=(1, 16, 16, 4))
    target = rng.normal(size=(1, 16, 16, 4))

    def f():
        return K.mse(K.unet_forward(params, x, base)[0], target)[0]

    out, cache = K.unet_forward(params, x, base)
    _, dout = K.mse(out, target)
    grads = K.unet_backward(params, cache, dout)
    for name in ("e0a", "e1b", "b", "d2", "d0", "head"):
        w, b = params[name]
        dw, db = grads[name]
        for _ in range(3):
            idx = tuple(int(rng.integers(0, s)) for s in w.shape)
            assert np.isclose(K.numerical_grad(f, w, idx), dw[idx], rtol=1e-4, atol=1e-9), name
        assert np.isclose(K.numerical_grad(f, b, (0,)), db[0], rtol=1e-4, atol=1e-9), name


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159], dtype=np.float32)
    r = K.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 3.14159) < 2 ** -6
