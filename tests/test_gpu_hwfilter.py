"""The hardware-filtered variant of the ray march (tvk_set_hardware_filtering):
every brick read through a texture object with the texture unit's trilinear
filter.  Its fixed-point filter weights make it differ from the exact path,
so it is held to a distance from the FP32 oracle, not to parity: the mean
per-channel difference within 2/255 and 99 % of pixels within 16/255 (the
measured distances are printed).  It must
also differ from the exact frame somewhere (the texture path really ran), and
switching it off gives the exact frame back bit for bit."""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Batch, Renderer, TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume
from test_gpu_render import ramp_tf, tf2d

pytestmark = pytest.mark.gpu

W, H = 96, 80
BS, OV = 18, 1
MEAN_BOUND = 2.0 / 255  # mean |difference| per channel against the FP32 oracle
P99_BOUND = 16.0 / 255  # 99th percentile of the per-pixel largest channel difference

CASES = [
    # id, dtype, mode, lighting, light model, eye
    ("u8_1d", np.uint8, 0, False, 0, (0.3, 0.4, 1.5)),
    ("u16_1d_lit", np.uint16, 0, True, 0, (-1.1, 0.2, -0.7)),
    ("u16_1d_lit_bp", np.uint16, 0, True, 1, (0.9, -0.6, 1.2)),
    ("u8_2d_lit", np.uint8, 1, True, 0, (0.3, 0.4, 1.5)),
    ("u16_iso", np.uint16, 2, False, 0, (0.9, 0.6, 1.0)),
]


def volume(dtype):
    vmax = 255 if dtype == np.uint8 else 4095
    return numpy_blob_volume((61, 47, 39), dtype, 9, (3, 11), (vmax * 0.3, vmax), vmax, 31, 3)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_hw_filter_close_to_oracle(cuda_ok, case):
    name, dtype, mode, lit, model, eye = case
    raw = volume(dtype)
    vol = Volume(raw, brick_size=(BS, BS, BS), overlap=OV)
    r = Renderer()
    r.RegisterDataset(vol)
    tf = tf2d(256, 32) if mode == 1 else ramp_tf(256 if dtype == np.uint8 else 4096)
    if mode == 1:
        r.Set2DTransFloat(tf)
    else:
        r.Set1DTransFloat(tf)
    iso = 0.5 * float(raw.max())
    if mode == 2:
        r.SetIsoValue(iso)
    r.SetRendermode(mode)
    r.SetUseLighting(lit)
    if model == 1:
        r.SetLightModel(1, 0.2, 0.6, 0.2, 32.0)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    exact = r.ReadBackPixels().copy()
    r.SetHardwareFiltering(True)
    r.Paint()
    tex = r.ReadBackPixels().copy()
    r.SetHardwareFiltering(False)
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), exact)  # the exact path is untouched
    kw = dict(width=W, height=H, eye=eye, mode=mode, lighting=lit, light_model=model)
    if mode == 2:
        kw["isovalue"] = iso
    ref, _, _ = O.render(raw, (BS, BS, BS), OV, tf, **kw)
    d = np.abs(tex.astype(np.float64) - ref.astype(np.float64))
    p99 = np.percentile(d.max(axis=2), 99)
    print(f"{name}: texture path vs FP32 oracle: max {d.max() * 255:.2f}/255, "
          f"mean {d.mean() * 255:.4f}/255, p99 {p99 * 255:.2f}/255")
    assert np.isfinite(tex).all()
    assert d.mean() <= MEAN_BOUND, f"{name}: mean {d.mean() * 255:.3f}/255"
    assert p99 <= P99_BOUND, f"{name}: p99 {p99 * 255:.2f}/255"
    assert np.abs(tex - exact).max() > 0, f"{name}: the texture path gave the exact frame"
    assert (tex[..., 3] > 0).mean() > 0.05


def test_gpu_hw_filter_refusals(cuda_ok):
    raw = volume(np.uint8)
    vol = Volume(raw, brick_size=(BS, BS, BS), overlap=OV)
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(ramp_tf(256))
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    r.Resize(W, H)
    r.SetHardwareFiltering(True)
    with pytest.raises(TvkError):
        Batch().Paint([r])  # batches use the exact lookups
    r.SetRendermode(2)
    r.SetIsoValue(120.0)
    r.SetCV(True)
    with pytest.raises(TvkError):
        r.Paint()  # ClearView frames
    rgba = np.stack([raw] * 4, axis=-1)
    c = Renderer()
    c.RegisterDataset(Volume(rgba, brick_size=(BS, BS, BS), overlap=OV))
    c.Set1DTransFloat(ramp_tf(256))
    c.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    c.Resize(W, H)
    c.SetHardwareFiltering(True)
    with pytest.raises(TvkError):
        c.Paint()  # colour volumes
