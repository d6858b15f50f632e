"""Learned reconstruction through the C ABI (tvk_paint_learned).

* the C++ network run equals the training-side forward pass (same kernels) bit
  for bit on the same reduced frame;
* the probe-ray judge falls back to the plain frame exactly;
* with the committed trained weights, the network beats the method without it
  (the bilinear upscale of the half-resolution, half-rate frame) on held-out
  poses of a volume it was not trained on.
"""
import ctypes as C
import math

import numpy as np
import pytest

from tuvok_gb300 import Renderer
from tuvok_gb300._native import check, lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def small_scene(w=200, h=120):
    from tuvok_gb300.learned import configure_lit, make_training_volume, random_bands_tf
    vol = make_training_volume(torch, 96, 3)
    r = Renderer()
    configure_lit(r, vol, random_bands_tf(np.random.default_rng(2)), width=w, height=h)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.4, 0.5, 1.4))
    return vol, r


def test_gpu_learned_equals_training_forward(cuda_ok):
    from tuvok_gb300.learned import LearnedRenderer, UNet, prepare_input, render_pair
    vol, r = small_scene()
    net = UNet(torch, seed=5)
    # a non-zero head so the residual matters
    net.layers["head"]["w"].normal_(0, 0.05)
    net.refresh()
    low, depth, base, full = render_pair(torch, r, (0.4, 0.5, 1.4))
    x = prepare_input(torch, low, depth)
    out = net.forward(x, base.new_zeros((1, 2 * x.shape[1], 2 * x.shape[2], 4)))
    ref = (out[0, :120, :200] + base).cpu().numpy()
    lr = LearnedRenderer(net.params())
    info = lr.Paint(r, threshold_db=0.0)
    assert info.fell_back == 0 and (info.reduced_width, info.reduced_height) == (100, 60)
    img = r.ReadBackPixels().copy()
    np.testing.assert_array_equal(img, ref)
    # the judge's probe PSNR is that of the probe pixels: one full-quality ray
    # per 8x8 block at offset (3, 1) on a network's first frame, marched on the
    # probe stream while the reduced frame and the network ran
    r.Paint()
    plain = r.ReadBackPixels()
    d = (img[1::8, 3::8].astype(np.float64) - plain[1::8, 3::8]) ** 2
    want = 10.0 * math.log10(1.0 / d.mean())
    assert abs(info.probe_psnr_db - want) < 1e-3, (info.probe_psnr_db, want)
    assert info.ms_probe > 0 and info.ms_frame >= info.ms_reduced + info.ms_network
    # the next frame moves the probes (offset (0, 4))
    info2 = lr.Paint(r, threshold_db=0.0)
    img2 = r.ReadBackPixels().copy()
    d2 = (img2[4::8, 0::8].astype(np.float64) - plain[4::8, 0::8]) ** 2
    assert abs(info2.probe_psnr_db - 10.0 * math.log10(1.0 / d2.mean())) < 1e-3


def test_gpu_learned_fallback_is_the_plain_frame(cuda_ok):
    from tuvok_gb300.learned import LearnedRenderer, UNet
    vol, r = small_scene()
    lr = LearnedRenderer(UNet(torch, seed=1).params())
    info = lr.Paint(r, threshold_db=1e9)
    assert info.fell_back == 1
    img = r.ReadBackPixels().copy()
    r.Paint()
    np.testing.assert_array_equal(img, r.ReadBackPixels())


def test_gpu_learned_beats_bilinear_on_held_out_poses(cuda_ok):
    from tuvok_gb300.learned import (WEIGHTS, LearnedRenderer, UNet, configure_lit,
                                     make_training_volume, psnr, render_pair)
    from tuvok_gb300.workloads import make_tf, orbit_poses
    if not WEIGHTS.exists():
        pytest.skip("no trained weights committed")
    vol = make_training_volume(torch, 512, 4321)  # a seed not among the training volumes
    r = Renderer()
    configure_lit(r, vol, make_tf("bands4096"))
    lr = LearnedRenderer(UNet.load_params())
    gains = []
    for eye, at, up in orbit_poses(6, 777):
        low, depth, base, full = render_pair(torch, r, eye, at)
        info = lr.Paint(r, threshold_db=0.0)
        img = torch.tensor(r.ReadBackPixels(), device="cuda")
        m_learned = float(((img - full) ** 2).mean())
        m_bilinear = float(((base - full) ** 2).mean())
        gains.append(psnr(m_learned) - psnr(m_bilinear))
    assert np.mean(gains) > 0.5, gains


def test_gpu_first_hit_depth(cuda_ok):
    """The first-hit depth of the reduced frame (a network input): non-zero
    exactly where the frame has opacity, 1 / (1 + t) with t the eye distance of
    the first contributing sample, so a camera farther away sees smaller
    values."""
    from tuvok_gb300.learned import render_pair
    vol, r = small_scene()
    means = []
    for dist in (1.3, 2.6):
        low, depth, base, full = render_pair(torch, r, (0.0, 0.0, dist))
        a = low[..., 3].cpu().numpy()
        d = depth.cpu().numpy()
        assert ((d > 0) == (a > 0)).all()
        hit = d[d > 0]
        assert hit.size > 0 and (hit < 1.0 / (1.0 + (dist - 0.9))).all() and (hit > 0.0).all()
        means.append(float(hit.mean()))
    assert means[1] < means[0]
