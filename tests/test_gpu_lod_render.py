"""Coarser LODs, reduced resolution / sample rate and the progressive frame
through the C ABI against the oracle.

* tvk_set_lod renders the bricks of one LOD (ComputeHierarchy + FillOverlap
  bricks, LOD aspect in the texture coordinates, opacity-correction exponent
  scaled by the LOD's voxel size);
* tvk_set_reduced_quality renders at 1/2 of the viewport and/or half the sample
  rate; the reduced image is stretched bilinearly over the viewport;
* tvk_paint_progressive follows AbstrRenderer::PlanFrame: start LOD, one LOD
  finer per subframe down to ComputeMinLODForCurrentView.

Same tolerance as the full-resolution tests (2/255 max, 0.25/255 mean against
the FP32 oracle); sample counts equal exactly.
"""
import math

import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Renderer, TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume
from test_gpu_render import compare, ramp_tf, tf2d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vols():
    return {
        "u8": numpy_blob_volume((61, 47, 39), np.uint8, 9, (3, 11), (80, 255), 255, 31, 3),
        "u16": numpy_blob_volume((50, 56, 33), np.uint16, 9, (3, 11), (900, 4000), 4095, 32, 20),
    }


def make(raw, bs, ov, tf, mode, lit, median=False, srm=1.0):
    vol = Volume(raw, brick_size=(bs, bs, bs), overlap=ov, median=median)
    r = Renderer()
    r.RegisterDataset(vol)
    if mode == 1:
        r.Set2DTransFloat(tf)
    elif mode == 0:
        r.Set1DTransFloat(tf)
    r.SetRendermode(mode)
    r.SetUseLighting(lit)
    r.SetSampleRateModifier(srm)
    return vol, r


def oracle(raw, bs, ov, tf, w, h, eye, mode, lit, **kw):
    return O.render(raw, (bs, bs, bs), ov, tf, width=w, height=h, eye=eye, mode=mode,
                    lighting=lit, want_counts=True, **kw)


CASES = [
    # id, volume, brick, overlap, mode, lighting, lod, median, srm
    ("u8_1d_lod1", "u8", 18, 1, 0, False, 1, False, 1.0),
    ("u8_1d_lod2_median", "u8", 18, 1, 0, False, 2, True, 1.5),
    ("u16_1d_lit_lod1", "u16", 18, 1, 0, True, 1, False, 1.0),
    ("u16_1d_lod3", "u16", 14, 2, 0, False, 3, False, 1.0),
    ("u8_2d_lit_lod1", "u8", 18, 1, 1, True, 1, False, 1.0),
    ("u8_iso_lod1", "u8", 18, 1, 2, False, 1, False, 1.0),
    ("u8_1d_coarsest", "u8", 18, 1, 0, False, 6, False, 1.0),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_lod_render_matches_oracle(cuda_ok, vols, case):
    name, vk, bs, ov, mode, lit, lod, median, srm = case
    raw = vols[vk]
    tf = tf2d() if mode == 1 else ramp_tf(256 if vk == "u8" else 1024)
    vol, r = make(raw, bs, ov, tf, mode, lit, median, srm)
    lod = min(lod, vol.GetLODLevelCount() - 1)
    r.SetLOD(lod)
    for eye in [(0.3, 0.4, 1.5), (-1.1, 0.2, -0.7)]:
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
        r.Resize(80, 64)
        r.Paint()
        img, cnt, st = r.ReadBackPixels(), r.ReadSampleCounts(), r.GetStats()
        ref, n, rc = oracle(raw, bs, ov, tf, 80, 64, eye, mode, lit, lod=lod, median=median,
                            srm=srm)
        compare(img, ref, f"{name} {eye}")
        if mode == 2:
            assert (cnt <= rc).all()
        else:
            np.testing.assert_array_equal(cnt, rc, err_msg=f"{name} {eye}")
            assert st.samples == n
        assert st.bricks_total == np.prod(vol.GetBrickLayout(lod))


@pytest.mark.parametrize("w,h,screen,sampling,lod", [
    (80, 64, True, False, 0), (81, 63, True, False, 0), (80, 64, False, True, 0),
    (80, 64, True, True, 1), (97, 55, True, True, 2)])
def test_gpu_reduced_quality_matches_oracle(cuda_ok, vols, w, h, screen, sampling, lod):
    raw = vols["u8"]
    tf = ramp_tf(256)
    for lit in (False, True):
        vol, r = make(raw, 18, 1, tf, 0, lit)
        r.SetLOD(lod)
        r.SetReducedQuality(screen, sampling)
        eye = (0.5, -0.3, 1.4)
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
        r.Resize(w, h)
        r.Paint()
        img, cnt, st = r.ReadBackPixels(), r.ReadSampleCounts(), r.GetStats()
        ref, n, rc = oracle(raw, 18, 1, tf, w, h, eye, 0, lit, lod=lod, dec_screen=screen,
                            dec_sampling=sampling)
        rw, rh = (int(w * 0.5 + 0.5), int(h * 0.5 + 0.5)) if screen else (w, h)
        assert r.GetRenderSize() == (rw, rh) and cnt.shape == (rh, rw) == rc.shape
        assert img.shape == (h, w, 4)
        compare(img, ref, f"{w}x{h} screen={screen} sampling={sampling} lit={lit}")
        np.testing.assert_array_equal(cnt, rc)
        assert st.samples == n


def test_gpu_reduced_quality_iso(cuda_ok, vols):
    raw = vols["u16"]
    vol, r = make(raw, 18, 1, None, 2, False)
    r.SetIsoValue(2200.0)
    r.SetReducedQuality(True, True)
    eye = (0.9, 0.6, 1.0)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(90, 70)
    r.Paint()
    img = r.ReadBackPixels()
    ref, n, rc = O.render(raw, (18, 18, 18), 1, ramp_tf(16), width=90, height=70, eye=eye, mode=2,
                          isovalue=2200.0, dec_screen=True, dec_sampling=True, want_counts=True)
    compare(img, ref, "iso reduced")
    assert (img[..., 3] > 0).mean() > 0.02


def min_lod_reference(dims, lod_count, eye, fovy, height, znear):
    """CullingLOD::GetLODLevel as ComputeMinLODForCurrentView calls it, in float32."""
    f = np.float32
    ext = np.array(dims, dtype=f)
    ext = ext / ext.max()
    err = (ext / np.array(dims, dtype=f)).max()
    lod_factor = f(2.0) * f(math.tan(f(fovy) * ((f(3.1416) / f(180.0)) / f(2.0)))) * f(1.0) / \
        f(height)
    z_center = -f(np.linalg.norm(np.array(eye, dtype=np.float64)))  # looking at the origin
    fz = max(f(znear), -z_center)
    level = int(math.floor(f(np.log(f(lod_factor * fz / err))) / f(np.log(f(2.0)))))
    return min(max(level, 0), lod_count - 1)


def test_gpu_min_lod_for_view(cuda_ok, vols):
    raw = vols["u8"]
    vol, r = make(raw, 18, 1, ramp_tf(256), 0, False)
    seen = set()
    for dist, height in [(1.5, 64), (6.0, 64), (30.0, 64), (200.0, 32), (0.3, 480)]:
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.0, 0.0, dist))
        r.Resize(64, height)
        got = r.ComputeMinLODForCurrentView()
        assert got == min_lod_reference((61, 47, 39), vol.GetLODLevelCount(), (0, 0, dist),
                                        50.0, height, 0.01)
        seen.add(got)
    assert len(seen) >= 3  # distance moves the LOD


def test_gpu_progressive_frame_sequence(cuda_ok, vols):
    raw = vols["u8"]
    tf = ramp_tf(256)
    vol, r = make(raw, 18, 1, tf, 0, False)
    eye = (0.0, 0.0, 3.0)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(72, 60)
    # GetLargestSingleBrickLOD: the first LOD that is one brick
    single = next(l for l in range(vol.GetLODLevelCount()) if vol.GetBrickCount(l) == 1)
    min_lod = r.ComputeMinLODForCurrentView()
    info = r.PaintProgressive(new_frame=True)
    assert info.start_lod == single and info.lod == single and info.min_lod == min_lod
    lods = [info.lod]
    while not info.frame_complete:
        info = r.PaintProgressive()
        lods.append(info.lod)
        assert info.render_width == 72 and not info.decreased_screen_res
    assert lods == list(range(single, min_lod - 1, -1))
    # the final subframe equals a plain paint at that LOD
    final = r.ReadBackPixels()
    ref, n, rc = oracle(raw, 18, 1, tf, 72, 60, eye, 0, False, lod=min_lod)
    compare(final, ref, "progressive final subframe")
    # nothing left: further calls render nothing
    again = r.PaintProgressive()
    assert again.frame_complete == 1 and again.ms == 0.0
    # The reference's frame timer starts at -1 ms (msecPassedCurrentFrame(-1.0f),
    # AbstrRenderer.cpp:96), so a sub-millisecond first subframe reads as "not
    # measured" and the second frame starts at the coarsest LOD again; from the
    # third frame on the fast frames move the start LOD one finer.
    starts = []
    for _ in range(2):
        info = r.PaintProgressive(new_frame=True)
        starts.append(info.start_lod)
        while not info.frame_complete:
            info = r.PaintProgressive()
    assert starts[0] in (single, max(min_lod, single - 1))
    assert starts[1] == max(min_lod, single - 1)


def test_gpu_progressive_low_res_when_too_slow(cuda_ok, vols):
    """A frame-rate target no subframe can meet: after three slow frames at the
    coarsest start LOD the planner decreases the screen resolution for the
    first subframe of each frame and re-renders that LOD at full resolution."""
    raw = vols["u8"]
    vol, r = make(raw, 18, 1, ramp_tf(256), 0, False)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.0, 0.0, 3.0))
    r.Resize(72, 60)
    r.SetPerfMeasures(min_framerate=10 ** 9, render_low_res_intermediate=True)
    seen_low = False
    for frame in range(8):
        info = r.PaintProgressive(new_frame=True)
        if info.decreased_screen_res:
            seen_low = True
            assert (info.render_width, info.render_height) == (36, 30)
            nxt = r.PaintProgressive()
            assert nxt.lod == info.lod and not nxt.decreased_screen_res
            assert nxt.render_width == 72
        while not info.frame_complete:
            info = r.PaintProgressive()
    assert seen_low


def test_gpu_lod_errors(cuda_ok, vols):
    raw = vols["u8"]
    vol = Volume(raw, brick_size=(18, 18, 18), overlap=1, lod0_only=True)
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(ramp_tf(256))
    r.Resize(16, 16)
    r.SetLOD(1)
    with pytest.raises(TvkError) as e:
        r.Paint()
    assert "UNSUPPORTED" in str(e.value)
    r.SetLOD(99)
    with pytest.raises(TvkError):
        r.Paint()
    with pytest.raises(TvkError):
        r.SetPerfMeasures(screen_res_dec_factor=0.5)
