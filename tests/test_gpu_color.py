"""Colour (RGBA8) volumes against the oracle: the bricks of every LOD with
their ghost layers bit for bit; 1D mode (VRender1D-Color / VRender1DLit-Color: the voxel's
colour times the TF entry at (r + g + b) / 3) and iso mode (the alpha
channel's surface, GLRaycaster-Color-FS + Compose-Color-FS) with the usual
image tolerance.  The opacity correction of a colour sample depends on the
voxel's alpha, so it runs per sample; GLSL's pow(x, y) = exp2(y * log2(x)) is
evaluated on both sides by the same float operations, so sample counts are
equal pixel for pixel.

The GridLeaper over a colour pool (GLGridLeaper-Method-*-color.glsl: the
voxel's colour with the TF's alpha at its alpha, 1D and 2D, lit and unlit; iso
on the alpha channel with the red channel's normal): one pass and a converged
frame against the oracle's pass over the same page table, sample counts and
missing-brick requests equal.  Colour bricks carry no value statistics
(range [0, 255]), so every brick is visible to a TF with any opacity."""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Batch, Pool, Renderer, TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume
from test_gpu_render import compare

pytestmark = pytest.mark.gpu

BS = 18
W, H = 80, 64


@pytest.fixture(scope="module")
def rgba():
    dims = (45, 38, 33)
    ch = [numpy_blob_volume(dims, np.uint8, 7, (3, 9), (60, 255), 255, 70 + k, 3)
          for k in range(4)]
    return np.stack(ch, axis=-1)


def color_tf(n=64):
    t = np.zeros((n, 4), dtype=np.float32)
    i = np.arange(n) / (n - 1)
    t[:, 0], t[:, 1], t[:, 2] = 0.4 + 0.6 * i, 1.0 - 0.5 * i, 0.7
    t[:, 3] = np.clip((i - 0.2) / 0.8, 0, 1) * 0.5
    return t


def renderer(vol, mode, lit, tf=None):
    r = Renderer()
    r.RegisterDataset(vol)
    if tf is not None:
        r.Set1DTransFloat(tf)
    r.SetRendermode(mode)
    r.SetUseLighting(lit)
    return r


@pytest.mark.parametrize("clamp,median", [(False, False), (True, False), (False, True)])
def test_gpu_color_bricks_match_oracle(cuda_ok, rgba, clamp, median):
    """Every LOD: each channel filtered on its own (the oracle's octree is the
    four channel octrees interleaved, pinned to the converter's RGBA files)."""
    vol = Volume(rgba, brick_size=(BS,) * 3, overlap=1, clamp_to_edge=clamp, median=median)
    ref = O.build_octree(rgba, (BS,) * 3, 1, clamp=clamp, median=median)
    k = 0
    for lod in range(vol.GetLODLevelCount()):
        for i in range(vol.GetBrickCount(lod)):
            np.testing.assert_array_equal(vol.GetBrick((0, lod, i)), ref[k], err_msg=f"{lod} {i}")
            k += 1
    assert k == len(ref)


CASES = [
    # id, mode, lighting, light model, eye, LOD
    ("1d", 0, False, 0, (0.3, 0.4, 1.5), 0),
    ("1d_lit", 0, True, 0, (-1.1, 0.2, -0.7), 0),
    ("1d_lit_bp", 0, True, 1, (0.9, -0.6, 1.0), 0),
    ("iso", 2, False, 0, (0.3, 0.4, 1.5), 0),
    ("iso_inside", 2, False, 0, (0.05, 0.02, 0.1), 0),
    ("1d_lit_lod1", 0, True, 0, (0.7, 0.5, 1.2), 1),
    ("iso_lod1", 2, False, 0, (-0.8, 0.6, 1.0), 1),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_color_render_matches_oracle(cuda_ok, rgba, case):
    name, mode, lit, model, eye, lod = case
    tf = color_tf()
    vol = Volume(rgba, brick_size=(BS,) * 3, overlap=1)
    r = renderer(vol, mode, lit, tf)
    if model == 1:
        r.SetLightModel(1, 0.2, 0.6, 0.2, 32.0)
    iso = 130.0
    if mode == 2:
        r.SetIsoValue(iso)
    r.SetSampleRateModifier(1.5)
    r.SetLOD(lod)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    img, cnt, st = r.ReadBackPixels(), r.ReadSampleCounts(), r.GetStats()
    kw = dict(width=W, height=H, eye=eye, mode=mode, lighting=lit, light_model=model,
              srm=1.5, want_counts=True, lod=lod)
    if mode == 2:
        kw["isovalue"] = iso
    ref, n, rc = O.render(rgba, (BS,) * 3, 1, tf, **kw)
    compare(img, ref, name)
    assert st.bricks_visible == st.bricks_total  # colour bricks are never skipped
    if mode == 2:
        assert (cnt <= rc).all()
        assert (img[..., 3] > 0).mean() > 0.05
    else:
        np.testing.assert_array_equal(cnt, rc, err_msg=name)
        assert (img[..., 3] > 0).mean() > 0.05


def test_gpu_color_clip_and_reduced(cuda_ok, rgba):
    tf = color_tf()
    vol = Volume(rgba, brick_size=(BS,) * 3, overlap=1)
    r = renderer(vol, 0, True, tf)
    eye = (0.5, 0.35, 1.3)
    r.SetClipPlane((0.3, -0.5, 0.8, 0.05))
    r.EnableClipPlane()
    r.SetReducedQuality(True, True)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    ref, _, _ = O.render(rgba, (BS,) * 3, 1, tf, width=W, height=H, eye=eye, lighting=True,
                         clip_plane=(0.3, -0.5, 0.8, 0.05), dec_screen=True, dec_sampling=True)
    compare(r.ReadBackPixels(), ref, "clip + reduced")


def test_gpu_color_refusals(cuda_ok, rgba):
    vol = Volume(rgba, brick_size=(BS,) * 3, overlap=1)
    r = renderer(vol, 1, False)
    r.Set2DTransFloat(np.ones((8, 16, 4), np.float32))
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    r.Resize(W, H)
    with pytest.raises(TvkError):
        r.Paint()  # 2D mode
    r.SetRendermode(0)
    r.Set1DTransFloat(color_tf())
    r.Paint()
    with pytest.raises(TvkError):
        Batch().Paint([r])
    with pytest.raises(TvkError):
        vol.GetHistogram()
    with pytest.raises(TvkError):
        vol.Rebrick((9, 9, 9))


LEAPER_CASES = [
    # id, mode, lighting, eye, srm
    ("leap_1d", 0, False, (0.3, 0.4, 1.5), 1.0),
    ("leap_1d_lit", 0, True, (-1.1, 0.2, -0.7), 1.0),
    ("leap_1d_lit_far", 0, True, (1.4, 1.9, 3.5), 1.7),
    ("leap_2d", 1, False, (0.9, -0.6, 1.2), 1.0),
    ("leap_2d_lit", 1, True, (0.3, 0.4, 1.5), 1.0),
    ("leap_iso", 2, False, (0.9, 0.6, 1.0), 1.0),
    ("leap_iso_far", 2, False, (-1.6, 1.4, 2.8), 1.0),
]


def leaper_setup(rgba, mode, lit, srm):
    from test_gpu_render import tf2d
    vol = Volume(rgba, brick_size=(BS,) * 3, overlap=1)
    r = Renderer()
    r.RegisterDataset(vol)
    tf = tf2d(256, 32) if mode == 1 else color_tf(256)
    if mode == 1:
        r.Set2DTransFloat(tf)
    elif mode == 0:
        r.Set1DTransFloat(tf)
    else:
        r.SetIsoValue(130.0)
    r.SetRendermode(mode)
    r.SetUseLighting(lit)
    r.SetSampleRateModifier(srm)
    r.Resize(W, H)
    return vol, r, tf


def leaper_oracle(rgba, tf, page, mode, lit, srm, eye):
    kw = dict(width=W, height=H, eye=eye, mode=mode, lighting=lit, srm=srm)
    if mode == 2:
        kw["isovalue"] = 130.0
    return O.leaper_render(rgba, (BS,) * 3, 1, tf, page, **kw)


@pytest.mark.parametrize("case", LEAPER_CASES, ids=[c[0] for c in LEAPER_CASES])
def test_gpu_color_leaper_matches_oracle(cuda_ok, rgba, case):
    from test_gpu_leaper import check_missing, compare_pass
    name, mode, lit, eye, srm = case
    vol, r, tf = leaper_setup(rgba, mode, lit, srm)
    pool = Pool(vol, 1 << 30)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    # cold pass: only the coarsest brick cached, nothing flagged empty
    info = pool.Paint(r, max_passes=1)
    page = pool.GetPageTable()
    assert info.passes == 1 and info.resident == 1 and page[-1] >= 3
    assert (page[:-1] == 0).all(), name
    img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
    ref, n, rc, missing = leaper_oracle(rgba, tf, page, mode, lit, srm, eye)
    compare_pass(img, cnt, ref, rc, name + " cold")
    check_missing(pool.GetRequests(), missing, name)
    assert missing.size > 0 and n > 0
    # converged: every brick the view needs is resident
    info = pool.Paint(r, max_passes=64)
    assert info.converged == 1 and info.missing_last == 0
    again = pool.Paint(r, max_passes=1)
    assert again.passes == 1 and again.paged == 0 and again.missing_last <= 2
    page = pool.GetPageTable()
    img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
    ref, n, rc, missing = leaper_oracle(rgba, tf, page, mode, lit, srm, eye)
    compare_pass(img, cnt, ref, rc, name + " converged")
    assert (img[..., 3] > 0).mean() > (0.02 if "far" in name else 0.05), name
