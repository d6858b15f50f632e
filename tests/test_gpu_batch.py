"""Batched frames (tvk_paint_batch): one persistent launch over many renderers,
each with its own volume, TF, mode, lighting, sample rate, viewport, LOD and
reduced-quality switches.  Every frame must be bit-identical to the
renderer's own tvk_paint (same device code, same parameters), also when the
captured CUDA graph is replayed after camera changes.
"""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Batch, Renderer, TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume, orbit_poses
from test_gpu_render import compare, ramp_tf, tf2d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def volumes():
    u8 = numpy_blob_volume((48, 40, 36), np.uint8, 8, (3, 10), (80, 255), 255, 21, 3)
    u16 = numpy_blob_volume((44, 50, 38), np.uint16, 8, (3, 10), (900, 4000), 4095, 22, 20)
    return {"u8": (u8, Volume(u8, brick_size=(18, 18, 18), overlap=1)),
            "u16": (u16, Volume(u16, brick_size=(18, 18, 18), overlap=1))}


# volume, mode, lighting, light model, srm, w, h, lod, reduce screen, reduce sampling
VIEWS = [
    ("u8", 0, False, 0, 1.0, 64, 48, 0, False, False),
    ("u16", 0, True, 0, 1.5, 96, 80, 0, False, False),
    ("u16", 0, True, 1, 2.0, 33, 17, 0, False, False),
    ("u8", 1, True, 0, 1.0, 128, 72, 0, False, False),
    ("u8", 2, False, 0, 1.0, 80, 64, 0, False, False),
    ("u16", 2, False, 0, 0.5, 70, 70, 1, False, False),
    ("u8", 0, False, 0, 1.0, 90, 60, 1, True, True),
    ("u16", 1, False, 0, 1.0, 40, 100, 0, True, False),
]


def make_renderers(volumes, views):
    rs = []
    for k, (vk, mode, lit, lm, srm, w, h, lod, ds, dsr) in enumerate(views):
        r = Renderer()
        r.RegisterDataset(volumes[vk][1])
        if mode == 0:
            r.Set1DTransFloat(ramp_tf(256 if vk == "u8" else 1024))
        elif mode == 1:
            r.Set2DTransFloat(tf2d(seed=k))
        r.SetRendermode(mode)
        r.SetUseLighting(lit)
        r.SetLightModel(lm)
        r.SetSampleRateModifier(srm)
        r.SetLOD(lod)
        r.SetReducedQuality(ds, dsr)
        r.Resize(w, h)
        rs.append(r)
    return rs


def set_poses(rs, seed):
    for r, (eye, _, _) in zip(rs, orbit_poses(len(rs), seed)):
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)


def singles(rs):
    out = []
    for r in rs:
        r.Paint()
        out.append((r.ReadBackPixels().copy(), r.ReadSampleCounts().copy(), r.GetStats().samples))
    return out


def check_equal(rs, ref):
    for k, (r, (img, cnt, n)) in enumerate(zip(rs, ref)):
        np.testing.assert_array_equal(r.ReadBackPixels(), img, err_msg=f"view {k}")
        np.testing.assert_array_equal(r.ReadSampleCounts(), cnt, err_msg=f"view {k}")
        assert r.GetStats().samples == n, k


def test_gpu_batch_equals_single_paints(cuda_ok, volumes):
    rs = make_renderers(volumes, VIEWS)
    b = Batch()
    for seed in (5, 6, 7):  # new cameras each round; the graph is replayed
        set_poses(rs, seed)
        ref = singles(rs)
        b.Paint(rs)
        check_equal(rs, ref)
        info = b.GetInfo()
        assert info.frames == len(rs) and info.ctas >= 152
        if seed == 5:
            assert info.autotuned == 1 and info.graph_reused == 0
        else:
            assert info.graph_reused == 1 and info.autotuned == 0
    # a changed viewport changes the launch shape: new graph, still identical
    rs[0].Resize(50, 50)
    ref = singles(rs)
    b.Paint(rs)
    check_equal(rs, ref)
    assert b.GetInfo().graph_reused == 0


def test_gpu_batch_against_oracle(cuda_ok, volumes):
    raw = volumes["u16"][0]
    rs = make_renderers(volumes, VIEWS[1:3])
    set_poses(rs, 11)
    b = Batch()
    b.SetAutotune(False, 2)
    b.Paint(rs)
    assert b.GetInfo().ctas_per_sm == 2
    for (vk, mode, lit, lm, srm, w, h, lod, ds, dsr), r, (eye, _, _) in zip(
            VIEWS[1:3], rs, orbit_poses(2, 11)):
        ref, n, rc = O.render(raw, (18, 18, 18), 1, ramp_tf(1024), width=w, height=h, eye=eye,
                              srm=srm, lighting=lit, light_model=lm, want_counts=True)
        compare(r.ReadBackPixels(), ref, "batched view")
        np.testing.assert_array_equal(r.ReadSampleCounts(), rc)


def test_gpu_batch_many_views(cuda_ok, volumes):
    """64 frames of mixed sizes (the batching configuration's view count)."""
    rng = np.random.default_rng(3)
    views = []
    for k in range(64):
        w, h = [(64, 64), (96, 96), (128, 72), (48, 80)][rng.integers(0, 4)]
        views.append(("u8" if k % 2 else "u16", int(rng.integers(0, 2)), bool(k % 3 == 0), 0,
                      float(rng.choice([0.5, 1.0, 2.0])), w, h, 0, False, False))
    rs = make_renderers(volumes, views)
    set_poses(rs, 21)
    ref = singles(rs)
    b = Batch()
    b.Paint(rs)
    check_equal(rs, ref)
    info = b.GetInfo()
    tw = 16 * info.rays_per_thread
    assert info.rays_per_thread in (1, 2)
    assert info.tiles == sum(((w + tw - 1) // tw) * ((h + 7) // 8)
                             for (_, _, _, _, _, w, h, _, _, _) in views)


@pytest.mark.parametrize("rays", [1, 2])
def test_gpu_batch_rays_per_thread(cuda_ok, volumes, rays):
    """Tiles of 16x8 pixels with one ray per thread, or 32x8 with two: every
    frame and sample count equals its own tvk_paint either way."""
    rs = make_renderers(volumes, VIEWS)
    set_poses(rs, 31)
    ref = singles(rs)
    b = Batch()
    b.SetRaysPerThread(rays)
    b.Paint(rs)
    check_equal(rs, ref)
    info = b.GetInfo()
    assert info.rays_per_thread == rays
    tw = 16 * rays
    assert info.tiles == sum(((r.GetRenderSize()[0] + tw - 1) // tw) *
                             ((r.GetRenderSize()[1] + 7) // 8) for r in rs)


def test_gpu_batch_errors(cuda_ok, volumes):
    rs = make_renderers(volumes, VIEWS[:2])
    set_poses(rs, 1)
    b = Batch()
    with pytest.raises(TvkError):
        b.Paint([rs[0], rs[0]])
    with pytest.raises(TvkError):
        b.GetInfo()  # nothing painted yet
