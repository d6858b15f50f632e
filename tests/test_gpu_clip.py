"""The clip plane (AbstrRenderer::SetClipPlane / EnableClipPlane) of the
brick-by-brick ray march against the oracle: each brick's ray segment is cut
at the plane (the capped brick box of GLRaycaster.cpp:328-337) and bricks
wholly on the cut side are skipped (AbstrRenderer::Clipped).  Same tolerance as
the other image tests; sample counts equal exactly."""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Pool, TvkError
from test_gpu_lod_render import make, vols  # noqa: F401  (fixture)
from test_gpu_render import compare, ramp_tf, tf2d

pytestmark = pytest.mark.gpu

PLANES = [(1.0, 0.0, 0.0, 0.0), (0.3, -0.5, 0.8, 0.1), (-1.0, -1.0, 0.0, 0.2),
          (0.0, 0.0, 2.0, -0.3)]
CASES = [
    # id, volume, mode, lighting
    ("u8_1d", "u8", 0, False),
    ("u16_1d_lit", "u16", 0, True),
    ("u8_2d_lit", "u8", 1, True),
    ("u8_iso", "u8", 2, False),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("plane", PLANES, ids=[str(p) for p in PLANES])
def test_gpu_clip_plane_matches_oracle(cuda_ok, vols, case, plane):  # noqa: F811
    name, vk, mode, lit = case
    raw = vols[vk]
    tf = tf2d() if mode == 1 else ramp_tf(256 if vk == "u8" else 1024)
    vol, r = make(raw, 18, 1, tf, mode, lit)
    iso = 150.0 if vk == "u8" else 2200.0
    if mode == 2:
        r.SetIsoValue(iso)
    r.SetClipPlane(plane)
    r.EnableClipPlane()
    for eye in [(0.3, 0.4, 1.5), (-1.1, 0.2, -0.7)]:
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
        r.Resize(80, 64)
        r.Paint()
        img, cnt, st = r.ReadBackPixels(), r.ReadSampleCounts(), r.GetStats()
        kw = dict(width=80, height=64, eye=eye, mode=mode, lighting=lit, want_counts=True,
                  clip_plane=plane)
        if mode == 2:
            kw["isovalue"] = iso
        ref, n, rc = O.render(raw, (18, 18, 18), 1, tf, **kw)
        compare(img, ref, f"{name} {plane} {eye}")
        if mode == 2:
            assert (cnt <= rc).all()
        else:
            np.testing.assert_array_equal(cnt, rc, err_msg=f"{name} {plane} {eye}")
            assert st.samples == n


def test_gpu_clip_plane_culls_bricks_and_toggles(cuda_ok, vols):  # noqa: F811
    raw = vols["u8"]
    tf = ramp_tf(256)
    vol, r = make(raw, 18, 1, tf, 0, False)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    r.Resize(80, 64)
    r.Paint()
    full, n_full = r.ReadBackPixels().copy(), r.GetStats().bricks_visible
    r.SetClipPlane((1.0, 0.0, 0.0, 0.0))  # cuts x >= 0: half the bricks
    r.EnableClipPlane()
    r.Paint()
    assert r.GetStats().bricks_visible < n_full
    half = r.ReadBackPixels().copy()
    assert not np.array_equal(half, full)
    r.DisableClipPlane()
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), full)
    # a plane beyond the volume cuts nothing, one behind everything cuts it all
    r.SetClipPlane((1.0, 0.0, 0.0, -10.0))
    r.EnableClipPlane()
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), full)
    r.SetClipPlane((1.0, 0.0, 0.0, 10.0))
    r.Paint()
    assert not r.ReadBackPixels().any() and r.GetStats().bricks_visible == 0


def test_gpu_clip_plane_errors(cuda_ok, vols):  # noqa: F811
    vol, r = make(vols["u8"], 18, 1, ramp_tf(256), 0, False)
    with pytest.raises(TvkError):
        r.SetClipPlane((0.0, 0.0, 0.0, 1.0))
    r.SetClipPlane((0.0, 1.0, 0.0, 0.0))
    r.EnableClipPlane()
    r.Resize(32, 32)
    pool = Pool(vol, 1 << 28)
    with pytest.raises(TvkError) as e:
        pool.Paint(r)
    assert "UNSUPPORTED" in str(e.value)
