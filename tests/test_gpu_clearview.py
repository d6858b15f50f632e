"""ClearView in iso mode (AbstrRenderer::SetCV): the context pass and the focus
pass of GLRaycaster-ISO-FS / -ISO-CV-FS per brick (GLRaycaster.cpp:421-436)
and the Compose-CV-FS shading, against the oracle.  Same tolerance as the other
image tests.  The GPU leaves out the passes whose hits cannot win their depth
tests (the context pass behind the nearest context hit, the focus pass after
the first focus hit), so its sample counts are at most the oracle's, and equal
on rays without a context hit when the focus isovalue is the larger."""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Batch, TvkError
from test_gpu_lod_render import make, vols  # noqa: F401  (fixture)
from test_gpu_render import compare

pytestmark = pytest.mark.gpu

BS = 18
W, H = 88, 72
FAR = (1e7, 1e7, 1e7, 0.0)

CASES = [
    # id, volume, isovalue, focus isovalue (None: the default 1.5x), focus pos, params, eye
    ("u8_default", "u8", None, None, (0.0, 0.0, 0.5, 1.0), None, (0.3, 0.4, 1.5)),
    ("u8_near_focus", "u8", 110.0, 170.0, (0.05, -0.05, 0.1, 1.0), (4.0, 0.5, 30.0),
     (-0.9, 0.5, 1.1)),
    ("u8_focus_below_context", "u8", 150.0, 100.0, (0.0, 0.1, 0.0, 1.0), (6.0, 1.0, 60.0),
     (0.6, -0.7, 1.0)),
    ("u16_default", "u16", None, None, (0.0, 0.0, 0.5, 1.0), None, (0.2, -0.6, 1.4)),
    ("u16_near_focus", "u16", 1800.0, 2600.0, (-0.1, 0.05, 0.0, 1.0), (3.0, 2.0, 20.0),
     (1.2, 0.3, -0.9)),
    ("u8_inside", "u8", 120.0, 180.0, (0.02, 0.0, 0.05, 1.0), (5.5, 1.0, 60.0),
     (0.05, 0.02, 0.1)),
]


def iso_renderer(raw, iso):
    vol, r = make(raw, BS, 1, None, 2, False)
    if iso is not None:
        r.SetIsoValue(iso)
    return vol, r


def cv_kw(cv_iso, pos, params, color=(1.0, 0.0, 0.0)):
    d = dict(pos=pos, color=color)
    if cv_iso is not None:
        d["isovalue"] = cv_iso
    if params is not None:
        d["size"], d["context_scale"], d["border_scale"] = params
    return d


def configure(r, cv_iso, pos, params, color=(1.0, 0.0, 0.0)):
    r.SetCV(True)
    if cv_iso is not None:
        r.SetCVIsoValue(cv_iso)
    if params is not None:
        r.SetCVParams(*params)
    r.SetCVColor(color)
    r.SetCVFocusPosFVec(pos)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_clearview_matches_oracle(cuda_ok, vols, case):  # noqa: F811
    name, vk, iso, cv_iso, pos, params, eye = case
    raw = vols[vk]
    vol, r = iso_renderer(raw, iso)
    configure(r, cv_iso, pos, params)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    img, cnt, st = r.ReadBackPixels(), r.ReadSampleCounts(), r.GetStats()
    ref, n, rc = O.render(raw, (BS,) * 3, 1, np.zeros((16, 4), np.float32), width=W, height=H,
                          eye=eye, mode=2, isovalue=iso, want_counts=True,
                          clearview=cv_kw(cv_iso, pos, params))
    compare(img, ref, name)
    assert (cnt <= rc).all() and st.samples <= n
    plain, _, _ = O.render(raw, (BS,) * 3, 1, np.zeros((16, 4), np.float32), width=W,
                           height=H, eye=eye, mode=2, isovalue=iso)
    if cv_iso is None or cv_iso >= (iso or 0):
        miss = plain[..., 3] == 0
        np.testing.assert_array_equal(cnt[miss], rc[miss], err_msg=name)
    # the focus surface shows somewhere, and only where the context surface is
    assert ((img[..., 3] == 0) == (ref[..., 3] == 0)).all()
    assert (img[..., 3] > 0).mean() > 0.02


def test_gpu_clearview_far_focus_is_the_plain_isosurface(cuda_ok, vols):  # noqa: F811
    """Focus point far away (a picking miss): blend 1, no border term, so the
    ClearView frame equals the plain iso frame bit for bit."""
    raw = vols["u16"]
    eye = (0.4, -0.3, 1.3)
    vol, r = iso_renderer(raw, 2000.0)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    plain = r.ReadBackPixels().copy()
    configure(r, 2800.0, FAR, None)
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), plain)
    r.SetCV(False)
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), plain)


@pytest.mark.parametrize("variant", ["reduced", "lod1", "clip"])
def test_gpu_clearview_reduced_lod_and_clip(cuda_ok, vols, variant):  # noqa: F811
    """Reduced resolution and sample rate (the compose runs on the reduced
    frame at the lower left of the viewport, then the frame is stretched), a
    coarser LOD, and a clip plane, each with ClearView on."""
    raw = vols["u8"]
    eye = (0.5, 0.35, 1.3)
    iso, cv_iso, pos, params = 110.0, 170.0, (0.0, 0.0, 0.1, 1.0), (4.0, 1.0, 40.0)
    vol, r = iso_renderer(raw, iso)
    configure(r, cv_iso, pos, params)
    kw = dict(width=W, height=H, eye=eye, mode=2, isovalue=iso, want_counts=True,
              clearview=cv_kw(cv_iso, pos, params))
    if variant == "reduced":
        r.SetReducedQuality(True, True)
        kw.update(dec_screen=True, dec_sampling=True)
    elif variant == "lod1":
        r.SetLOD(1)
        kw.update(lod=1)
    else:
        r.SetClipPlane((0.3, -0.5, 0.8, 0.05))
        r.EnableClipPlane()
        kw.update(clip_plane=(0.3, -0.5, 0.8, 0.05))
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(W, H)
    r.Paint()
    img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
    ref, n, rc = O.render(raw, (BS,) * 3, 1, np.zeros((16, 4), np.float32), **kw)
    compare(img, ref, variant)
    assert cnt.shape == rc.shape and (cnt <= rc).all()


def trilinear(raw, p):
    """Value of raw ([z, y, x]) at model-space point p (the volume spans
    dims / max(dims) around the origin, texel centres at (i + 0.5) / n)."""
    dims = np.array(raw.shape[::-1], dtype=np.float64)
    u = (np.asarray(p[:3], dtype=np.float64) / (dims / dims.max()) + 0.5) * dims - 0.5
    u = np.clip(u, 0, dims - 1)
    i0 = np.minimum(np.floor(u).astype(int), (dims - 2).astype(int))
    f = u - i0
    v = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[0] if dx else 1 - f[0]) * (f[1] if dy else 1 - f[1]) * \
                    (f[2] if dz else 1 - f[2])
                v += w * float(raw[i0[2] + dz, i0[1] + dy, i0[0] + dx])
    return v


def test_gpu_clearview_focus_picking(cuda_ok, vols):  # noqa: F811
    """SetCVFocusPos: the context hit under a pixel, in model space, lies on the
    context isosurface; a pixel without a hit sends the focus far away."""
    raw = vols["u8"]
    iso = 120.0
    vol, r = iso_renderer(raw, iso)
    with pytest.raises(TvkError):
        r.SetCVFocusPos(3, 3)  # no ClearView frame yet
    configure(r, 180.0, (0.0, 0.0, 0.5, 1.0), None)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    r.Resize(W, H)
    r.Paint()
    img = r.ReadBackPixels()
    ys, xs = np.nonzero(img[..., 3] > 0)
    assert len(xs) > 20
    for k in np.linspace(0, len(xs) - 1, 6).astype(int):
        r.SetCVFocusPos(int(xs[k]), int(ys[k]))
        p = r.GetCVFocusPos()
        assert p[3] == 1.0
        assert abs(trilinear(raw, p) - iso) < 6.0, (xs[k], ys[k], p)
    ys0, xs0 = np.nonzero(img[..., 3] == 0)
    r.SetCVFocusPos(int(xs0[0]), int(ys0[0]))
    assert r.GetCVFocusPos() == (1e7, 1e7, 1e7, 0.0)
    r.SetCVFocusPos(W + 5, 0)  # outside the frame: no hit
    assert r.GetCVFocusPos()[3] == 0.0
    # the picked focus is used by the next frame
    r.SetCVFocusPos(int(xs[len(xs) // 2]), int(ys[len(xs) // 2]))
    pos = r.GetCVFocusPos()
    r.Paint()
    ref, _, _ = O.render(raw, (BS,) * 3, 1, np.zeros((16, 4), np.float32), width=W, height=H,
                         eye=(0.3, 0.4, 1.5), mode=2, isovalue=iso,
                         clearview=dict(isovalue=180.0, pos=pos))
    compare(r.ReadBackPixels(), ref, "picked focus")


def test_gpu_clearview_refused_by_batches(cuda_ok, vols):  # noqa: F811
    raw = vols["u8"]
    vol, r = iso_renderer(raw, 120.0)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    r.Resize(W, H)
    r.SetCV(True)
    b = Batch()
    with pytest.raises(TvkError):
        b.Paint([r])
    r.SetCV(False)
    b.Paint([r])
