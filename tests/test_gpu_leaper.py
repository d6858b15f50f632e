"""The GridLeaper (tvk_pool_* / tvk_leaper_paint) against the oracle.

* visibility: the page table after RecomputeVisibility equals the oracle's
  restatement for the TF's value range or the isovalue, cached bricks included;
* one traversal pass over a page table: image, per-pixel samples and the set of
  bricks reported missing equal the oracle's pass over the same table.  The
  oracle reads every brick from its own octree, so a brick paged into the
  wrong slot, or a slot overwritten too early, shows up as an image difference;
* paging: with a cache smaller than the working set a frame pages over several
  passes (oldest slots first, the coarsest brick kept); paging from pinned host
  memory gives the same frames as paging from the device pool;
* convergence: with room for every brick the passes end when nothing is
  missing, and the resumed image matches one pass over the final table.

The LOD of a sample is ComputeLOD's uint(log2(x)), taken on both sides as the
binary exponent of the same IEEE quotient, so every pixel is held to 2/255
(max) and 0.25/255 (mean), sample counts are equal pixel for pixel and the
missing-brick requests are the same set.
"""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Pool, Renderer, TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume
from test_gpu_render import MAX_TOL, MEAN_TOL, ramp_tf, tf2d

pytestmark = pytest.mark.gpu

W, H = 80, 64
BS, OV = 18, 1


@pytest.fixture(scope="module")
def vols():
    return {
        "u8": numpy_blob_volume((61, 47, 39), np.uint8, 9, (3, 11), (80, 255), 255, 31, 3),
        "u16": numpy_blob_volume((50, 56, 33), np.uint16, 9, (3, 11), (900, 4000), 4095, 32, 20),
    }


def band_tf(n, lo, hi):
    """A TF that is zero outside [lo, hi] of its columns (empty bricks exist)
    and at least 0.04 opaque inside (so coarse bricks can be visible)."""
    t = ramp_tf(n)
    t[:, 3] = np.maximum(t[:, 3], 0.04)
    t[:int(lo * n), 3] = 0.0
    t[int(hi * n):, 3] = 0.0
    return t


def setup(raw, tf, mode, lit, iso=None, srm=1.0):
    vol = Volume(raw, brick_size=(BS, BS, BS), overlap=OV)
    r = Renderer()
    r.RegisterDataset(vol)
    if mode == 1:
        r.Set2DTransFloat(tf)
    elif mode == 0:
        r.Set1DTransFloat(tf)
    if iso is not None:
        r.SetIsoValue(iso)
    r.SetRendermode(mode)
    r.SetUseLighting(lit)
    r.SetSampleRateModifier(srm)
    r.Resize(W, H)
    return vol, r


def oracle_kw(mode, lit, iso, srm, eye):
    kw = dict(width=W, height=H, eye=eye, mode=mode, lighting=lit, srm=srm)
    if iso is not None:
        kw["isovalue"] = iso
    return kw


def compare_pass(img, cnt, ref, rc, what, count_check=True):
    d = np.abs(img.astype(np.float64) - ref.astype(np.float64))
    assert np.isfinite(img).all(), what
    assert d.max() <= MAX_TOL, f"{what}: max |diff| {d.max() * 255:.3f}/255"
    assert d.mean() <= MEAN_TOL, f"{what}: mean |diff| {d.mean() * 255:.4f}/255"
    if count_check:
        off = (cnt != rc).mean()
        assert off == 0.0, f"{what}: {off:.4%} of pixels with other sample counts"


def check_visibility(raw, tf, mode, iso, page, what):
    cached = {int(i): int(page[i]) for i in np.nonzero(page >= 3)[0]}
    if mode == 2:
        exp = O.leaper_visibility(raw, (BS, BS, BS), OV, cached, isovalue=iso)
    else:
        lo, hi = O.tf_value_limits(tf, raw.max())
        exp = O.leaper_visibility(raw, (BS, BS, BS), OV, cached, lo=lo, hi=hi)
    np.testing.assert_array_equal(page, exp, err_msg=what)


def check_missing(got, ref, what):
    diff = np.setxor1d(got, ref)
    assert diff.size == 0, f"{what}: requests differ in {diff.tolist()}"


CASES = [
    # id, volume, mode, lighting, iso value, srm, eye, TF band (1D)
    ("u8_1d", "u8", 0, False, None, 1.0, (0.3, 0.4, 1.5), (0.05, 0.95)),
    ("u8_1d_band", "u8", 0, False, None, 1.0, (0.3, 0.4, 1.5), (0.3, 0.9)),
    ("u8_1d_far", "u8", 0, False, None, 1.0, (1.4, 1.9, 3.5), (0.05, 0.95)),
    ("u16_1d_lit", "u16", 0, True, None, 1.0, (-1.1, 0.2, -0.7), (0.05, 0.95)),
    ("u8_1d_lit_srm", "u8", 0, True, None, 1.7, (0.9, -0.6, 1.2), (0.1, 0.9)),
    ("u8_2d_lit", "u8", 1, True, None, 1.0, (0.3, 0.4, 1.5), None),
    ("u8_iso", "u8", 2, False, 150.0, 1.0, (0.9, 0.6, 1.0), None),
    ("u8_iso_low", "u8", 2, False, 20.0, 1.0, (0.2, -0.5, 1.4), None),
    ("u16_iso", "u16", 2, False, 2200.0, 1.0, (-0.8, 1.1, 1.3), None),
]


def tf_for(vk, mode, band=(0.05, 0.95)):
    if mode == 1:
        return tf2d(256, 32)
    return band_tf(256 if vk == "u8" else 1024, *(band or (0.05, 0.95)))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_leaper_cold_pass_matches_oracle(cuda_ok, vols, case):
    """First pass with only the coarsest brick cached: every ray falls back to
    it and reports its own brick; the visibility flags let rays leap."""
    name, vk, mode, lit, iso, srm, eye, band = case
    raw = vols[vk]
    tf = tf_for(vk, mode, band)
    vol, r = setup(raw, tf, mode, lit, iso, srm)
    pool = Pool(vol, 1 << 30)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    info = pool.Paint(r, max_passes=1)
    page = pool.GetPageTable()
    assert info.passes == 1 and info.paged == 0 and info.resident == 1
    # only the coarsest brick is cached (flagged EMPTY when it shows nothing)
    assert (page >= 3).sum() == (1 if page[-1] >= 3 else 0)
    check_visibility(raw, tf, mode, iso, page, name)
    img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
    ref, n, rc, missing = O.leaper_render(raw, (BS, BS, BS), OV, tf, page,
                                          **oracle_kw(mode, lit, iso, srm, eye))
    compare_pass(img, cnt, ref, rc, name)
    got = pool.GetRequests()
    assert info.missing_last == got.size
    check_missing(got, missing, name)
    assert missing.size > 0 and info.converged == 0
    if page[-1] >= 3:
        assert n > 0  # rays fell back to the coarsest brick and marched it


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_leaper_converged_frame_matches_oracle(cuda_ok, vols, case):
    """Room for every brick: the frame pages until nothing is missing; its
    resumed image matches one pass over the final table, and the next frame is
    a single pass that needs nothing."""
    name, vk, mode, lit, iso, srm, eye, band = case
    raw = vols[vk]
    tf = tf_for(vk, mode, band)
    vol, r = setup(raw, tf, mode, lit, iso, srm)
    pool = Pool(vol, 1 << 30)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    info = pool.Paint(r, max_passes=64)
    assert info.converged == 1 and info.missing_last == 0 and info.passes >= 2
    assert info.paged > 0 and info.resident == info.paged + 1
    page = pool.GetPageTable()
    check_visibility(raw, tf, mode, iso, page, name)
    img = r.ReadBackPixels()
    kw = oracle_kw(mode, lit, iso, srm, eye)
    ref, n, rc, missing = O.leaper_render(raw, (BS, BS, BS), OV, tf, page, **kw)
    assert missing.size <= 1
    # resumed rays restart from the stored position: direction and step
    # rounding differ from one pass, so only the mean is held tight
    d = np.abs(img.astype(np.float64) - ref)
    assert d.mean() <= 2 * MEAN_TOL and (d.max(axis=2) > 8 / 255).mean() <= 0.01, name
    # (a fresh ray may pick another LOD than its resumed self where the level
    # lands on an integer, so a brick or two may still be asked for)
    again = pool.Paint(r, max_passes=1)
    assert again.passes == 1 and again.paged == 0 and again.missing_last <= 2
    np.testing.assert_array_equal(pool.GetPageTable(), page)
    img2, cnt2 = r.ReadBackPixels(), r.ReadSampleCounts()
    compare_pass(img2, cnt2, ref, rc, name + " second frame")


def test_gpu_leaper_paging_small_cache(cuda_ok, vols):
    """A cache of 10 slots for a view that wants more: frames page oldest
    slots first, keep the coarsest brick, and each single pass still matches
    the oracle over the table it saw."""
    raw = vols["u8"]
    tf = tf_for("u8", 0)
    vol, r = setup(raw, tf, 0, True)
    slot_bytes = BS ** 3
    pool = Pool(vol, 10 * slot_bytes)
    assert pool.GetInfo().slots == 10
    eye = (0.2, 0.3, 1.1)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    seen = set()
    for frame in range(4):
        info = pool.Paint(r, max_passes=3)
        assert info.resident == 10
        page = pool.GetPageTable()
        res = np.nonzero(page >= 3)[0]
        assert res.size == 10 and np.unique(page[res]).size == 10 and page[-1] >= 3
        assert info.paged <= 9 * (info.passes - 1)
        seen.update(res.tolist())
        # a one-pass frame sees exactly this table (no paging after its pass)
        one = pool.Paint(r, max_passes=1)
        assert one.passes == 1 and one.paged == 0
        np.testing.assert_array_equal(pool.GetPageTable(), page)
        img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
        ref, n, rc, missing = O.leaper_render(raw, (BS, BS, BS), OV, tf, page,
                                              **oracle_kw(0, True, None, 1.0, eye))
        compare_pass(img, cnt, ref, rc, f"frame {frame}")
        check_missing(pool.GetRequests(), missing, f"frame {frame}")
    assert len(seen) > 10  # bricks were replaced
    assert pool.GetInfo().paged_total >= len(seen) - 1


def test_gpu_leaper_host_paging_equals_device_paging(cuda_ok, vols):
    raw = vols["u16"]
    tf = tf_for("u16", 0)
    frames = {}
    for host in (False, True):
        vol, r = setup(raw, tf, 0, True)
        pool = Pool(vol, 12 * BS ** 3 * 2, host_source=host)
        assert pool.GetInfo().host_source == int(host)
        out = []
        for eye in [(0.3, 0.4, 1.2), (-0.9, 0.5, 0.8), (0.2, -1.3, 0.4)]:
            r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
            info = pool.Paint(r, max_passes=4)
            out.append((r.ReadBackPixels(), pool.GetPageTable(), info.paged, info.passes))
        frames[host] = out
    for (a, pa, na, sa), (b, pb, nb, sb) in zip(frames[False], frames[True]):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(pa, pb)
        assert (na, sa) == (nb, sb)


def test_gpu_leaper_visibility_follows_tf(cuda_ok, vols):
    """A TF change recomputes the flags: cached bricks that hold nothing
    visible any more become EMPTY / CHILD_EMPTY (and are evicted first)."""
    raw = vols["u8"]
    wide = band_tf(256, 0.3, 0.9)
    vol, r = setup(raw, wide, 0, False)
    pool = Pool(vol, 1 << 30)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.5))
    info = pool.Paint(r, max_passes=64)
    assert info.converged == 1
    cached_before = np.nonzero(pool.GetPageTable() >= 3)[0]
    narrow = band_tf(256, 0.8, 0.95)
    r.Set1DTransFloat(narrow)
    pool.Paint(r, max_passes=1)
    page = pool.GetPageTable()
    check_visibility(raw, narrow, 0, None, page, "narrow TF")
    still = np.nonzero(page >= 3)[0]
    assert still.size < cached_before.size  # some cached bricks turned empty
    assert set(still.tolist()) <= set(cached_before.tolist())
    # back to the wide TF: the flagged bricks are restored from their slots
    r.Set1DTransFloat(wide)
    back = pool.Paint(r, max_passes=1)
    assert back.paged == 0 and back.missing_last <= 2
    np.testing.assert_array_equal(np.nonzero(pool.GetPageTable() >= 3)[0], cached_before)


def test_gpu_leaper_errors(cuda_ok, vols):
    raw = vols["u8"]
    flat = Volume(raw, brick_size=(BS, BS, BS), overlap=OV, lod0_only=True)
    with pytest.raises(TvkError) as e:
        Pool(flat, 1 << 30)
    assert "UNSUPPORTED" in str(e.value)
    vol, r = setup(raw, ramp_tf(256), 0, False)
    with pytest.raises(TvkError):
        Pool(vol, BS ** 3)  # fewer than two slots
    other = Volume(raw[:20, :20, :20].copy(), brick_size=(BS, BS, BS), overlap=OV)
    pool = Pool(other, 1 << 30)
    with pytest.raises(TvkError) as e:
        pool.Paint(r)
    assert "STATE" in str(e.value)


def test_gpu_leaper_released_device_bricks(cuda_ok, vols):
    """Out-of-core set-up: the pool pages from its pinned host copy after the
    volume's device bricks are freed; frames equal those of a volume that
    keeps them, and every device-brick reader fails loudly."""
    raw = vols["u8"]
    tf = tf_for("u8", 0)
    imgs = []
    for release in (False, True):
        vol, r = setup(raw, tf, 0, True)
        pool = Pool(vol, 12 * BS ** 3, host_source=True)
        if release:
            vol.ReleaseBricks()
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.3, 0.4, 1.3))
        info = pool.Paint(r, max_passes=8)
        imgs.append((r.ReadBackPixels(), pool.GetPageTable(), info.paged))
        if release:
            with pytest.raises(TvkError) as e:
                r.Paint()
            assert "STATE" in str(e.value)
            with pytest.raises(TvkError):
                vol.GetBrick((0, 0, 0))
            with pytest.raises(TvkError):
                Pool(vol, 1 << 30)
    np.testing.assert_array_equal(imgs[0][0], imgs[1][0])
    np.testing.assert_array_equal(imgs[0][1], imgs[1][1])
    assert imgs[0][2] == imgs[1][2] > 0


def test_gpu_leaper_request_table_and_reset(cuda_ok, vols):
    """A 4-entry request table reports at most 4 bricks per pass, so the frame
    needs more passes to converge; PH_Reset empties the cache and the next
    pass equals a cold pass."""
    raw = vols["u8"]
    tf = tf_for("u8", 0)
    eye = (0.3, 0.4, 1.5)
    out = {}
    for size in (0, 4):
        vol, r = setup(raw, tf, 0, False)
        pool = Pool(vol, 1 << 30)
        pool.SetRequestTable(size, 10)
        assert pool.GetInfo().hash_size == (4 if size else 2859)
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
        info = pool.Paint(r, max_passes=200)
        assert info.converged == 1
        out[size] = (info.passes, info.paged, pool.GetPageTable())
        if size == 4:
            assert info.passes >= 1 + (info.paged + 3) // 4
            cold_vol, cold_r = setup(raw, tf, 0, False)
            cold = Pool(cold_vol, 1 << 30)
            cold_r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
            cold.Paint(cold_r, max_passes=1)
            pool.Reset()
            page = pool.GetPageTable()
            assert (page >= 3).sum() <= 1
            one = pool.Paint(r, max_passes=1)
            assert one.resident <= 1 and one.paged == 0
            np.testing.assert_array_equal(pool.GetPageTable(), cold.GetPageTable())
            np.testing.assert_array_equal(r.ReadBackPixels(), cold_r.ReadBackPixels())
    assert out[4][0] > out[0][0]
