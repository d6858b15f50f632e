"""The CPU oracle's bricking half, pinned against the reference.

* IO/test/rebricking.h golden vectors (8x8x1 uint16 ramp, brick 16, overlap 2:
  12x12x5 bricks, inner voxels equal the ramp, min/max including ghost);
* fixtures made by the reference's own ExtendedOctreeConverter
  (tests/golden/make_golden.py): every LOD-0 brick and its statistics;
* the live reference converter on fresh random inputs, where it was built.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import refconv

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("*.npz"))


def load(path):
    d = np.load(path)
    x, y, z, bs, ov, clamp = (int(v) for v in d["meta"])
    return d, (x, y, z), (bs, bs, bs), ov, bool(clamp)


def test_rebricking_h_ramp():
    # IO/test/rebricking.h:12-35, 214-242
    raw = np.arange(64, dtype=np.uint16).reshape(1, 8, 8)
    sizes, counts = O.lod_table((8, 8, 1), (16, 16, 16), 2)
    assert sizes[0] == (8, 8, 1) and counts[0] == (1, 1, 1)
    assert len(sizes) == 4  # 8 -> 4 -> 2 -> 1, one brick each
    b = O.lod0_brick(raw, (16, 16, 16), 2, False, (0, 0, 0))
    assert b.shape == (5, 12, 12)  # rebricking.h:223-225 (x=12, y=12, z=5)
    assert (b[2, 2:10, 2:10] == raw[0]).all()  # rebricking.h:176-187
    assert O.brick_stats(b) == (0.0, 63.0)  # min 0 from the zero ghost
    # everything outside the inner 8x8x1 is ghost and zero without clamping
    m = np.ones_like(b, dtype=bool)
    m[2, 2:10, 2:10] = False
    assert (b[m] == 0).all()


def test_lod_tables_of_the_configs():
    # ExtendedOctree::ComputeMetadata: 256^3 at brick 66/overlap 1 -> 9 LODs, 79 bricks;
    # 1024^3 at brick 130/overlap 1 -> 11 LODs, 592 bricks
    s, c = O.lod_table((256, 256, 256), (66, 66, 66), 1)
    assert len(s) == 9 and sum(a * b * d for a, b, d in c) == 79
    s, c = O.lod_table((1024, 1024, 1024), (130, 130, 130), 1)
    assert len(s) == 11 and sum(a * b * d for a, b, d in c) == 592


def past_eof_mask(dims, bsize, ov, counts, coords, shape):
    """Voxels whose scanline read in GetInputBrick (ExtendedOctreeConverter.cpp:
    288-373) starts past the end of the raw file.  Without clamping the brick
    buffer was zeroed first, so they read 0; with clamping the reference leaves
    whatever the previous brick left in its reused buffer there (undefined), and
    ClampToEdge (:376-462) copies such voxels on into the border planes."""
    nz, ny, nx = shape
    core = [b - 2 * ov for b in bsize]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    g = []
    inside = np.ones(shape, dtype=bool)
    for a, loc in enumerate((i, j, k)):
        first, last = coords[a] == 0, coords[a] == counts[a] - 1
        if first:
            loc = np.maximum(loc, ov)
        if last:
            loc = np.minimum(loc, shape[2 - a] - 1 - ov)
        s = ov if first else 0
        e = shape[2 - a] - (ov if last else 0)
        inside &= (loc >= s) & (loc < e)
        g.append(coords[a] * core[a] + loc - ov)
    lin = g[0] + g[1] * dims[0] + g[2] * dims[0] * dims[1]
    return inside & (lin >= dims[0] * dims[1] * dims[2])


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_lod0_equals_reference_converter(path):
    d, dims, bsize, ov, clamp = load(path)
    raw = d["raw"]
    coords, sizes, minmax = d["coords"], d["sizes"], d["minmax"]
    lod_sizes, lod_counts = O.lod_table(dims, bsize, ov)
    # the converter's brick list covers every LOD of the oracle's table
    assert len(coords) == sum(a * b * c for a, b, c in lod_counts)
    n0 = 0
    for i, c in enumerate(coords):
        if c[3] != 0:
            continue
        n0 += 1
        b = O.lod0_brick(raw, bsize, ov, clamp, tuple(c[:3]))
        assert b.shape == tuple(sizes[i][::-1])
        ref = d[f"brick{i}"]
        undefined = np.zeros(b.shape, dtype=bool)
        if clamp:
            undefined = past_eof_mask(dims, bsize, ov, lod_counts[0], c[:3], b.shape)
        np.testing.assert_array_equal(b[~undefined], ref[~undefined], err_msg=f"brick {tuple(c)}")
        if not undefined.any():
            assert O.brick_stats(b) == tuple(minmax[i])
    assert n0 == lod_counts[0][0] * lod_counts[0][1] * lod_counts[0][2]


def is_median(d):
    return "median" in d.files and bool(d["median"][0])


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_octree_equals_reference_converter(path):
    """Every LOD >= 1 brick: DownsampleBrick (mean or median) + FillOverlap in
    the reference's sequential order, including the corner ghosts it leaves
    at zero.  With clamping the reference reuses an uncleared buffer, so only
    inner voxels are defined there."""
    d, dims, bsize, ov, clamp = load(path)
    bricks = O.build_octree(d["raw"], bsize, ov, clamp=clamp, median=is_median(d))
    assert len(bricks) == len(d["coords"])
    for i, c in enumerate(d["coords"]):
        if c[3] == 0:
            continue
        ref = d[f"brick{i}"]
        assert bricks[i].shape == ref.shape
        if clamp:
            np.testing.assert_array_equal(bricks[i][ov:-ov, ov:-ov, ov:-ov],
                                          ref[ov:-ov, ov:-ov, ov:-ov], err_msg=str(tuple(c)))
        else:
            np.testing.assert_array_equal(bricks[i], ref, err_msg=str(tuple(c)))
            assert O.brick_stats(bricks[i]) == tuple(d["minmax"][i])


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_histogram_counts_every_voxel_once(path):
    d, dims, bsize, ov, clamp = load(path)
    raw = d["raw"]
    h, n = O.histogram1d(raw, bsize, ov)
    ref = np.bincount(raw.reshape(-1).astype(np.int64), minlength=h.size)
    np.testing.assert_array_equal(h, ref)
    assert n == int(raw.max()) + 1


def test_oracle_metadata_tiles_the_unit_box():
    sizes, counts = O.lod_table((37, 29, 23), (16, 16, 16), 1)
    c, e, n = O.brick_metadata(sizes[0], counts[0], (16, 16, 16), 1)
    lo = (c - e / 2).min(axis=0)
    hi = (c + e / 2).max(axis=0)
    norm = np.array([37, 29, 23]) / 37.0
    np.testing.assert_allclose(lo, -norm / 2, atol=1e-6)
    np.testing.assert_allclose(hi, norm / 2, atol=1e-6)
    assert (n[:, 0] <= 16).all()


@pytest.mark.skipif(not refconv.available(), reason="reference converter not built here")
@pytest.mark.parametrize("dims,dtype,bs,ov,clamp", [
    ((50, 20, 17), np.uint8, 18, 1, False),
    ((50, 20, 17), np.uint16, 18, 1, True),
    ((31, 31, 9), np.uint16, 10, 3, False),
])
def test_oracle_matches_live_reference(dims, dtype, bs, ov, clamp, tmp_path):
    rng = np.random.default_rng(7)
    raw = rng.integers(0, 200, size=dims[::-1]).astype(dtype)
    bricks = refconv.convert(raw, (bs, bs, bs), ov, clamp=clamp, scratch=str(tmp_path))
    for b in bricks:
        if b["coords"][3] != 0:
            continue
        mine = O.lod0_brick(raw, (bs, bs, bs), ov, clamp, b["coords"][:3])
        np.testing.assert_array_equal(mine, b["data"])
        assert O.brick_stats(mine) == (b["min"], b["max"])


@pytest.mark.skipif(not refconv.available(), reason="reference converter not built here")
@pytest.mark.parametrize("dims,dtype,bs,ov,clamp,bins", [
    ((37, 29, 23), np.uint8, 16, 1, False, 0),
    ((30, 20, 25), np.uint16, 12, 2, False, 0),
    ((40, 33, 21), np.uint8, 18, 1, True, 0),
    ((40, 33, 21), np.uint8, 18, 1, False, 64),     # values scaled into fewer bins
    ((26, 19, 31), np.uint16, 14, 1, False, 300),
    ((16, 16, 16), np.uint8, 10, 1, False, 0),      # flat volume with one bump
])
def test_oracle_histograms_equal_live_reference(dims, dtype, bs, ov, clamp, bins, tmp_path):
    """Histogram1DDataBlock and Histogram2DDataBlock of the reference, run on the
    same input, against the oracle's restatement."""
    from tuvok_gb300.workloads import numpy_blob_volume
    vmax = 255 if dtype == np.uint8 else 4095
    if dims == (16, 16, 16):
        raw = np.full(dims[::-1], 40, dtype=dtype)
        raw[7:9, 6:10, 5:8] = 90
    else:
        raw = numpy_blob_volume(dims, dtype, 6, (3, 9), (vmax * 0.3, vmax * 0.9), vmax, seed=3,
                                noise=3)
    h1, h2, g = refconv.histograms(raw, (bs, bs, bs), ov, clamp, value_bins=bins,
                                   scratch=str(tmp_path))
    o1, n = O.histogram1d(raw, (bs, bs, bs), ov)
    assert len(h1) == n
    np.testing.assert_array_equal(h1, o1[:n])
    o2, og = O.histogram2d(raw, (bs, bs, bs), ov, clamp, value_bins=bins or n)
    assert h2.shape == o2.shape
    np.testing.assert_array_equal(h2, o2)
    assert g == float(np.float32(og))
    assert int(h2.sum()) == raw.size


def test_round_half_is_ieee_rne():
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.normal(0, 2, 2000), rng.uniform(-70000, 70000, 200),
                         [1e-8, 3e-8, 6e-5, 65504.0, 65519.99, 65520.0, 0.0, -0.0]])
    for x in xs.astype(np.float32):
        with np.errstate(over="ignore"):  # |x| >= 65520 rounds to infinity, as intended
            want = float(np.float32(np.float16(x)))
        assert O.round_half(x) == want, x


def test_glsl_pow_is_within_a_few_ulp():
    """The FP32 oracle's pow(x, y) = exp2(y log2 x) (opacity correction of
    colour samples, specular exponents other than 8 and 32) stays within one
    ulp of the exact power over opacity-correction and specular ranges."""
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(0, 1, 600), 1 - rng.uniform(0, 1e-4, 150),
                         rng.uniform(0, 1e-3, 100), [2.0 ** -24, 0.5, 0.25, 1 - 2.0 ** -24]])
    ys = np.concatenate([[1 / 1.5, 1.0, 2.0, 1 / 0.75, 0.5, 3.7, 16.0, 64.0, 128.0],
                         rng.uniform(0.1, 100, 6)])
    worst = 0.0
    for y in ys.astype(np.float32):
        for x in xs.astype(np.float32):
            got = np.float32(O.pow01(x, y))
            exact = float(x) ** float(y)
            if exact < 2.0 ** -125:
                assert got <= 2.0 ** -124
                continue
            ulp = np.spacing(np.float32(exact))
            worst = max(worst, abs(float(got) - exact) / float(ulp))
    assert worst <= 1.0, worst
    assert O.pow01(0.0, 1.5) == 0.0 and O.pow01(1.0, 1.5) == 1.0 and O.pow01(0.3, 0.0) == 1.0


def test_oracle_clip_plane_properties():
    """The oracle's clip plane: a plane beyond the volume changes nothing, one
    that cuts everything leaves an empty frame, and a half cut removes samples."""
    import numpy as np
    from tuvok_gb300.workloads import numpy_blob_volume
    raw = numpy_blob_volume((24, 20, 18), np.uint8, 4, (3, 7), (80, 255), 255, 5, 0)
    tf = np.zeros((256, 4), dtype=np.float32)
    tf[:, 0] = tf[:, 3] = np.linspace(0, 0.5, 256)
    kw = dict(width=24, height=20, eye=(0.3, 0.4, 1.5), want_counts=True)
    base, n, _ = O.render(raw, (10, 10, 10), 1, tf, **kw)
    same, n2, _ = O.render(raw, (10, 10, 10), 1, tf, clip_plane=(1, 0, 0, -10), **kw)
    assert np.array_equal(base, same) and n == n2
    none, n3, _ = O.render(raw, (10, 10, 10), 1, tf, clip_plane=(1, 0, 0, 10), **kw)
    assert not none.any() and n3 == 0
    half, n4, _ = O.render(raw, (10, 10, 10), 1, tf, clip_plane=(1, 0, 0, 0), **kw)
    assert 0 < n4 < n


def test_oracle_clearview_properties():
    """The oracle's ClearView (Compose-CV-FS.glsl): with the focus point far
    away (the picking miss, GLRenderer.cpp:2848-2850) the blend factor is 1 and
    the border term 0, so the frame is the plain isosurface frame bit for bit;
    the focus pass adds samples; a focus point on the surface with no
    curvature weight reveals the focus surface (red) around it."""
    from tuvok_gb300.workloads import numpy_blob_volume
    raw = numpy_blob_volume((26, 22, 20), np.uint8, 5, (3, 7), (80, 255), 255, 7, 0)
    tf = np.zeros((16, 4), dtype=np.float32)
    kw = dict(width=40, height=32, eye=(0.4, 0.3, 1.4), mode=2, isovalue=90.0,
              want_counts=True)
    iso, n_iso, c_iso = O.render(raw, (10, 10, 10), 1, tf, **kw)
    assert (iso[..., 3] > 0).mean() > 0.05
    far = dict(isovalue=160.0, pos=(1e7, 1e7, 1e7, 0.0))
    cv, n_cv, c_cv = O.render(raw, (10, 10, 10), 1, tf, clearview=far, **kw)
    assert np.array_equal(cv, iso)
    assert n_cv > n_iso and (c_cv >= c_iso).all()
    near = dict(isovalue=160.0, pos=(0.0, 0.0, 0.0, 1.0), context_scale=0.0, size=3.0,
                color=(1.0, 0.0, 0.0))
    cv2, _, _ = O.render(raw, (10, 10, 10), 1, tf, clearview=near, **kw)
    changed = np.abs(cv2 - iso).max(axis=-1) > 1e-3
    assert changed.any() and not changed.all()
    assert ((cv2[..., 3] == 0) == (iso[..., 3] == 0)).all()


def test_oracle_color_volume_properties():
    """The oracle's colour (RGBA8) volumes: bricks copy the 4-byte voxels with
    their ghost layer; zero alpha draws nothing; the alpha channel's isosurface
    covers the pixels a scalar volume of the same alpha bytes covers."""
    from tuvok_gb300.workloads import numpy_blob_volume
    dims = (22, 18, 16)
    ch = [numpy_blob_volume(dims, np.uint8, 4, (3, 7), (80, 255), 255, 40 + k, 2)
          for k in range(4)]
    rgba = np.stack(ch, axis=-1)
    for clamp in (False, True):
        for c in [(0, 0, 0), (1, 1, 1), (2, 1, 0)]:
            b = O.lod0_brick(rgba, (10, 10, 10), 1, clamp, c)
            for k in range(4):
                np.testing.assert_array_equal(b[..., k], O.lod0_brick(ch[k], (10, 10, 10), 1,
                                                                      clamp, c))
    tf = np.ones((64, 4), dtype=np.float32)
    kw = dict(width=30, height=24, eye=(0.4, 0.3, 1.4), want_counts=True)
    clear = rgba.copy()
    clear[..., 3] = 0
    img, n, _ = O.render(clear, (10, 10, 10), 1, tf, **kw)
    assert n > 0 and not img.any()
    img, n, _ = O.render(rgba, (10, 10, 10), 1, tf, lighting=True, **kw)
    assert (img[..., 3] > 0).mean() > 0.05 and np.isfinite(img).all()
    ciso, _, _ = O.render(rgba, (10, 10, 10), 1, tf, mode=2, isovalue=120.0, **kw)
    siso, _, _ = O.render(ch[3], (10, 10, 10), 1, tf, mode=2, isovalue=120.0, **kw)
    cov_c, cov_s = ciso[..., 3] > 0, siso[..., 3] > 0
    assert (cov_c | ~cov_s).all() and (cov_c != cov_s).mean() < 0.01 and cov_c.mean() > 0.05
