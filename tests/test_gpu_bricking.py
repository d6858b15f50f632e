"""GPU bricking through the C ABI against the reference and the oracle.

Bit-exact: every LOD-0 brick (ghost voxels included) equals the brick the
reference's own ExtendedOctreeConverter wrote (tests/golden fixtures), per-brick
min/max equals its statistics, the global histogram counts every voxel once,
per-brick histograms, brick metadata and the maximum gradient magnitude equal
the oracle's.  Voxels the reference leaves undefined (a clamped brick whose
scanline read runs past the end of the file keeps the previous brick's bytes)
are excluded; the GPU writes the clamped value of zero there.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Volume
from tuvok_gb300.workloads import PLAIN_SMALL, numpy_blob_volume
from test_oracle_golden import FIXTURES, load, past_eof_mask

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_gpu_bricks_equal_reference_converter(cuda_ok, path):
    d, dims, bsize, ov, clamp = load(path)
    raw = d["raw"]
    vol = Volume(raw, brick_size=bsize, overlap=ov, clamp_to_edge=clamp)
    lod_sizes, lod_counts = O.lod_table(dims, bsize, ov)
    assert vol.GetLODLevelCount() == len(lod_sizes)
    assert vol.GetBrickLayout(0) == lod_counts[0]
    for lod in range(len(lod_sizes)):
        assert vol.GetDomainSize(lod) == lod_sizes[lod]
        assert vol.GetBrickLayout(lod) == lod_counts[lod]
    for i, c in enumerate(d["coords"]):
        if c[3] != 0:
            continue
        idx = vol.IndexFrom4D(c[0], c[1], c[2], 0)
        assert vol.IndexTo4D(0, idx) == (c[0], c[1], c[2], 0)
        b = vol.GetBrick((0, 0, idx))
        ref = d[f"brick{i}"]
        assert b.shape == ref.shape
        undefined = np.zeros(b.shape, dtype=bool)
        if clamp:
            undefined = past_eof_mask(dims, bsize, ov, lod_counts[0], c[:3], b.shape)
        np.testing.assert_array_equal(b[~undefined], ref[~undefined], err_msg=str(tuple(c)))
        mm = vol.MaxMinForKey((0, 0, idx))
        if not undefined.any():
            assert (mm.min_scalar, mm.max_scalar) == tuple(d["minmax"][i])
        assert (mm.min_scalar, mm.max_scalar) == O.brick_stats(b)
    h, n = vol.GetHistogram()
    np.testing.assert_array_equal(h, np.bincount(raw.reshape(-1).astype(np.int64),
                                                 minlength=h.size))
    assert n == int(raw.max()) + 1
    assert vol.GetRange() == (float(raw.min()), float(raw.max()))


@pytest.mark.parametrize("dims,dtype,bs,ov,clamp", [
    ((37, 29, 23), np.uint8, 16, 1, False),
    ((37, 29, 23), np.uint16, 16, 1, True),
    ((70, 40, 33), np.uint16, 34, 1, False),
    ((25, 14, 13), np.uint8, 16, 2, False),
    ((64, 64, 64), np.uint8, 66, 1, False),  # one brick per axis
])
def test_gpu_statistics_equal_oracle(cuda_ok, dims, dtype, bs, ov, clamp):
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 6, (3, 9), (vmax * 0.3, vmax * 0.9), vmax, seed=11,
                            noise=3)
    vol = Volume(raw, brick_size=(bs, bs, bs), overlap=ov, clamp_to_edge=clamp)
    sizes, counts = O.lod_table(dims, (bs, bs, bs), ov)
    c, e, n = O.brick_metadata(sizes[0], counts[0], (bs, bs, bs), ov)
    hist, shift = vol.GetBrickHistograms()
    assert shift == max(0, int(raw.max()).bit_length() - 8)
    nb = counts[0][0] * counts[0][1] * counts[0][2]
    for k in range(nb):
        x, y, z, _ = vol.IndexTo4D(0, k)
        ob = O.lod0_brick(raw, (bs, bs, bs), ov, clamp, (x, y, z))
        gb = vol.GetBrick((0, 0, k))
        np.testing.assert_array_equal(gb, ob)
        md = vol.GetBrickMetadata((0, 0, k))
        assert tuple(md.center) == tuple(c[k]) and tuple(md.extents) == tuple(e[k])
        assert tuple(md.n_voxels) == tuple(n[k])
        np.testing.assert_array_equal(hist[k], O.brick_hist256(ob, ov, shift))
    mg = O.max_gradient(raw, (bs, bs, bs), ov, clamp)
    assert vol.MaxGradientMagnitude() == float(np.float32(mg))


def test_gpu_bricking_plain_small_full_size(cuda_ok):
    """The 256^3 uint8 configuration at full size: every brick bit-exact."""
    w = PLAIN_SMALL
    raw = numpy_blob_volume((128, 128, 128), np.uint8, 16, (4, 20), (64, 255), 255, seed=5,
                            noise=4)
    raw = np.tile(raw, (2, 2, 2))  # 256^3 from a cheaper 128^3 source
    vol = Volume(raw, brick_size=w.brick_size, overlap=w.overlap)
    assert vol.GetBrickCount(0) == 64
    assert sum(np.prod(vol.GetBrickLayout(l)) for l in range(vol.GetLODLevelCount())) == 79
    for k in range(64):
        x, y, z, _ = vol.IndexTo4D(0, k)
        ob = O.lod0_brick(raw, w.brick_size, w.overlap, False, (x, y, z))
        np.testing.assert_array_equal(vol.GetBrick((0, 0, k)), ob)
        mm = vol.MaxMinForKey((0, 0, k))
        assert (mm.min_scalar, mm.max_scalar) == O.brick_stats(ob)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_gpu_octree_equals_reference_converter(cuda_ok, path):
    """Every LOD >= 1 brick (DownsampleBrick + FillOverlap) against the
    reference converter; with clamping only inner voxels are defined there."""
    from test_oracle_golden import is_median
    d, dims, bsize, ov, clamp = load(path)
    vol = Volume(d["raw"], brick_size=bsize, overlap=ov, clamp_to_edge=clamp, median=is_median(d))
    for i, c in enumerate(d["coords"]):
        x, y, z, lod = (int(v) for v in c)
        if lod == 0:
            continue
        k = vol.IndexFrom4D(x, y, z, lod)
        b = vol.GetBrick((0, lod, k))
        ref = d[f"brick{i}"]
        assert b.shape == ref.shape, (tuple(c), b.shape, ref.shape)
        if clamp:
            np.testing.assert_array_equal(b[ov:-ov, ov:-ov, ov:-ov], ref[ov:-ov, ov:-ov, ov:-ov],
                                          err_msg=str(tuple(c)))
        else:
            np.testing.assert_array_equal(b, ref, err_msg=str(tuple(c)))
            mm = vol.MaxMinForKey((0, lod, k))
            assert (mm.min_scalar, mm.max_scalar) == tuple(d["minmax"][i])


@pytest.mark.parametrize("dims,dtype,bs,ov,clamp,median", [
    ((61, 47, 39), np.uint16, 18, 1, False, False),
    ((61, 47, 39), np.uint8, 18, 1, True, False),
    ((50, 50, 50), np.uint8, 10, 1, False, True),
    ((33, 70, 21), np.uint16, 14, 2, False, True),
])
def test_gpu_octree_equals_oracle(cuda_ok, dims, dtype, bs, ov, clamp, median):
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 9, (2, 8), (vmax * 0.2, vmax), vmax, seed=41, noise=5)
    vol = Volume(raw, brick_size=(bs, bs, bs), overlap=ov, clamp_to_edge=clamp, median=median)
    ref = O.build_octree(raw, (bs, bs, bs), ov, clamp=clamp, median=median)
    sizes, counts = O.lod_table(dims, (bs, bs, bs), ov)
    i = 0
    for lod, lc in enumerate(counts):
        for k in range(lc[0] * lc[1] * lc[2]):
            b = vol.GetBrick((0, lod, k))
            if clamp and lod > 0:  # both sides define inner voxels only
                np.testing.assert_array_equal(b[ov:-ov, ov:-ov, ov:-ov],
                                              ref[i][ov:-ov, ov:-ov, ov:-ov])
            else:
                np.testing.assert_array_equal(b, ref[i], err_msg=f"lod {lod} brick {k}")
                mm = vol.MaxMinForKey((0, lod, k))
                assert (mm.min_scalar, mm.max_scalar) == O.brick_stats(ref[i])
            i += 1
    assert i == len(ref)


@pytest.mark.parametrize("dims,dtype,bs,ov,clamp,bins", [
    ((37, 29, 23), np.uint8, 16, 1, False, 0),
    ((30, 20, 25), np.uint16, 12, 2, False, 0),
    ((40, 33, 21), np.uint8, 18, 1, True, 0),
    ((40, 33, 21), np.uint8, 18, 1, False, 64),
    ((26, 19, 31), np.uint16, 14, 1, False, 300),
    ((70, 64, 45), np.uint16, 34, 1, False, 0),
])
def test_gpu_histogram2d_equals_oracle(cuda_ok, dims, dtype, bs, ov, clamp, bins):
    """Histogram2DDataBlock's value x |gradient| counts, bin for bin."""
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 6, (3, 9), (vmax * 0.3, vmax * 0.9), vmax, seed=3,
                            noise=3)
    vol = Volume(raw, brick_size=(bs, bs, bs), overlap=ov, clamp_to_edge=clamp)
    h, g = vol.Get2DHistogram(bins)
    n = int(raw.max()) + 1
    ref, rg = O.histogram2d(raw, (bs, bs, bs), ov, clamp, value_bins=bins or n)
    assert h.shape == ref.shape
    np.testing.assert_array_equal(h, ref)
    assert g == float(np.float32(rg))


def test_gpu_histogram2d_flat_and_no_overlap(cuda_ok):
    raw = np.full((16, 16, 16), 40, dtype=np.uint8)
    vol = Volume(raw, brick_size=(10, 10, 10), overlap=1, clamp_to_edge=True)
    h, g = vol.Get2DHistogram()
    # clamped borders, so max |g| = 0: every voxel lands in gradient bin 0
    assert g == 0.0 and h.shape == (41, 256) and int(h[40, 0]) == raw.size
    assert int(h.sum()) == raw.size
    raw[7:9, 6:10, 5:8] = 90
    vol = Volume(raw, brick_size=(10, 10, 10), overlap=1)
    ref, _ = O.histogram2d(raw, (10, 10, 10), 1)
    np.testing.assert_array_equal(vol.Get2DHistogram()[0], ref)
    from tuvok_gb300 import TvkError
    with pytest.raises(TvkError) as e:
        Volume(raw, brick_size=(8, 8, 8), overlap=0).Get2DHistogram()
    assert "UNSUPPORTED" in str(e.value)


def test_gpu_histogram2d_full_size_properties(cuda_ok):
    """256^3 uint8: every inner voxel counted once, each value row sums to the
    1D histogram, and the top gradient bin is occupied."""
    w = PLAIN_SMALL
    raw = numpy_blob_volume((128, 128, 128), np.uint8, 16, (4, 20), (64, 255), 255, seed=5,
                            noise=4)
    raw = np.tile(raw, (2, 2, 2))
    vol = Volume(raw, brick_size=w.brick_size, overlap=w.overlap)
    h, g = vol.Get2DHistogram()
    h1, n = vol.GetHistogram()
    assert h.shape == (n, 256)
    np.testing.assert_array_equal(h.sum(axis=1), h1[:n])
    assert int(h[:, 254:].sum()) >= 1 and g == vol.MaxGradientMagnitude()


def test_gpu_brick_key_errors(cuda_ok):
    raw = np.zeros((8, 8, 8), dtype=np.uint8)
    vol = Volume(raw, brick_size=(6, 6, 6), overlap=1)
    from tuvok_gb300 import TvkError
    with pytest.raises(TvkError):
        vol.GetBrick((0, 0, 10 ** 6))
    assert vol.GetBrick((0, 1, 0)).shape == (6, 6, 6)  # LOD 1: 4^3 inner + ghost
    with pytest.raises(TvkError):
        vol.GetBrick((0, vol.GetLODLevelCount(), 0))
    with pytest.raises(TvkError):
        vol.IndexFrom4D(9, 0, 0, 0)
    only0 = Volume(raw, brick_size=(6, 6, 6), overlap=1, lod0_only=True)
    with pytest.raises(TvkError) as e:
        only0.GetBrick((0, 1, 0))
    assert "UNSUPPORTED" in str(e.value)


def cell_tables(d):
    """Macro-cell (min, max) of a brick [z, y, x]: cell c covers voxels 2c ..
    2c + 2 on each axis, clamped to the brick."""
    lo, hi = d.astype(np.int64), d.astype(np.int64)
    for axis in (2, 1, 0):
        n = d.shape[axis]
        i0 = 2 * np.arange((n - 1) // 2 + 1)
        idx = [i0, np.minimum(i0 + 1, n - 1), np.minimum(i0 + 2, n - 1)]
        lo = np.minimum.reduce([np.take(lo, i, axis=axis) for i in idx])
        hi = np.maximum.reduce([np.take(hi, i, axis=axis) for i in idx])
    return lo, hi


@pytest.mark.parametrize("dims,dtype,bs,ov", [
    ((61, 47, 39), np.uint16, (18, 18, 18), 1),
    ((50, 41, 33), np.uint8, (17, 12, 9), 1),      # odd and even brick sizes, odd LODs
    ((250, 30, 21), np.uint16, (226, 18, 10), 1),  # > 96 cells along x: two passes
    ((25, 14, 13), np.uint8, (16, 16, 16), 2),
])
def test_gpu_cell_minmax_equals_brick_data(cuda_ok, dims, dtype, bs, ov):
    """The empty-space tables of every brick of every LOD: min/max of the
    (up to) 3^3 voxels each cell's samples can touch, from the brick itself."""
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 7, (2, 8), (vmax * 0.2, vmax), vmax, seed=23, noise=5)
    vol = Volume(raw, brick_size=bs, overlap=ov)
    i = 0
    for lod in range(vol.GetLODLevelCount()):
        for k in range(vol.GetBrickCount(lod)):
            b = vol.GetBrick((0, lod, k))
            lo, hi = vol.GetCellMinMax(i)
            rlo, rhi = cell_tables(b)
            np.testing.assert_array_equal(lo, rlo, err_msg=f"lod {lod} brick {k} min")
            np.testing.assert_array_equal(hi, rhi, err_msg=f"lod {lod} brick {k} max")
            i += 1
