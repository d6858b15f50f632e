"""The DynamicBrickingDS restatement in oracle/rebrick.cpp against the golden
values of the reference's own tests (IO/test/rebricking.h).

The reference source there is an 8x8x1 ramp 0..63 converted with bricks of 16
and an overlap of 2 (rebricking.h:12-45); brick sizes given to DynamicBrickingDS
include the ghost voxels.
"""
import numpy as np
import pytest

import oracle as O

RAMP = np.arange(64, dtype=np.uint8).reshape(1, 8, 8)
SRC = (16, 16, 16)


def reb(tgt, mm_mode=1, raw=RAMP, src=SRC, ov=2, **kw):
    return O.rebrick(raw, src, ov, tgt, mm_mode=mm_mode, **kw)


def test_same_size_rebrick_keeps_the_source_bricks():
    # tsimple / tdata_simple / tvoxel_count / tbsizes (rebricking.h:117-120, 209-243, 275-285, 357-367)
    r = reb((16, 16, 16))
    lod0 = [b for b in r if b["lod"] == 0]
    assert len(lod0) == 1 and lod0[0]["n_voxels"] == (12, 12, 5)
    src = O.lod0_brick(RAMP, SRC, 2, False, (0, 0, 0))
    np.testing.assert_array_equal(lod0[0]["data"], src)
    assert (lod0[0]["data"][2, 2:10, 2:10] == RAMP[0]).all()
    # GetMaxUsedBrickSizes over every brick
    used = np.max([b["n_voxels"] for b in r], axis=0)
    assert tuple(used) == (12, 12, 5)


def test_two_way_splits_give_five_bricks():
    # tmake_two, ty (rebricking.h:122-126, 134-139): 2 at LOD 0 + 1 per coarser LOD
    assert len(reb((8, 16, 16))) == 5
    assert len(reb((16, 8, 16))) == 5


@pytest.mark.parametrize("tgt", [(9, 16, 16), (9, 9, 16)])
def test_uneven_split_throws(tgt):
    # tuneven, tuneven_multiple_dims (rebricking.h:128-131, 141-145)
    with pytest.raises(O.RebrickError) as e:
        reb(tgt)
    assert e.value.code == -1


def test_half_split_voxels():
    # verify_half_split / tdata_half_split / tvoxel_count (rebricking.h:245-272, 286-296)
    r = reb((6, 16, 16))
    b0, b1 = r[0], r[1]
    assert b0["lod"] == 0 and b0["n_voxels"] == (6, 12, 5) and b1["n_voxels"] == (6, 12, 5)
    d = b0["data"]
    assert d.size == 6 * 12 * 5
    # d[slice*2 + y*6 + x] == data[y-2][x-2] for y in [2, 10), x in [2, 4)
    np.testing.assert_array_equal(d[2, 2:10, 2:4], RAMP[0, 0:8, 0:2])


def test_minmax_dynamic_includes_the_ghost():
    # tminmax_dynamic (rebricking.h:390-416)
    for mode in (1, 2):  # MM_PRECOMPUTE and MM_DYNAMIC agree
        r = reb((16, 8, 16), mm_mode=mode)
        assert r[0]["data"].size == 12 * 8 * 5
        assert (r[0]["min"], r[0]["max"]) == (0.0, 47.0)  # 47: includes the ghost
        assert (r[1]["min"], r[1]["max"]) == (0.0, 63.0)
    # MM_SOURCE forwards the source brick's statistics
    r = reb((16, 8, 16), mm_mode=0)
    assert (r[0]["min"], r[0]["max"]) == (0.0, 63.0) and r[0]["src_index"] == 0


def test_metadata_unchanged_when_bricks_cover_the_source():
    # tmetadata (rebricking.h:298-313)
    r = reb((16, 16, 16))
    c, e, n = O.brick_metadata((8, 8, 1), (1, 1, 1), SRC, 2)
    assert r[0]["center"] == tuple(c[0])
    assert r[0]["extents"][2] == e[0][2]


def test_engine_sized_split():
    # trealdata_make_two_lod2 (rebricking.h:331-356): a 256x256x128 uint8 volume
    # bricked at 256 / overlap 2, rebricked to 130x256x256.  Sizes do not depend
    # on the values, so a seeded random volume stands in for the engine data.
    rng = np.random.default_rng(1)
    raw = rng.integers(0, 256, size=(128, 256, 256), dtype=np.uint8)
    r = reb((130, 256, 256), raw=raw, src=(256, 256, 256))
    lod0 = [b for b in r if b["lod"] == 0]
    assert lod0[0]["n_voxels"] == (130, 256, 132)
    assert lod0[1]["n_voxels"] == (130, 256, 132)
    assert lod0[2]["n_voxels"] == (8, 256, 132)
    lod1 = [b for b in r if b["lod"] == 1]
    assert lod1[0]["data"].size == 130 * 132 * 68
    sizes, counts = O.lod_table((256, 256, 128), (256, 256, 256), 2)
    lod2 = [b for b in r if b["lod"] == 2]
    assert lod2[0]["n_voxels"] == tuple(O.brick_size(sizes[2], counts[2], (256, 256, 256), 2,
                                                     (0, 0, 0)))
    # every LOD-0 target brick is a window of its source brick
    src = O.build_octree(raw, (256, 256, 256), 2)
    for b in lod0:
        s = src[b["src_index"]]
        nx, ny, nz = b["n_voxels"]
        ox = ((b["index"] % 3) % 2) * 126  # 3 target bricks along x, 2 per source brick
        np.testing.assert_array_equal(b["data"], s[:nz, :ny, ox:ox + nx])


def test_lod0_only_source_rebricks_lod0():
    r = reb((8, 16, 16), lod0_only=True)
    assert [b["lod"] for b in r] == [0, 0]
