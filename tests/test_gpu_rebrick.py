"""GPU rebricking (tvk_volume_rebrick, DynamicBrickingDS) against the oracle.

Bit-exact per target brick: voxels, n_voxels, centre/extents (float bits),
min/max for each MaxMinForKey mode, and the same refusals (an uneven split is
TVK_ERR_INVALID_ARG where the reference throws; a window past the end of its
source brick is TVK_ERR_UNSUPPORTED where the reference reads outside its
buffer).  The oracle is pinned to IO/test/rebricking.h in test_oracle_rebrick.py.
"""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import TvkError, Volume
from tuvok_gb300.workloads import numpy_blob_volume

pytestmark = pytest.mark.gpu

RAMP = np.arange(64, dtype=np.uint8).reshape(1, 8, 8)


def compare(raw, src_bs, ov, tgt, mm_mode, clamp=False, median=False, lod0_only=False):
    try:
        ref = O.rebrick(raw, src_bs, ov, tgt, mm_mode=mm_mode, clamp=clamp, median=median,
                        lod0_only=lod0_only)
    except O.RebrickError as e:
        src = Volume(raw, brick_size=src_bs, overlap=ov, clamp_to_edge=clamp, median=median,
                     lod0_only=lod0_only)
        with pytest.raises(TvkError) as g:
            src.Rebrick(tgt, mm_mode)
        assert ("INVALID_ARG" if e.code == -1 else "UNSUPPORTED") in str(g.value)
        return None
    src = Volume(raw, brick_size=src_bs, overlap=ov, clamp_to_edge=clamp, median=median,
                 lod0_only=lod0_only)
    vol = src.Rebrick(tgt, mm_mode)
    del src  # the rebricked volume owns its bricks
    assert vol.GetMaxBrickSize() == tuple(tgt)
    assert vol.GetMaxUsedBrickSizes() == tuple(np.max([b["n_voxels"] for b in ref], axis=0))
    for b in ref:
        key = (0, b["lod"], b["index"])
        md = vol.GetBrickMetadata(key)
        assert tuple(md.n_voxels) == b["n_voxels"], key
        np.testing.assert_array_equal(np.float32(md.center), np.float32(b["center"]))
        np.testing.assert_array_equal(np.float32(md.extents), np.float32(b["extents"]))
        if clamp and b["lod"] > 0:
            # LOD >= 1 clamped ghosts are undefined in the reference; the source
            # pools agree on inner voxels only
            continue
        np.testing.assert_array_equal(vol.GetBrick(key), b["data"], err_msg=str(key))
        mm = vol.MaxMinForKey(key)
        assert (mm.min_scalar, mm.max_scalar) == (b["min"], b["max"]), key
    return vol


@pytest.mark.parametrize("tgt", [(16, 16, 16), (8, 16, 16), (16, 8, 16), (6, 16, 16),
                                 (8, 8, 16), (9, 16, 16), (9, 9, 16)])
@pytest.mark.parametrize("mm_mode", [0, 2])
def test_gpu_rebrick_reference_test_cases(cuda_ok, tgt, mm_mode):
    compare(RAMP, (16, 16, 16), 2, tgt, mm_mode)
    compare(RAMP.astype(np.uint16) * 1000, (16, 16, 16), 2, tgt, mm_mode)


def test_gpu_rebrick_minmax_modes(cuda_ok):
    # rebricking.h:390-416: 47 and 63 include the ghost voxels
    src = Volume(RAMP, brick_size=(16, 16, 16), overlap=2)
    dyn = src.Rebrick((16, 8, 16), Volume.MM_DYNAMIC)
    assert dyn.GetBrickCount(0) == 2 and sum(
        dyn.GetBrickCount(l) for l in range(dyn.GetLODLevelCount())) == 5
    m0, m1 = dyn.MaxMinForKey((0, 0, 0)), dyn.MaxMinForKey((0, 0, 1))
    assert (m0.min_scalar, m0.max_scalar, m1.min_scalar, m1.max_scalar) == (0, 47, 0, 63)
    srcmm = src.Rebrick((16, 8, 16), Volume.MM_SOURCE).MaxMinForKey((0, 0, 0))
    assert (srcmm.min_scalar, srcmm.max_scalar) == (0, 63)


@pytest.mark.parametrize("dims,dtype,src_bs,ov,tgt,clamp,median", [
    ((61, 47, 39), np.uint16, 20, 2, (12, 12, 12), False, False),
    ((61, 47, 39), np.uint8, 20, 2, (8, 12, 20), True, False),
    ((50, 50, 50), np.uint8, 36, 2, (12, 20, 36), False, True),
    ((70, 33, 20), np.uint16, 34, 1, (18, 18, 34), False, False),  # overlap 1: the 4-quirk
    ((40, 40, 40), np.uint8, 18, 1, (10, 18, 18), False, False),
])
def test_gpu_rebrick_equals_oracle(cuda_ok, dims, dtype, src_bs, ov, tgt, clamp, median):
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 7, (2, 8), (vmax * 0.2, vmax), vmax, seed=19, noise=4)
    for mode in (0, 1):
        compare(raw, (src_bs,) * 3, ov, tgt, mode, clamp=clamp, median=median)


def test_gpu_rebrick_engine_sized(cuda_ok):
    # rebricking.h:331-356 sizes on a 256x256x128 volume bricked at 256 / overlap 2
    rng = np.random.default_rng(1)
    raw = rng.integers(0, 256, size=(128, 256, 256), dtype=np.uint8)
    vol = compare(raw, (256, 256, 256), 2, (130, 256, 256), 2)
    assert tuple(vol.GetBrickMetadata((0, 0, 0)).n_voxels) == (130, 256, 132)
    assert tuple(vol.GetBrickMetadata((0, 0, 2)).n_voxels) == (8, 256, 132)
    assert vol.GetBrick((0, 1, 0)).size == 130 * 132 * 68


def test_gpu_rebrick_lod0_only_and_refusals(cuda_ok):
    vol = compare(RAMP, (16, 16, 16), 2, (8, 16, 16), 1, lod0_only=True)
    with pytest.raises(TvkError) as e:
        vol.GetBrick((0, 1, 0))
    assert "UNSUPPORTED" in str(e.value)
    src = Volume(RAMP, brick_size=(16, 16, 16), overlap=2)
    reb = src.Rebrick((8, 16, 16))
    assert reb.GetRange() == src.GetRange()
    assert reb.MaxGradientMagnitude() == src.MaxGradientMagnitude()
    with pytest.raises(TvkError):
        reb.Get2DHistogram()
    with pytest.raises(TvkError):
        reb.Rebrick((8, 16, 16))
    from tuvok_gb300 import Renderer
    r = Renderer()
    with pytest.raises(TvkError) as e:
        r.RegisterDataset(reb)
    assert "UNSUPPORTED" in str(e.value)
