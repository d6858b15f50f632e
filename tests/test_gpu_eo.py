"""tvk_volume_open_extended_octree over the converter-written fixtures
(tests/golden/eo, made by the reference's ExtendedOctreeConverter), whatever
flags the caller guesses: every brick of every LOD of the loaded volume is the
file's brick (the decoded bytes), its statistics are those bricks' min/max,
and LOD 0, the data range, the maximum gradient and a rendered frame equal the
volume bricked from the same voxels.  (The converter leaves stale data of its
reused buffers in some ghost voxels of coarser bricks -- the loader keeps those
bricks from the file, a direct build has zeros there.)  Malformed files are
refused without touching the GPU state."""
import json
import shutil
from pathlib import Path

import numpy as np
import pytest

from tuvok_gb300 import Renderer, TvkError, Volume
from test_gpu_render import ramp_tf

pytestmark = pytest.mark.gpu

EO = Path(__file__).resolve().parent / "golden" / "eo"
CASES = json.loads((EO / "cases.json").read_text())


def direct(case):
    raw = np.load(EO / f"{case['name']}.npy")
    return raw, Volume(raw, brick_size=case["brick_size"], overlap=case["overlap"],
                       clamp_to_edge=case["clamp"], median=case["median"])


def all_keys(v):
    return [(0, lod, k) for lod in range(v.GetLODLevelCount())
            for k in range(v.GetBrickCount(lod))]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
@pytest.mark.parametrize("guess", ["right", "wrong"])
def test_gpu_eo_matches_direct_bricking(cuda_ok, case, guess):
    raw, ref = direct(case)
    flip = guess == "wrong"
    v = Volume.FromExtendedOctree(EO / f"{case['name']}.eo",
                                  clamp_to_edge=case["clamp"] ^ flip,
                                  median=case["median"] ^ flip)
    color = case["components"] == 4
    import test_eo_fixtures as F
    buf = (EO / f"{case['name']}.eo").read_bytes()
    toc = F.parse(buf)["toc"]
    for k, key in enumerate(all_keys(ref)):
        got = v.GetBrick(key)
        off, length, comp = toc[k][0], toc[k][1], toc[k][2]
        want = np.frombuffer(F.expand(buf[off:off + length], comp, got.nbytes),
                             dtype=got.dtype).reshape(got.shape)
        np.testing.assert_array_equal(got, want, err_msg=f"file brick {key}")
        if key[1] == 0:
            np.testing.assert_array_equal(got, ref.GetBrick(key), err_msg=str(key))
        if not color:
            mm = v.MaxMinForKey(key)
            assert (mm.min_scalar, mm.max_scalar) == (float(got.min()), float(got.max()))
    assert v.GetRange() == ref.GetRange()
    assert v.MaxGradientMagnitude() == ref.MaxGradientMagnitude()
    imgs = []
    for vol in (v, ref):
        r = Renderer()
        r.RegisterDataset(vol)
        r.Set1DTransFloat(ramp_tf(256 if case["dtype"] == "u8" else 1024))
        r.SetUseLighting(True)
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.4, 0.3, 1.4))
        r.Resize(48, 40)
        r.Paint()
        imgs.append(r.ReadBackPixels().copy())
    np.testing.assert_array_equal(imgs[0], imgs[1])  # LOD 0 frames


def test_gpu_eo_refuses_malformed_files(cuda_ok, tmp_path):
    with pytest.raises(TvkError):
        Volume.FromExtendedOctree(tmp_path / "missing.eo")
    src = EO / "u8_none_scanline.eo"
    with pytest.raises(TvkError):
        Volume.FromExtendedOctree(src, uvf_version=4)
    data = src.read_bytes()
    short = tmp_path / "short.eo"
    short.write_bytes(data[: len(data) // 2])
    with pytest.raises(TvkError):
        Volume.FromExtendedOctree(short)
    # a LOD-0 ghost voxel that its neighbour does not hold: no rebuild matches
    import test_eo_fixtures as F
    bad = bytearray(data)
    bad[F.parse(data)["toc"][0][0]] ^= 0x5A  # brick (0, 0, 0), corner ghost voxel
    (tmp_path / "bad.eo").write_bytes(bytes(bad))
    with pytest.raises(TvkError):
        Volume.FromExtendedOctree(tmp_path / "bad.eo")
    # a corrupt LZ4 stream: the bounded decoder refuses it
    lz = bytearray((EO / "u8_lz4hc_hilbert.eo").read_bytes())
    for i in range(len(lz) - 4000, len(lz), 7):
        lz[i] = 0xFF
    (tmp_path / "lz.eo").write_bytes(bytes(lz))
    with pytest.raises(TvkError):
        Volume.FromExtendedOctree(tmp_path / "lz.eo")
    # the same file at an offset inside a larger file (a UVF TOC block)
    wrapped = tmp_path / "wrapped.bin"
    wrapped.write_bytes(b"\0" * 123 + data)
    v = Volume.FromExtendedOctree(wrapped, offset=123)
    assert v.GetBrickCount(0) > 1
    shutil.rmtree(tmp_path, ignore_errors=True)


def test_gpu_eo_keeps_unreproducible_coarse_bricks(cuda_ok):
    """The clamp + overlap-2 fixture: the converter's coarser bricks hold stale
    buffer data in some ghost corners, so the loader keeps those bricks from
    the file (with their min/max) and every other brick from the rebuild."""
    case = [c for c in CASES if c["clamp"] and c["overlap"] == 2][0]
    raw, ref = direct(case)
    v = Volume.FromExtendedOctree(EO / f"{case['name']}.eo", clamp_to_edge=True, median=True)
    data = (EO / f"{case['name']}.eo").read_bytes()
    import test_eo_fixtures as F
    h = F.parse(data)
    differ = 0
    for key in all_keys(ref):
        a = v.GetBrick(key)
        lod, k = key[1], key[2]
        toc = sum(c[0] * c[1] * c[2] for c in h["counts"][:lod]) + k
        off, length, comp, _, _, _ = h["toc"][toc]
        stored = data[off:off + length]
        if comp == 3:
            stored = F.lz4_block(stored, a.nbytes)
        np.testing.assert_array_equal(a, np.frombuffer(stored, a.dtype).reshape(a.shape))
        mm = v.MaxMinForKey(key)
        assert (mm.min_scalar, mm.max_scalar) == (float(a.min()), float(a.max()))
        differ += int(not np.array_equal(a, ref.GetBrick(key)))
    assert differ > 0
