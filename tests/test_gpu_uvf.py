"""tvk_volume_open_uvf over the UVF fixtures written by the reference's UVF
writer (tests/golden/uvf, see make_uvf_fixtures.py): the volume of timestep t
is the ExtendedOctree of the t-th TOC block, brick for brick the file's bytes,
with LOD 0, the data range, the maximum gradient and a rendered frame equal to
the volume bricked directly from timestep t's voxels; the MD5 is checked when
asked for."""
import json
from pathlib import Path

import numpy as np
import pytest

from tuvok_gb300 import Renderer, TvkError, Volume, read_uvf_blocks
from test_gpu_render import ramp_tf

pytestmark = pytest.mark.gpu

UVF = Path(__file__).resolve().parent / "golden" / "uvf"
CASES = json.loads((UVF / "cases.json").read_text())
TIMESTEPS = [(c, t) for c in CASES for t in range(c["timesteps"])]


def frame(vol, bins):
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(ramp_tf(bins))
    r.SetUseLighting(True)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.4, 0.3, 1.4))
    r.Resize(48, 40)
    r.Paint()
    return r.ReadBackPixels().copy()


@pytest.mark.parametrize("case,t", TIMESTEPS, ids=[f"{c['name']}-t{t}" for c, t in TIMESTEPS])
def test_gpu_uvf_timestep_matches_direct_bricking(cuda_ok, case, t):
    path = UVF / f"{case['name']}.uvf"
    raw = np.load(UVF / f"{case['name']}.npy")[t]
    v = Volume.FromUVF(path, timestep=t, verify=case["checksum"] == 2,
                       clamp_to_edge=case["clamp"])
    ref = Volume(raw, brick_size=case["brick_size"], overlap=case["overlap"],
                 clamp_to_edge=case["clamp"])
    _, blocks = read_uvf_blocks(path)
    toc = [b for b in blocks if b["semantics"] == 9][t]
    eo = Volume.FromExtendedOctree(path, offset=toc["offset"] + toc["header_bytes"],
                                   clamp_to_edge=case["clamp"])
    assert v.GetLODLevelCount() == eo.GetLODLevelCount() == ref.GetLODLevelCount()
    for lod in range(v.GetLODLevelCount()):
        for k in range(v.GetBrickCount(lod)):
            key = (0, lod, k)
            got = v.GetBrick(key)
            np.testing.assert_array_equal(got, eo.GetBrick(key), err_msg=str(key))
            if lod == 0:
                np.testing.assert_array_equal(got, ref.GetBrick(key), err_msg=str(key))
    assert v.GetRange() == ref.GetRange()
    assert v.MaxGradientMagnitude() == ref.MaxGradientMagnitude()
    bins = 256 if case["dtype"] == "u8" else 1024
    np.testing.assert_array_equal(frame(v, bins), frame(ref, bins))


def test_gpu_uvf_timesteps_differ(cuda_ok):
    """Each timestep opens its own TOC block: the frames of timesteps 0 and 1
    differ, as their voxels do."""
    case = next(c for c in CASES if c["timesteps"] >= 2 and c["components"] == 1)
    path = UVF / f"{case['name']}.uvf"
    a = frame(Volume.FromUVF(path, timestep=0), 256)
    b = frame(Volume.FromUVF(path, timestep=1), 256)
    assert not np.array_equal(a, b)


def test_gpu_uvf_refuses_damaged_checksum(cuda_ok, tmp_path):
    case = next(c for c in CASES if c["checksum"] == 2)
    buf = bytearray((UVF / f"{case['name']}.uvf").read_bytes())
    buf[-1] ^= 0x5A
    bad = tmp_path / "bad.uvf"
    bad.write_bytes(bytes(buf))
    with pytest.raises(TvkError, match="checksum"):
        Volume.FromUVF(bad, verify=True)
    v = Volume.FromUVF(bad, verify=False, clamp_to_edge=case["clamp"])
    assert v.GetBrickCount(0) > 0
