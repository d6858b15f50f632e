"""Writes the UVF fixtures in tests/golden/uvf/ with the reference's own UVF
writer (UVF::Create / Close with TOCBlock::FlatDataToBrickedLOD, the histogram,
max/min and key/value blocks, assembled as RAWConverter::ConvertRAWDataset
does; oracle/ref/ref_uvf.cpp, built into oracle/_ref by
tuvok_gb300.build.build_reference and bound in tests/refconv.py).  Run once in
a checkout that has the reference sources; the fixtures are committed, so the
tests need neither the reference nor this script.

Each case: seeded volumes, one per timestep (saved as .npy, [t, z, y, x] or
[t, z, y, x, 4]), the .uvf file, and in cases.json the block table that the
reference's own parser (UVF::Open, with the checksum verified where the file
has an MD5) reports for it.  The 2D histogram block is left out of the
committed files for size (a 16-bit volume's holds up to 4096 x 256 counts);
the live cross-check in tests/test_uvf.py writes files with it."""
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import refconv  # noqa: E402
from tuvok_gb300.workloads import numpy_blob_volume  # noqa: E402

OUT = Path(__file__).resolve().parent / "uvf"

# name, dims (x, y, z), dtype, components, timesteps, brick size, overlap,
# clamp, compression (0 none, 1 zlib, 3 LZ4), level, layout (0 scanline,
# 1 Morton, 2 Hilbert), checksum (0 none, 1 CRC32, 2 MD5), big-endian headers,
# metadata block first, histograms (0 none, 1 the 1D block)
CASES = [
    ("u8_two_timesteps_md5", (21, 17, 13), "u8", 1, 2, (8, 8, 8), 1, False, 0, 0, 0, 2, False,
     False, 1),
    ("u16_lz4_bigendian_md5_kvfirst", (20, 23, 11), "u16", 1, 1, (10, 9, 8), 2, True, 3, 1, 1, 2,
     True, True, 1),
    ("rgba_zlib_hilbert_md5", (14, 12, 10), "u8", 4, 1, (8, 8, 8), 1, True, 1, 6, 2, 2, False,
     False, 0),
    ("u8_crc32_three_timesteps", (12, 10, 9), "u8", 1, 3, (8, 8, 8), 1, False, 0, 0, 0, 1, False,
     False, 0),
]


def volumes(dims, dt, comps, timesteps, seed):
    out = []
    for t in range(timesteps):
        s = seed + 7 * t
        if comps == 4:
            v = np.stack([numpy_blob_volume(dims, np.uint8, 3, (2, 5), (60, 255), 255, s + k, 3)
                          for k in range(4)], axis=-1)
        elif dt == "u8":
            v = numpy_blob_volume(dims, np.uint8, 4, (2, 6), (60, 255), 255, s, 3)
        else:
            v = numpy_blob_volume(dims, np.uint16, 4, (2, 6), (900, 4000), 4095, s, 20)
        out.append(v)
    return np.ascontiguousarray(np.stack(out))


def main():
    OUT.mkdir(exist_ok=True)
    meta = []
    with tempfile.TemporaryDirectory() as tmp:
        for i, (name, dims, dt, comps, ts, bs, ov, clamp, comp, level, layout, checksum, be,
                kv_first, hist) in enumerate(CASES):
            raw = volumes(dims, dt, comps, ts, 900 + 10 * i)
            np.save(OUT / f"{name}.npy", raw)
            path = OUT / f"{name}.uvf"
            refconv.write_uvf(path, raw, bs, ov, clamp=clamp, compression=comp, level=level,
                              layout=layout, checksum=checksum, big_endian=be,
                              kv_first=kv_first, histograms=hist, components=comps,
                              scratch=tmp)
            table, why = refconv.read_uvf(path, verify=checksum == 2)
            assert table is not None, why
            meta.append(dict(name=name, dims=dims, dtype=dt, components=comps, timesteps=ts,
                             brick_size=bs, overlap=ov, clamp=clamp, compression=comp,
                             level=level, layout=layout, checksum=checksum, big_endian=be,
                             kv_first=kv_first, histograms=hist, reference=table))
    (OUT / "cases.json").write_text(json.dumps(meta, indent=1) + "\n")


if __name__ == "__main__":
    main()
