"""Writes the ExtendedOctree fixtures in tests/golden/eo/ with the reference's
own converter (ExtendedOctreeConverter::Convert, built from the reference
sources into oracle/_ref by tuvok_gb300.build.build_reference).  Run once in a
checkout that has the reference sources; the fixtures are committed, so the
tests need neither the reference nor this script.

Each case: a small seeded volume (saved as .npy, [z, y, x] or [z, y, x, 4])
and the .eo file the converter writes for it, with the settings in
cases.json."""
import ctypes as C
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tuvok_gb300.workloads import numpy_blob_volume  # noqa: E402

OUT = Path(__file__).resolve().parent / "eo"

# Every last brick's core is at least the overlap thick: otherwise the
# converter's scanline read for the brick before it runs past the end of the
# input (GetInputBrick, ExtendedOctreeConverter.cpp:288-373) and, with
# clamp-to-edge, keeps whatever the reused buffer held there.
# name, dims (x, y, z), dtype, components, brick size, overlap, clamp, median,
# compression (0 none, 1 zlib, 2 LZMA, 3 LZ4, 4 bzip2), level, layout (0 scanline,
# 1 Morton, 2 Hilbert, 3 random)
CASES = [
    ("u8_none_scanline", (21, 17, 13), "u8", 1, (8, 8, 8), 1, False, False, 0, 0, 0),
    ("u16_lz4_morton_clamp_median", (20, 23, 11), "u16", 1, (10, 9, 8), 2, True, True, 3, 1, 1),
    ("u8_lz4hc_hilbert", (30, 9, 17), "u8", 1, (12, 6, 12), 1, False, False, 3, 9, 2),
    ("rgba_none_random", (14, 12, 10), "u8", 4, (8, 8, 8), 1, True, False, 0, 0, 3),
    # compression 1 zlib, 2 LZMA, 4 bzip2 (ExtendedOctree.cpp:337-350)
    ("u8_zlib_scanline", (21, 17, 13), "u8", 1, (8, 8, 8), 1, False, False, 1, 6, 0),
    ("u16_zlib9_morton", (26, 20, 15), "u16", 1, (10, 10, 10), 2, True, False, 1, 9, 1),
    # LZMA at levels 8 and 9: the converter compresses with level - 1 and
    # asserts that the properties equal those of the level itself, which holds
    # only where both levels have the same dictionary size
    ("u8_lzma_hilbert", (30, 9, 17), "u8", 1, (12, 6, 12), 1, False, False, 2, 9, 2),
    ("u16_lzma8_scanline_median", (20, 23, 11), "u16", 1, (10, 9, 8), 2, False, True, 2, 8, 0),
    ("u8_bzip2_scanline", (23, 21, 19), "u8", 1, (10, 10, 10), 1, False, False, 4, 9, 0),
    ("u16_bzip2_random", (18, 20, 22), "u16", 1, (9, 9, 9), 1, False, False, 4, 1, 3),
    ("rgba_lzma_morton", (14, 12, 10), "u8", 4, (8, 8, 8), 1, False, False, 2, 9, 1),
]


def volume(dims, dt, comps, seed):
    if comps == 4:
        ch = [numpy_blob_volume(dims, np.uint8, 3, (2, 5), (60, 255), 255, seed + k, 3)
              for k in range(4)]
        return np.stack(ch, axis=-1)
    if dt == "u8":
        return numpy_blob_volume(dims, np.uint8, 4, (2, 6), (60, 255), 255, seed, 3)
    return numpy_blob_volume(dims, np.uint16, 4, (2, 6), (900, 4000), 4095, seed, 20)


def main():
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libtuvok_ref.so"))
    lib.ref_write_eo.restype = C.c_int
    lib.ref_write_eo.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_uint32), C.c_uint32, C.c_int, C.c_int, C.c_int,
                                 C.c_uint32, C.c_int, C.c_char_p, C.c_char_p]
    OUT.mkdir(exist_ok=True)
    meta = []
    with tempfile.TemporaryDirectory() as tmp:
        for i, (name, dims, dt, comps, bs, ov, clamp, median, comp, level, layout) in \
                enumerate(CASES):
            raw = np.ascontiguousarray(volume(dims, dt, comps, 500 + 10 * i))
            np.save(OUT / f"{name}.npy", raw)
            ok = lib.ref_write_eo(raw.ctypes.data_as(C.c_void_p), 0 if dt == "u8" else 1, comps,
                                  (C.c_uint64 * 3)(*dims), (C.c_uint32 * 3)(*bs), ov, int(clamp),
                                  int(median), comp, level, layout,
                                  str(OUT / f"{name}.eo").encode(), tmp.encode())
            assert ok == 1, name
            meta.append(dict(name=name, dims=dims, dtype=dt, components=comps, brick_size=bs,
                             overlap=ov, clamp=clamp, median=median, compression=comp,
                             level=level, layout=layout))
    (OUT / "cases.json").write_text(json.dumps(meta, indent=1) + "\n")


if __name__ == "__main__":
    main()
