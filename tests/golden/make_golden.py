"""Generates the bricking golden fixtures from the reference's own converter.

Runs Tuvok's ExtendedOctreeConverter::Convert (built from the reference sources
into oracle/_ref/libtuvok_ref.so by oracle/ref/Makefile) on small seeded
volumes and stores, per case, every brick of every LOD with its size and the
converter's min/max statistics.  The GPU machine has no reference sources, so the
tests there compare against these files.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import refconv  # noqa: E402

CASES = [
    # name, dims (x, y, z), dtype, brick size, overlap, clamp, value max, seed
    ("ramp8x8x1_u16", (8, 8, 1), np.uint16, 16, 2, False, None, 0),
    ("rand37x29x23_u8", (37, 29, 23), np.uint8, 16, 1, False, 255, 1),
    ("rand37x29x23_u8_clamp", (37, 29, 23), np.uint8, 16, 1, True, 255, 2),
    ("rand40x33x20_u16", (40, 33, 20), np.uint16, 12, 2, False, 4095, 3),
    ("rand40x33x20_u16_clamp", (40, 33, 20), np.uint16, 12, 2, True, 4095, 4),
    ("wrap25x14x13_u8", (25, 14, 13), np.uint8, 16, 2, False, 255, 5),
    ("cube64_u8", (64, 64, 64), np.uint8, 34, 1, False, 255, 6),
]
# the same converter with the 7-value median filter instead of the mean
MEDIAN_CASES = [
    ("median37x29x23_u8", (37, 29, 23), np.uint8, 16, 1, False, 255, 7),
    ("median40x33x20_u16", (40, 33, 20), np.uint16, 12, 2, False, 4095, 8),
]


def make_input(dims, dtype, vmax, seed):
    x, y, z = dims
    if vmax is None:  # IO/test/rebricking.h:12-21 ramp
        return np.arange(x * y * z, dtype=dtype).reshape(z, y, x)
    rng = np.random.default_rng(seed)
    return rng.integers(0, vmax + 1, size=(z, y, x)).astype(dtype)


def main():
    if not refconv.available():
        raise SystemExit("oracle/_ref/libtuvok_ref.so missing: build it with make -C oracle/ref")
    cases = [c + (False,) for c in CASES] + [c + (True,) for c in MEDIAN_CASES]
    for name, dims, dtype, bs, ov, clamp, vmax, seed, median in cases:
        raw = make_input(dims, dtype, vmax, seed)
        bricks = refconv.convert(raw, (bs, bs, bs), ov, clamp=clamp, median=median)
        arrays = {"raw": raw,
                  "meta": np.array([dims[0], dims[1], dims[2], bs, ov, int(clamp)], dtype=np.int64),
                  "median": np.array([int(median)], dtype=np.int64),
                  "coords": np.array([b["coords"] for b in bricks], dtype=np.int64),
                  "sizes": np.array([b["size"] for b in bricks], dtype=np.int64),
                  "minmax": np.array([(b["min"], b["max"]) for b in bricks], dtype=np.float64)}
        for i, b in enumerate(bricks):
            arrays[f"brick{i}"] = b["data"]
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        print(name, len(bricks), "bricks")


if __name__ == "__main__":
    main()
