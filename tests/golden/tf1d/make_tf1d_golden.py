"""Generates the TransferFunction1D golden vectors from the reference's own
class (IO/TransferFunction1D.cpp, built from the reference sources into
oracle/_ref/libtuvok_ref.so by oracle/ref/Makefile).

Every case stores its inputs and the reference's resulting table and non-zero
limits; tests/test_tf1d.py compares tuvok_gb300's tvk_tf1d_* functions with
them (and with the live reference where it is built).

    python tests/golden/tf1d/make_tf1d_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import refconv  # noqa: E402

OUT = HERE / "tf1d.npz"


def std_cases():
    rng = np.random.default_rng(21)
    out = []
    for n in (1, 2, 7, 256, 1000, 4096):
        centers = (-0.2, 0.0, 0.3, 0.5, 0.77, 1.0, 1.3) if n <= 256 else (0.0, 0.37, 0.77, 1.0)
        grads = (0.0, 0.1, 0.5, 1.0, 1.5) if n <= 256 else (0.1, 0.45, 1.0)
        for center in centers:
            for grad in grads:
                for comp, inv in ((-1, 0), (0, 0), (3, 1), (2, 1)):
                    # the channels not written keep the input: a constant keeps
                    # the fixture small, random inputs on the short tables
                    t = (rng.uniform(-0.5, 1.5, (n, 4)) if n <= 7 else
                         np.full((n, 4), 0.25)).astype(np.float32)
                    out.append((t, center, grad, comp, inv))
    return out


def byte_cases():
    rng = np.random.default_rng(22)
    out = [rng.integers(0, 256, (256, 4)).astype(np.uint8) for _ in range(3)]
    t = rng.integers(40, 200, (300, 4)).astype(np.uint8)
    t[0, 0] = 5  # entry 0's red is below every other channel's values
    out.append(t)
    t = rng.integers(0, 256, (64, 4)).astype(np.uint8)
    t[:, 1] = 77  # a constant channel whose value differs from entry 0's red
    t[0, 0] = 9
    out.append(t)
    t = rng.integers(0, 256, (33, 4)).astype(np.uint8)
    t[:, 2] = t[0, 0]  # a constant channel equal to entry 0's red
    out.append(t)
    return out


def resample_cases():
    rng = np.random.default_rng(23)
    out = []
    for n in (1, 7, 256, 4096):
        for target in (1, 3, 100, 256, 300, 1000, 4096):
            if n * target > 256 * 4096:
                continue
            # entries on a 1/256 grid: exact in float, and a small fixture
            out.append(((rng.integers(0, 257, (n, 4)) / 256.0).astype(np.float32), target))
    return out


def main():
    if not refconv.available():
        raise SystemExit("oracle/_ref/libtuvok_ref.so missing: build it with make -C oracle/ref")
    arrays = {}
    for i, (t, c, g, comp, inv) in enumerate(std_cases()):
        r, lim = refconv.tf1d_std(t, c, g, comp, inv)
        arrays[f"std{i}_in"] = t
        arrays[f"std{i}_args"] = np.array([c, g, comp, inv], dtype=np.float64)
        arrays[f"std{i}_out"] = r
        arrays[f"std{i}_lim"] = np.array(lim, dtype=np.uint64)
    for i, b in enumerate(byte_cases()):
        with np.errstate(all="ignore"):
            r, lim = refconv.tf1d_set(b)
        arrays[f"set{i}_in"] = b
        arrays[f"set{i}_out"] = r
        arrays[f"set{i}_lim"] = np.array(lim, dtype=np.uint64)
    for i, (t, target) in enumerate(resample_cases()):
        r, lim = refconv.tf1d_resample(t, target)
        arrays[f"res{i}_in"] = t
        arrays[f"res{i}_out"] = r
        arrays[f"res{i}_lim"] = np.array(lim, dtype=np.uint64)
        arrays[f"fot{i}_out"] = refconv.tf1d_fill_or_truncate(t, target)
    rng = np.random.default_rng(24)
    for i, rng_ in enumerate((255, 200, 17)):
        t = rng.uniform(-0.5, 1.5, (512, 4)).astype(np.float32)
        arrays[f"bytes{i}_in"] = t
        arrays[f"bytes{i}_range"] = np.array([rng_], dtype=np.int64)
        arrays[f"bytes{i}_out"] = refconv.tf1d_bytes(t, rng_)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(arrays)} arrays)")


if __name__ == "__main__":
    main()
