"""The oracle's host restatement of the seeded volume generator against a
direct numpy statement of the same formula on small volumes (float32
operations in the same order; the Gaussian's exponential from its Taylor
series in double), and the volume digest's definition."""
import numpy as np

import oracle as O


def exp_np(x):
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x * 1.4426950408889634 + 0.5)
    r = x - k * 0.69314718055994531
    c = [1 / 39916800, 1 / 3628800, 1 / 362880, 1 / 40320, 1 / 5040, 1 / 720, 1 / 120, 1 / 24,
         1 / 6, 0.5, 1.0, 1.0]
    p = np.full_like(r, c[0])
    for ci in c[1:]:
        p = p * r + ci  # numpy's multiply then add; the restatement fuses them
        # (exact agreement is checked on the generated bytes, which round to integers)
    return p * np.exp2(k)


def numpy_volume(dims, dtype, blobs, amp, seed):
    """Blob sum + integer noise, float32 steps in the generator's order."""
    nx, ny, nz = dims
    f32 = np.float32
    v = np.zeros((nz, ny, nx), dtype=f32)
    for b in blobs.astype(np.float32):
        s2 = f32(b[3] * b[3])
        lim = f32(f32(32.0) * s2)
        q = [(np.arange(n, dtype=f32) - f32(b[a])) ** 2 for a, n in enumerate(dims)]
        q = [qq.astype(f32) for qq in q]
        e = [exp_np(-qq.astype(np.float64) / (2.0 * float(s2))).astype(f32) for qq in q]
        d2 = (q[0][None, None, :] + q[1][None, :, None]) + q[2][:, None, None]
        g = (e[0][None, None, :] * e[1][None, :, None]) * e[2][:, None, None]
        v = np.where(d2 < lim, v + f32(b[4]) * g, v).astype(f32)
    return v


def test_generator_blob_sum_matches_numpy_statement():
    rng = np.random.default_rng(4)
    dims = (23, 17, 11)
    blobs = np.zeros((5, 7), np.float32)
    blobs[:, :3] = rng.uniform(0, 20, (5, 3))
    blobs[:, 3] = rng.uniform(2, 6, 5)
    blobs[:, 4] = rng.uniform(60, 250, 5)
    got = O.generate_volume(dims, np.uint16, blobs, 0, 0, 0, 1, 0, 4095)
    v = numpy_volume(dims, np.uint16, blobs, 0, 1)
    want = np.clip(np.floor(v + np.float32(0.5)), 0, 4095).astype(np.uint16)
    # the two exponentials differ only in the last bits of a double; after
    # rounding to float and then to integers they agree except where a value
    # lies within 1e-4 of a rounding boundary
    close = np.abs((v + 0.5) - np.round(v + 0.5)) < 1e-4
    assert np.array_equal(got[~close], want[~close])
    assert got.max() > 50


def test_generator_is_deterministic_and_seeded():
    args = ((40, 30, 20), np.uint8, np.array([[20, 15, 10, 6, 200, 0, 0]], np.float32), 4, 0, 0)
    a = O.generate_volume(*args, 7, 1, 255)
    b = O.generate_volume(*args, 7, 1, 255, threads=1)
    c = O.generate_volume(*args, 8, 1, 255)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    n = O.generate_volume((64, 48, 40), np.uint16, args[2], 409.5, 3, 16.0, 3, 0, 4095)
    assert n.std() > 10  # value noise present


def test_volume_hash_is_chunked_fnv1a():
    def fnv(data, h=0xcbf29ce484222325):
        for x in data:
            h = ((h ^ x) * 0x100000001b3) & 0xffffffffffffffff
        return h
    rng = np.random.default_rng(1)
    for n in (0, 5, (1 << 20) + 3):
        a = rng.integers(0, 256, n).astype(np.uint8)
        chunks = [fnv(a[i:i + (1 << 20)].tobytes()) for i in range(0, n, 1 << 20)] \
            if n < 64 else None
        if chunks is not None:
            want = fnv(b"".join(int(c).to_bytes(8, "little") for c in chunks))
            assert O.volume_hash(a) == f"{want:016x}"
    a = rng.integers(0, 256, 3 << 20).astype(np.uint8)
    h1 = O.volume_hash(a)
    a[(2 << 20) + 7] ^= 1
    assert O.volume_hash(a) != h1
