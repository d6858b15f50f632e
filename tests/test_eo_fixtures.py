"""The ExtendedOctree fixtures (written by the reference's converter, see
tests/golden/make_eo_fixtures.py) read back on the CPU with a restatement of
the format (ExtendedOctree::Open, ExtendedOctree.cpp:67-172; GetBrickData
:313-361; the public LZ4 block format, and Python's zlib, LZMA and bzip2
decoders for the other codecs): every LOD-0 brick equals the oracle's brick of
the saved volume, and the inner voxels tile the volume.  The library's own
decoders (tvk_eo_read_brick, host code) give the same bytes for every brick of
every LOD, and refuse corrupted bricks."""
import bz2
import ctypes as C
import json
import lzma
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

import oracle as O

EO = Path(__file__).resolve().parent / "golden" / "eo"
CASES = json.loads((EO / "cases.json").read_text())


def lz4_block(src, n):
    out = bytearray()
    i = 0
    while True:
        tok = src[i]
        i += 1
        lit = tok >> 4
        if lit == 15:
            while True:
                b = src[i]
                i += 1
                lit += b
                if b != 255:
                    break
        out += src[i:i + lit]
        i += lit
        if len(out) == n:
            return bytes(out)
        off = src[i] | (src[i + 1] << 8)
        i += 2
        ml = tok & 15
        if ml == 15:
            while True:
                b = src[i]
                i += 1
                ml += b
                if b != 255:
                    break
        ml += 4
        assert 0 < off <= len(out)
        for _ in range(ml):
            out.append(out[-off])
        if len(out) == n:
            return bytes(out)


def expand(data, comp, nbytes):
    """A stored brick in its original bytes (CT_NONE 0, CT_ZLIB 1, CT_LZMA 2,
    CT_LZ4 3, CT_BZLIB 4)."""
    if comp == 0:
        assert len(data) == nbytes
        return data
    if comp == 1:
        return zlib.decompress(data)
    if comp == 2:
        # LzmaCompression.cpp: raw LZMA1, lc 3 lp 0 pb 2, no end marker
        d = lzma.LZMADecompressor(lzma.FORMAT_RAW, filters=[
            {"id": lzma.FILTER_LZMA1, "lc": 3, "lp": 0, "pb": 2, "dict_size": 1 << 26}])
        return d.decompress(data, max_length=nbytes)
    if comp == 3:
        return lz4_block(data, nbytes)
    if comp == 4:
        return bz2.decompress(data)
    raise AssertionError(f"compression {comp}")


def parse(buf):
    ctype, comps = struct.unpack_from("<IQ", buf, 0)
    p = 12
    normals = buf[p]
    p += 1
    dims = struct.unpack_from("<3Q", buf, p); p += 24
    aspect = struct.unpack_from("<3d", buf, p); p += 24
    bs = struct.unpack_from("<3Q", buf, p); p += 24
    ov, version = struct.unpack_from("<II", buf, p); p += 8
    size, = struct.unpack_from("<Q", buf, p); p += 8
    if version > 1:
        p += 4
    sizes, counts = O.lod_table(dims, bs, ov)
    n = sum(c[0] * c[1] * c[2] for c in counts)
    toc = []
    for _ in range(n):
        toc.append(struct.unpack_from("<QQIQII", buf, p))
        p += 36
    return dict(ctype=ctype, comps=comps, normals=normals, dims=dims, aspect=aspect, bs=bs,
                ov=ov, version=version, size=size, toc=toc, sizes=sizes, counts=counts)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_eo_fixture_lod0_bricks(case):
    buf = (EO / f"{case['name']}.eo").read_bytes()
    raw = np.load(EO / f"{case['name']}.npy")
    h = parse(buf)
    assert h["version"] >= 1 and h["comps"] == case["components"]
    assert tuple(h["dims"]) == tuple(case["dims"]) and h["ov"] == case["overlap"]
    vb = (1 if case["dtype"] == "u8" else 2) * case["components"]
    dt = np.uint8 if case["dtype"] == "u8" else np.uint16
    lc = h["counts"][0]
    comp_types = set()
    for k in range(lc[0] * lc[1] * lc[2]):
        c = (k % lc[0], (k // lc[0]) % lc[1], k // (lc[0] * lc[1]))
        n = O.brick_size(h["sizes"][0], lc, case["brick_size"], case["overlap"], c)
        off, length, comp, _, _, _ = h["toc"][k]
        data = buf[off:off + length]
        comp_types.add(comp)
        nbytes = n[0] * n[1] * n[2] * vb
        data = expand(data, comp, nbytes)
        assert len(data) == nbytes
        shape = (n[2], n[1], n[0]) + ((4,) if case["components"] == 4 else ())
        brick = np.frombuffer(data, dtype=dt).reshape(shape)
        ref = O.lod0_brick(raw, case["brick_size"], case["overlap"], case["clamp"], c)
        np.testing.assert_array_equal(brick, ref, err_msg=f"{case['name']} brick {c}")
    if case["compression"]:
        assert case["compression"] in comp_types, "the fixture should hold compressed bricks"


@pytest.mark.parametrize("case", [c for c in CASES if not (c["clamp"] and c["overlap"] >= 2)],
                         ids=lambda c: c["name"])
def test_eo_fixture_every_lod_equals_oracle_octree(case):
    """Every brick of every LOD the converter wrote equals the oracle's octree
    (ComputeHierarchy + FillOverlap restated; colour volumes per channel).
    Clamp-to-edge with an overlap of 2 or more is left out: there the
    converter's coarser ghost corners hold stale buffer data."""
    buf = (EO / f"{case['name']}.eo").read_bytes()
    raw = np.load(EO / f"{case['name']}.npy")
    h = parse(buf)
    bricks = O.build_octree(raw, case["brick_size"], case["overlap"], clamp=case["clamp"],
                            median=case["median"])
    assert len(bricks) == len(h["toc"])
    for k, ref in enumerate(bricks):
        off, length, comp, _, _, _ = h["toc"][k]
        data = expand(buf[off:off + length], comp, ref.nbytes)
        np.testing.assert_array_equal(np.frombuffer(data, ref.dtype).reshape(ref.shape), ref,
                                      err_msg=f"{case['name']} brick {k}")


def lib_brick(path, index):
    from tuvok_gb300 import _native as N
    n = C.c_size_t()
    N.check(N.lib().tvk_eo_read_brick(str(path).encode(), 0, 5, index, None, 0, C.byref(n)))
    out = (C.c_uint8 * n.value)()
    N.check(N.lib().tvk_eo_read_brick(str(path).encode(), 0, 5, index, out, n.value,
                                      C.byref(n)))
    return bytes(out)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_library_decoders_read_every_brick(case):
    """tvk_eo_read_brick (the library's zlib / LZMA / LZ4 / bzip2 decoders,
    host code) against the restatement above, every brick of every LOD."""
    path = EO / f"{case['name']}.eo"
    buf = path.read_bytes()
    h = parse(buf)
    vb = (1 if case["dtype"] == "u8" else 2) * case["components"]
    k = 0
    for lod, (ls, lc) in enumerate(zip(h["sizes"], h["counts"])):
        for i in range(lc[0] * lc[1] * lc[2]):
            c = (i % lc[0], (i // lc[0]) % lc[1], i // (lc[0] * lc[1]))
            n = O.brick_size(ls, lc, case["brick_size"], case["overlap"], c)
            off, length, comp, _, _, _ = h["toc"][k]
            want = expand(buf[off:off + length], comp, n[0] * n[1] * n[2] * vb)
            assert lib_brick(path, k) == want, f"{case['name']} brick {k} (LOD {lod})"
            k += 1


@pytest.mark.parametrize("comp", [1, 2, 4], ids=["zlib", "lzma", "bzip2"])
def test_library_decoders_refuse_corrupt_bricks(tmp_path, comp):
    """Flipped bytes inside a compressed brick are refused with a message
    (checksums for zlib and bzip2, range / distance checks for LZMA), never a
    crash or an out-of-range write."""
    from tuvok_gb300 import TvkError
    case = next(c for c in CASES if c["compression"] == comp)
    buf = bytearray((EO / f"{case['name']}.eo").read_bytes())
    h = parse(bytes(buf))
    k = next(i for i, t in enumerate(h["toc"]) if t[2] == comp and t[1] > 64)
    off, length = h["toc"][k][0], h["toc"][k][1]
    rng = np.random.default_rng(comp)
    refused = 0
    for trial in range(12):
        bad = bytearray(buf)
        for p in rng.integers(off + 2, off + length, 6):
            bad[int(p)] ^= 0xA5
        path = tmp_path / f"bad{trial}.eo"
        path.write_bytes(bytes(bad))
        try:
            got = lib_brick(path, k)
        except TvkError as e:
            assert "corrupt" in str(e) or "ExtendedOctree" in str(e)
            refused += 1
            continue
        # LZMA has no checksum: a changed stream may decode to other bytes
        assert comp == 2 and len(got) > 0
    assert refused >= (6 if comp == 2 else 12)
