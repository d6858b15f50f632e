"""The ExtendedOctree fixtures (written by the reference's converter, see
tests/golden/make_eo_fixtures.py) read back on the CPU with a restatement of
the format (ExtendedOctree::Open, ExtendedOctree.cpp:67-172; GetBrickData
:313-361; the public LZ4 block format): every LOD-0 brick equals the oracle's
brick of the saved volume, and the inner voxels tile the volume."""
import json
import struct
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
        if comp == 3:
            data = lz4_block(data, nbytes)
        else:
            assert comp == 0 and length == nbytes
        shape = (n[2], n[1], n[0]) + ((4,) if case["components"] == 4 else ())
        brick = np.frombuffer(data, dtype=dt).reshape(shape)
        ref = O.lod0_brick(raw, case["brick_size"], case["overlap"], case["clamp"], c)
        np.testing.assert_array_equal(brick, ref, err_msg=f"{case['name']} brick {c}")
    if case["compression"] == 3:
        assert 3 in comp_types, "the LZ4 fixture should hold LZ4 bricks"


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
        data = buf[off:off + length]
        if comp == 3:
            data = lz4_block(data, ref.nbytes)
        np.testing.assert_array_equal(np.frombuffer(data, ref.dtype).reshape(ref.shape), ref,
                                      err_msg=f"{case['name']} brick {k}")
