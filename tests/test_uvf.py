"""UVF container reading (tvk_uvf_read_blocks, host code) against the
reference's own parser.

* The committed fixtures (written by the reference's UVF writer, see
  tests/golden/make_uvf_fixtures.py) hold, in cases.json, the block table that
  UVF::Open reported for them (UVF.cpp:74-95, 269-291): the library's walk
  gives the same offsets, semantics, compression and chain links, the same
  octree offsets for the TOC blocks, and checks the same MD5 checksums.
* The ExtendedOctree at each TOC block's payload holds that timestep's volume:
  its LOD-0 bricks, decoded on the host, equal the oracle's bricks of the saved
  volume.
* Damaged files (checksum, magic, truncation, broken chain links) are refused
  with a message, never read past their end.
* Where the reference's sources were built into oracle/_ref, files written
  there and then (2D histograms, three timesteps, either big-endian flag,
  metadata first or last) are walked by both parsers and compared.  The flag
  changes no byte: the reference's swap is a no-op, and files flagged
  big-endian hold little-endian values.
"""
import ctypes as C
import json
import struct
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import refconv
from test_eo_fixtures import expand, parse
from tuvok_gb300 import TvkError, read_uvf_blocks
from tuvok_gb300 import _native as N

UVF = Path(__file__).resolve().parent / "golden" / "uvf"
CASES = json.loads((UVF / "cases.json").read_text())
TOC = N.TVK_UVF_BS_TOC_BLOCK


def assert_same_table(path, head, blocks, ref):
    assert head["file_version"] == ref["version"]
    assert head["big_endian"] == ref["big_endian"]
    assert head["file_bytes"] == Path(path).stat().st_size
    assert head["block_count"] == len(ref["blocks"]) == len(blocks)
    for i, (b, r) in enumerate(zip(blocks, ref["blocks"])):
        got = (b["offset"], b["semantics"], b["compression"], b["offset_to_next"],
               b["header_bytes"] - 32)
        assert got == tuple(r[:5]), f"block {i}"
        if r[1] == TOC:
            assert b["offset"] + b["header_bytes"] == r[5], f"octree offset of block {i}"
    assert blocks[-1]["offset_to_next"] == 0
    accepted = [r for r in ref["blocks"] if r[1] == TOC and r[6] in (1, 4)]
    assert head["timestep_count"] == len(accepted)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_uvf_fixture_block_table_equals_reference_parser(case):
    path = UVF / f"{case['name']}.uvf"
    verify = case["checksum"] == 2
    head, blocks = read_uvf_blocks(path, verify=verify)
    assert_same_table(path, head, blocks, case["reference"])
    assert head["timestep_count"] == case["timesteps"]
    assert head["checksum_semantics"] == case["checksum"]
    assert head["checksum_verified"] == int(verify)
    assert head["big_endian"] == int(case["big_endian"])
    sem = [b["semantics"] for b in blocks]
    assert (sem[0] == N.TVK_UVF_BS_KEY_VALUE_PAIRS) == case["kv_first"]
    assert sem.count(N.TVK_UVF_BS_MAXMIN_VALUES) == case["timesteps"]
    assert sem.count(N.TVK_UVF_BS_1D_HISTOGRAM) == case["timesteps"] * case["histograms"]
    assert all(b["id"] for b in blocks)


def lib_brick(path, offset, index):
    n = C.c_size_t()
    N.check(N.lib().tvk_eo_read_brick(str(path).encode(), offset, 5, index, None, 0,
                                      C.byref(n)))
    out = (C.c_uint8 * n.value)()
    N.check(N.lib().tvk_eo_read_brick(str(path).encode(), offset, 5, index, out, n.value,
                                      C.byref(n)))
    return bytes(out)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_uvf_fixture_toc_blocks_hold_each_timestep(case):
    """Timestep t's TOC block holds the octree of volume t: every LOD-0 brick,
    decoded by the restatement and by tvk_eo_read_brick at the block's payload,
    equals the oracle's brick of the saved volume."""
    path = UVF / f"{case['name']}.uvf"
    buf = path.read_bytes()
    raw = np.load(UVF / f"{case['name']}.npy")
    _, blocks = read_uvf_blocks(path)
    tocs = [b for b in blocks if b["semantics"] == TOC]
    assert len(tocs) == case["timesteps"] == raw.shape[0]
    vb = (1 if case["dtype"] == "u8" else 2) * case["components"]
    dt = np.uint8 if case["dtype"] == "u8" else np.uint16
    for t, b in enumerate(tocs):
        base = b["offset"] + b["header_bytes"]
        h = parse(buf[base:])
        assert tuple(h["dims"]) == tuple(case["dims"]) and h["comps"] == case["components"]
        lc = h["counts"][0]
        for k in range(lc[0] * lc[1] * lc[2]):
            c = (k % lc[0], (k // lc[0]) % lc[1], k // (lc[0] * lc[1]))
            n = O.brick_size(h["sizes"][0], lc, case["brick_size"], case["overlap"], c)
            off, length, comp, _, _, _ = h["toc"][k]
            nbytes = n[0] * n[1] * n[2] * vb
            data = expand(buf[base + off:base + off + length], comp, nbytes)
            assert lib_brick(path, base, k) == data, f"t {t} brick {k}"
            shape = (n[2], n[1], n[0]) + ((4,) if case["components"] == 4 else ())
            ref = O.lod0_brick(raw[t], case["brick_size"], case["overlap"], case["clamp"], c)
            np.testing.assert_array_equal(np.frombuffer(data, dt).reshape(shape), ref,
                                          err_msg=f"{case['name']} t {t} brick {c}")


def status_of(path, verify=False):
    try:
        read_uvf_blocks(path, verify=verify)
    except TvkError as e:
        return e.status, str(e)
    return N.TVK_OK, ""


def test_uvf_checksum_mismatch_is_refused(tmp_path):
    """One flipped payload byte (the file's last, inside a metadata string):
    the MD5 no longer matches (refused with verification, the reference's
    parser agrees where it is built), while the block walk alone still reads
    the file."""
    case = next(c for c in CASES if c["checksum"] == 2)
    buf = bytearray((UVF / f"{case['name']}.uvf").read_bytes())
    buf[-1] ^= 0x5A
    bad = tmp_path / "bad.uvf"
    bad.write_bytes(bytes(buf))
    st, msg = status_of(bad, verify=True)
    assert st == 1 and "checksum mismatch" in msg
    assert status_of(bad, verify=False)[0] == N.TVK_OK
    if refconv.available():
        table, why = refconv.read_uvf(bad, verify=True)
        assert table is None and "checksum" in why
        assert refconv.read_uvf(bad, verify=False)[0] is not None


def test_uvf_crc32_checksums_are_not_verified():
    case = next(c for c in CASES if c["checksum"] == 1)
    path = UVF / f"{case['name']}.uvf"
    st, msg = status_of(path, verify=True)
    assert st == 4 and "CRC32" in msg
    head, _ = read_uvf_blocks(path)
    assert head["checksum_semantics"] == N.TVK_UVF_CS_CRC32 and head["checksum_bytes"] == 4


def test_uvf_damaged_headers_are_refused(tmp_path):
    """Wrong magic, chain links past the end or shorter than a header, an id
    longer than the file, and truncation anywhere before the last block's
    header: all TVK_ERR_INVALID_ARG."""
    case = next(c for c in CASES if c["timesteps"] == 2)
    src = (UVF / f"{case['name']}.uvf").read_bytes()
    head, blocks = read_uvf_blocks(UVF / f"{case['name']}.uvf")

    def refused(buf, name):
        p = tmp_path / name
        p.write_bytes(bytes(buf))
        st, msg = status_of(p)
        assert st == 1, (name, st, msg)
        return msg

    bad = bytearray(src)
    bad[3] = ord("X")
    assert "magic" in refused(bad, "magic.uvf")
    b1 = blocks[1]
    for name, value in (("far", len(src)), ("short", 5), ("huge", 1 << 62)):
        bad = bytearray(src)
        at = b1["offset"] + b1["header_bytes"] - 8
        struct.pack_into("<Q", bad, at, value)
        refused(bad, f"next_{name}.uvf")
    bad = bytearray(src)
    struct.pack_into("<Q", bad, b1["offset"], 1 << 40)
    assert "id" in refused(bad, "idlen.uvf")
    cuts = [0, 7, 20, 40, head["data_offset"], head["data_offset"] + 10,
            blocks[1]["offset"] + 4, blocks[-1]["offset"] + 20]
    for cut in cuts:
        refused(src[:cut], f"cut{cut}.uvf")


def test_uvf_truncation_never_reads_past_the_end(tmp_path):
    """Every cut of a small file returns TVK_OK or TVK_ERR_INVALID_ARG; the
    walk never reads past the end of the file."""
    case = next(c for c in CASES if c["checksum"] == 1)
    src = (UVF / f"{case['name']}.uvf").read_bytes()
    rng = np.random.default_rng(7)
    for cut in sorted(set(int(x) for x in rng.integers(0, len(src), 60))):
        p = tmp_path / f"cut{cut}.uvf"
        p.write_bytes(src[:cut])
        assert status_of(p)[0] in (N.TVK_OK, 1)


def minimal_uvf(blocks, big_endian=False):
    """A hand-assembled UVF file: the global header (no checksum) and blocks of
    (semantics, payload bytes) chained in order.  Values are little-endian
    whatever the flag, as the reference writes them (its byte swap is a
    no-op)."""
    e = "<"
    out = bytearray(b"UVF-DATA") + bytes([1 if big_endian else 0])
    out += struct.pack(e + "QQQQ", 5, 0, 0, 0)
    for i, (sem, payload) in enumerate(blocks):
        ident = f"block {i}".encode()
        size = 32 + len(ident) + len(payload)
        nxt = 0 if i == len(blocks) - 1 else size
        out += struct.pack(e + "Q", len(ident)) + ident + struct.pack(e + "QQQ", sem, 0, nxt)
        out += payload
    return bytes(out)


@pytest.mark.parametrize("big_endian", [False, True])
def test_uvf_hand_assembled_chain(tmp_path, big_endian):
    """A chain built by hand, with either big-endian flag, is walked block by
    block; TOC blocks of 2-component volumes are not timesteps
    (VerifyTOCBlock)."""
    eo2 = struct.pack("<IQ", 0, 2) + bytes(20)
    eo1 = struct.pack("<IQ", 1, 1) + bytes(20)
    p = tmp_path / "hand.uvf"
    p.write_bytes(minimal_uvf([(4, b"kv"), (TOC, eo2), (TOC, eo1), (7, bytes(16))], big_endian))
    head, blocks = read_uvf_blocks(p)
    assert head["big_endian"] == int(big_endian) and head["data_offset"] == 41
    assert [b["semantics"] for b in blocks] == [4, TOC, TOC, 7]
    assert [b["id"] for b in blocks] == [f"block {i}" for i in range(4)]
    assert head["timestep_count"] == 1
    off = 41
    for b in blocks:
        assert b["offset"] == off
        off += b["offset_to_next"]


def open_status(path, timestep=0):
    h = C.c_void_p()
    st = N.lib().tvk_volume_open_uvf(str(path).encode(), timestep, 0, C.byref(h))
    assert not h.value
    return st, N.lib().tvk_last_error().decode()


def test_uvf_open_refusals_before_any_device_work(tmp_path):
    """tvk_volume_open_uvf refuses, before touching the GPU: a timestep past
    the last TOC block, a file of RasterDataBlock volumes (UVF without TOC
    blocks), and a file with no volume at all."""
    case = next(c for c in CASES if c["timesteps"] == 2)
    st, msg = open_status(UVF / f"{case['name']}.uvf", timestep=2)
    assert st == 1 and "timestep" in msg
    p = tmp_path / "raster.uvf"
    p.write_bytes(minimal_uvf([(1, bytes(64))]))
    st, msg = open_status(p)
    assert st == 4 and "RasterDataBlock" in msg
    p = tmp_path / "kv.uvf"
    p.write_bytes(minimal_uvf([(4, b"x")]))
    st, msg = open_status(p)
    assert st == 1 and "TOC" in msg


LIVE = [
    # dtype, components, timesteps, brick, overlap, clamp, compression, level, layout,
    # checksum, big-endian, metadata first, histograms
    ("u8", 1, 3, (8, 8, 8), 1, False, 0, 0, 0, 2, False, False, 2),
    ("u16", 1, 2, (10, 9, 8), 2, True, 3, 1, 1, 2, True, True, 2),
    ("u8", 4, 2, (8, 8, 8), 1, False, 1, 4, 2, 0, True, False, 0),
    ("u16", 1, 1, (16, 16, 16), 1, False, 4, 9, 3, 2, False, True, 1),
]


@pytest.mark.skipif(not refconv.available(), reason="reference sources not built (oracle/_ref)")
@pytest.mark.parametrize("cfg", LIVE, ids=[f"live{i}" for i in range(len(LIVE))])
def test_uvf_walk_equals_reference_parser_live(tmp_path, cfg):
    dt, comps, ts, bs, ov, clamp, comp, level, layout, checksum, be, kv_first, hist = cfg
    rng = np.random.default_rng(len(tmp_path.name))
    dims = (19, 15, 12)
    shape = (ts, dims[2], dims[1], dims[0]) + ((4,) if comps == 4 else ())
    top = 255 if dt == "u8" else 4095
    raw = rng.integers(0, top + 1, size=shape).astype(np.uint8 if dt == "u8" else np.uint16)
    path = tmp_path / "live.uvf"
    refconv.write_uvf(path, raw, bs, ov, clamp=clamp, compression=comp, level=level,
                      layout=layout, checksum=checksum, big_endian=be, kv_first=kv_first,
                      histograms=hist, components=comps, scratch=str(tmp_path))
    verify = checksum == 2
    table, why = refconv.read_uvf(path, verify=verify)
    assert table is not None, why
    head, blocks = read_uvf_blocks(path, verify=verify)
    assert_same_table(path, head, blocks, table)
    assert head["timestep_count"] == ts and head["checksum_verified"] == int(verify)
    if hist == 2 and comps == 1:
        assert sum(b["semantics"] == N.TVK_UVF_BS_2D_HISTOGRAM for b in blocks) == ts


def md5_uvf(payload_len):
    """A hand-assembled UVF file with an MD5 checksum (computed with hashlib)
    over everything after the checksum, and one metadata block whose payload
    makes the checksummed range payload_len + 32 + id bytes long."""
    import hashlib
    ident = b"md5 case"
    block = struct.pack("<Q", len(ident)) + ident + struct.pack("<QQQ", 4, 0, 0) + bytes(
        (i * 7) & 255 for i in range(payload_len))
    tail = struct.pack("<Q", 0) + block  # offset to the first block, then the block
    head = b"UVF-DATA" + bytes([0]) + struct.pack("<QQQ", 5, N.TVK_UVF_CS_MD5, 16)
    return head + hashlib.md5(tail).digest() + tail


@pytest.mark.parametrize("payload_len", [0, 7, 8, 15, 16, 23, 24, 100, 5_000_000],
                         ids=lambda n: f"payload{n}")
def test_uvf_md5_matches_hashlib(tmp_path, payload_len):
    """The library's MD5 (RFC 1321) against Python's over lengths around the
    64-byte block and 56-byte padding boundaries, and across its 4 MiB read
    chunks; one flipped byte fails the check."""
    buf = md5_uvf(payload_len)
    p = tmp_path / "md5.uvf"
    p.write_bytes(buf)
    head, blocks = read_uvf_blocks(p, verify=True)
    assert head["checksum_verified"] == 1 and len(blocks) == 1
    bad = bytearray(buf)
    bad[-1 if payload_len else 60] ^= 1
    p.write_bytes(bytes(bad))
    st, msg = status_of(p, verify=True)
    assert st == 1 and "checksum" in msg


def test_uvf_cpp_host_lists_the_same_blocks(tmp_path):
    """A C++ host over include/tvk_renderer.hpp (tests/cpp/uvf_list.cpp)
    lists the same blocks as the Python binding, and reports a damaged
    checksum as an error."""
    import re
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = Path(__file__).resolve().parent.parent
    lib_dir = Path(N.LIB_PATH).resolve().parent
    exe = tmp_path / "uvf_list"
    subprocess.run([gxx, "-std=c++17", "-O2", f"-I{root / 'include'}",
                    "-I/usr/local/cuda/include", str(root / "tests" / "cpp" / "uvf_list.cpp"),
                    "-o", str(exe), f"-L{lib_dir}", "-ltvk", f"-Wl,-rpath,{lib_dir}",
                    "-L/usr/local/cuda/lib64", "-Wl,-rpath,/usr/local/cuda/lib64"], check=True)
    case = next(c for c in CASES if c["checksum"] == 2)
    path = UVF / f"{case['name']}.uvf"
    out = subprocess.run([str(exe), str(path), "verify"], check=True, capture_output=True,
                         text=True).stdout
    head, blocks = read_uvf_blocks(path, verify=True)
    first = dict(re.findall(r"(\w+)=(\d+)", out.splitlines()[0]))
    assert int(first["blocks"]) == head["block_count"] and int(first["verified"]) == 1
    assert int(first["timesteps"]) == head["timestep_count"]
    rows = [dict(re.findall(r"(\w+)=(\d+)", line)) for line in out.splitlines()[1:]]
    assert [(int(r["offset"]), int(r["next"]), int(r["semantics"])) for r in rows] == \
        [(b["offset"], b["offset_to_next"], b["semantics"]) for b in blocks]
    bad = bytearray(path.read_bytes())
    bad[-1] ^= 0x5A
    p = tmp_path / "bad.uvf"
    p.write_bytes(bytes(bad))
    r = subprocess.run([str(exe), str(p), "verify"], capture_output=True, text=True)
    assert r.returncode == 1 and "checksum" in r.stderr


def test_uvf_offset_to_first_block_is_honoured(tmp_path):
    """GlobalHeader::GetDataPos adds ulOffsetToFirstDataBlock (GlobalHeader.cpp:
    33-36, 59-61): bytes between the header and the first block are skipped."""
    body = minimal_uvf([(4, b"kv"), (7, bytes(16))])
    pad = 24
    head = bytearray(body[:41])
    struct.pack_into("<Q", head, 33, pad)  # no checksum: the offset follows the length
    p = tmp_path / "pad.uvf"
    p.write_bytes(bytes(head) + bytes(pad) + body[41:])
    info, blocks = read_uvf_blocks(p)
    assert info["data_offset"] == 41 + pad
    assert [b["offset"] for b in blocks] == [41 + pad, 41 + pad + blocks[0]["offset_to_next"]]
    assert [b["semantics"] for b in blocks] == [4, 7]
