"""Binding of oracle/_ref/libtuvok_ref.so: the reference's own
ExtendedOctreeConverter and UVF histogram blocks, built from the reference
sources by oracle/ref/Makefile.

Present only where the reference sources were available at build time; tests
that need it skip otherwise.
"""
import ctypes as C
from pathlib import Path

import numpy as np

PATH = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "libtuvok_ref.so"
_lib = None


def available():
    return PATH.exists()


def _load():
    global _lib
    if _lib is None:
        L = C.CDLL(str(PATH))
        L.ref_convert.restype = C.c_void_p
        L.ref_convert.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_uint32), C.c_uint32, C.c_int, C.c_int, C.c_char_p]
        L.ref_brick_count.argtypes = [C.c_void_p]
        L.ref_brick_count.restype = C.c_uint64
        L.ref_lod_count.argtypes = [C.c_void_p]
        L.ref_lod_count.restype = C.c_uint64
        L.ref_brick_info.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint64), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
        L.ref_brick_info.restype = None
        L.ref_brick_data.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        L.ref_brick_data.restype = None
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_free.restype = None
        L.ref_histograms.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint32), C.c_uint32, C.c_int, C.c_char_p,
                                     C.c_uint64, C.POINTER(C.c_uint64), C.c_size_t,
                                     C.POINTER(C.c_size_t),
                                     C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_size_t),
                                     C.POINTER(C.c_float)]
        L.ref_histograms.restype = C.c_int
        _lib = L
    return _lib


def convert(raw, brick_size, overlap, clamp=False, median=False, scratch="/tmp"):
    """Runs the reference converter on raw ([z, y, x]); returns a list of dicts
    {coords: (x, y, z, lod), size: (x, y, z), min, max, data: [z, y, x]}."""
    L = _load()
    raw = np.ascontiguousarray(raw)
    dims = (C.c_uint64 * 3)(raw.shape[2], raw.shape[1], raw.shape[0])
    h = L.ref_convert(raw.ctypes.data_as(C.c_void_p), 0 if raw.dtype == np.uint8 else 1, dims,
                      (C.c_uint32 * 3)(*brick_size), overlap, int(clamp), int(median),
                      scratch.encode())
    if not h:
        raise RuntimeError("reference conversion failed")
    out = []
    try:
        for i in range(L.ref_brick_count(h)):
            c = (C.c_uint64 * 4)()
            s = (C.c_uint64 * 3)()
            mn, mx = C.c_double(), C.c_double()
            L.ref_brick_info(h, i, c, s, C.byref(mn), C.byref(mx))
            data = np.zeros((s[2], s[1], s[0]), dtype=raw.dtype)
            L.ref_brick_data(h, i, data.ctypes.data_as(C.c_void_p))
            out.append({"coords": tuple(c), "size": tuple(s), "min": mn.value, "max": mx.value,
                        "data": data})
    finally:
        L.ref_free(h)
    return out


def histograms(raw, brick_size, overlap, clamp=False, value_bins=0, scratch="/tmp"):
    """The reference's Histogram1DDataBlock and Histogram2DDataBlock of raw
    ([z, y, x]) as RAWConverter computes them: (hist1d, hist2d [bins, 256],
    max gradient magnitude as float).  value_bins != 0 overrides the 2D
    histogram's value-bin count (default: the 1D histogram's length)."""
    L = _load()
    raw = np.ascontiguousarray(raw)
    dims = (C.c_uint64 * 3)(raw.shape[2], raw.shape[1], raw.shape[0])
    cap1 = 1 << (8 * raw.dtype.itemsize)
    h1 = np.zeros(cap1, dtype=np.uint64)
    h2 = np.zeros(max(cap1, value_bins) * 256, dtype=np.uint64)
    n1, nv = C.c_size_t(), C.c_size_t()
    g = C.c_float()
    rc = L.ref_histograms(raw.ctypes.data_as(C.c_void_p), 0 if raw.dtype == np.uint8 else 1,
                          dims, (C.c_uint32 * 3)(*brick_size), overlap, int(clamp),
                          scratch.encode(), value_bins,
                          h1.ctypes.data_as(C.POINTER(C.c_uint64)), cap1,
                          C.byref(n1), h2.ctypes.data_as(C.POINTER(C.c_uint64)), h2.size,
                          C.byref(nv), C.byref(g))
    if rc != 0:
        raise RuntimeError(f"reference histograms failed ({rc})")
    return h1[:n1.value], h2[:nv.value * 256].reshape(nv.value, 256), g.value


# ---- TransferFunction1D (oracle/ref/ref_tf1d.cpp over IO/TransferFunction1D.cpp)

def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def tf1d_std(table, center, inv_gradient, component=-1, inverted=False):
    """SetStdFunction on a copy of table (n x 4); component -1 = the
    2-argument overload.  Returns (table, (lo, hi) non-zero limits)."""
    L = _load()
    t = np.ascontiguousarray(table, dtype=np.float32)
    out = np.zeros_like(t)
    lim = (C.c_uint64 * 2)()
    L.ref_tf1d_std.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.c_float, C.c_float, C.c_int,
                               C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_uint64)]
    L.ref_tf1d_std(_f32p(t), t.shape[0], center, inv_gradient, component, int(inverted),
                   _f32p(out), lim)
    return out, (lim[0], lim[1])


def tf1d_set(rgba_bytes):
    L = _load()
    b = np.ascontiguousarray(rgba_bytes, dtype=np.uint8).reshape(-1)
    out = np.zeros((b.size // 4, 4), dtype=np.float32)
    lim = (C.c_uint64 * 2)()
    L.ref_tf1d_set.argtypes = [C.POINTER(C.c_uint8), C.c_uint64, C.POINTER(C.c_float),
                               C.POINTER(C.c_uint64)]
    L.ref_tf1d_set(b.ctypes.data_as(C.POINTER(C.c_uint8)), b.size // 4, _f32p(out), lim)
    return out, (lim[0], lim[1])


def tf1d_resample(table, target):
    L = _load()
    t = np.ascontiguousarray(table, dtype=np.float32)
    out = np.zeros((target, 4), dtype=np.float32)
    lim = (C.c_uint64 * 2)()
    L.ref_tf1d_resample.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.c_uint64,
                                    C.POINTER(C.c_float), C.POINTER(C.c_uint64)]
    L.ref_tf1d_resample(_f32p(t), t.shape[0], target, _f32p(out), lim)
    return out, (lim[0], lim[1])


def tf1d_fill_or_truncate(table, target):
    L = _load()
    t = np.ascontiguousarray(table, dtype=np.float32)
    out = np.zeros((target, 4), dtype=np.float32)
    L.ref_tf1d_fill_or_truncate.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.c_uint64,
                                            C.POINTER(C.c_float)]
    L.ref_tf1d_fill_or_truncate(_f32p(t), t.shape[0], target, _f32p(out))
    return out


def tf1d_bytes(table, used_range=255):
    L = _load()
    t = np.ascontiguousarray(table, dtype=np.float32)
    out = np.zeros(t.size, dtype=np.uint8)
    L.ref_tf1d_bytes.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.c_uint8,
                                 C.POINTER(C.c_uint8)]
    L.ref_tf1d_bytes(_f32p(t), t.shape[0], used_range, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def tf1d_save(table, path):
    L = _load()
    t = np.ascontiguousarray(table, dtype=np.float32)
    L.ref_tf1d_save.argtypes = [C.POINTER(C.c_float), C.c_uint64, C.c_char_p]
    return bool(L.ref_tf1d_save(_f32p(t), t.shape[0], str(path).encode()))


def tf1d_load(path, cap=1 << 16):
    """(table, ok) as TransferFunction1D::Load(filename) leaves it."""
    L = _load()
    out = np.zeros((cap, 4), dtype=np.float32)
    n = C.c_uint64()
    L.ref_tf1d_load.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.c_uint64,
                                C.POINTER(C.c_uint64)]
    ok = L.ref_tf1d_load(str(path).encode(), _f32p(out), cap, C.byref(n))
    return (out[:n.value].copy(), True) if ok else (None, False)


# ---- UVF container (oracle/ref/ref_uvf.cpp over IO/UVF/UVF.cpp and its blocks)

def write_uvf(path, raw, brick_size, overlap, clamp=False, compression=0, level=0, layout=0,
              checksum=2, big_endian=False, kv_first=False, histograms=2, components=1,
              scratch="/tmp"):
    """The reference's UVF writer, blocks as RAWConverter assembles them: raw
    is [t, z, y, x] (or [t, z, y, x, 4]) uint8 / uint16, one TOC block per
    timestep.  checksum 0 none, 1 CRC32, 2 MD5; histograms 0 none, 1 the 1D
    block, 2 both."""
    L = _load()
    L.ref_write_uvf.restype = C.c_int
    L.ref_write_uvf.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_uint32, C.c_int,
                                C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                C.c_uint32, C.c_int, C.c_int, C.c_uint32, C.c_int, C.c_int,
                                C.c_int, C.c_int, C.c_int]
    raw = np.ascontiguousarray(raw)
    dims = (C.c_uint64 * 3)(raw.shape[3], raw.shape[2], raw.shape[1])
    ok = L.ref_write_uvf(str(path).encode(), str(scratch).encode(),
                         raw.ctypes.data_as(C.c_void_p), raw.shape[0],
                         0 if raw.dtype == np.uint8 else 1, components, dims,
                         (C.c_uint32 * 3)(*brick_size), overlap, int(clamp), compression, level,
                         layout, checksum, int(big_endian), int(kv_first), histograms)
    if ok != 1:
        raise RuntimeError("reference UVF writer failed")


def read_uvf(path, verify=False):
    """UVF::Open(bMustBeSameVersion = false, bVerify = verify) and its block
    table: ({version, big_endian, blocks: rows of (offset, semantics,
    compression, offset to next, id length, octree offset, components, LOD
    count)}, "") or (None, the parser's reason)."""
    L = _load()
    L.ref_read_uvf.restype = C.c_int64
    L.ref_read_uvf.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_int),
                               C.POINTER(C.c_uint64), C.c_size_t, C.c_char_p, C.c_size_t]
    version, be = C.c_uint64(), C.c_int()
    rows = (C.c_uint64 * (8 * 256))()
    why = C.create_string_buffer(512)
    n = L.ref_read_uvf(str(path).encode(), int(verify), C.byref(version), C.byref(be), rows, 256,
                       why, 512)
    if n < 0:
        return None, why.value.decode(errors="replace")
    return dict(version=version.value, big_endian=be.value,
                blocks=[list(rows[8 * i:8 * i + 8]) for i in range(min(n, 256))]), ""
