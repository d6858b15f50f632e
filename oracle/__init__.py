"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it as the checker / CPU baseline.  The
product (tuvok_gb300, libtvk.so) never imports or calls it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "liboracle.so"
REF_PATH = Path(__file__).resolve().parent / "_ref" / "libtuvok_ref.so"

_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)


class Scene(C.Structure):
    _fields_ = [
        ("raw", C.c_void_p), ("dtype", C.c_int), ("dims", C.c_uint64 * 3),
        ("brick_size", C.c_uint32 * 3), ("overlap", C.c_uint32), ("clamp_to_edge", C.c_int),
        ("user_scale", C.c_double * 3), ("tf", C.POINTER(C.c_float)), ("tf_w", C.c_uint32),
        ("tf_h", C.c_uint32), ("tf_rgba8", C.c_int), ("render_mode", C.c_int),
        ("lighting", C.c_int), ("light_model", C.c_int), ("ambient", C.c_float * 4),
        ("diffuse", C.c_float * 4), ("specular", C.c_float * 4), ("light_dir", C.c_float * 3),
        ("bp_ka", C.c_float), ("bp_kd", C.c_float), ("bp_ks", C.c_float),
        ("bp_shininess", C.c_float), ("isovalue", C.c_float),
        ("sample_rate_modifier", C.c_float), ("frame_ert", C.c_float), ("eye", C.c_float * 3),
        ("at", C.c_float * 3), ("up", C.c_float * 3), ("fovy_deg", C.c_float),
        ("znear", C.c_float), ("zfar", C.c_float), ("width", C.c_uint32),
        ("height", C.c_uint32), ("use_double", C.c_int), ("row_stride", C.c_uint32),
        ("row_phase", C.c_uint32), ("threads", C.c_int), ("iso_color", C.c_float * 3),
        ("lod", C.c_uint32), ("median", C.c_int), ("decrease_screen_res", C.c_int),
        ("decrease_sampling_rate", C.c_int), ("screen_res_dec_factor", C.c_float),
        ("sample_dec_factor", C.c_float), ("clip_on", C.c_int), ("clip_plane", C.c_float * 4),
        ("cv_on", C.c_int), ("cv_isovalue", C.c_float), ("cv_color", C.c_float * 3),
        ("cv_size", C.c_float), ("cv_context_scale", C.c_float), ("cv_border_scale", C.c_float),
        ("cv_pos", C.c_float * 4), ("tf_bias_scale", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} missing: run tuvok_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        L.orc_lod_table.argtypes = [_u64p, _u32p, C.c_uint32, _u64p, _u64p, C.c_int]
        L.orc_lod_table.restype = C.c_int
        L.orc_brick_size.argtypes = [_u64p, _u64p, _u32p, C.c_uint32, _u64p, _u64p]
        L.orc_brick_size.restype = None
        L.orc_lod0_brick.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int,
                                     _u64p, C.c_void_p]
        L.orc_lod0_brick.restype = None
        L.orc_brick_stats.argtypes = [C.c_void_p, C.c_int, C.c_uint64,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_brick_stats.restype = None
        L.orc_histogram1d.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, _u64p]
        L.orc_histogram1d.restype = C.c_uint64
        L.orc_brick_hist256.argtypes = [C.c_void_p, C.c_int, _u64p, C.c_uint32, C.c_uint32,
                                        _u32p]
        L.orc_brick_hist256.restype = None
        L.orc_brick_metadata.argtypes = [_u64p, _u64p, _u32p, C.c_uint32,
                                         C.POINTER(C.c_double), C.POINTER(C.c_float),
                                         C.POINTER(C.c_float), _u32p]
        L.orc_brick_metadata.restype = None
        L.orc_max_gradient.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int]
        L.orc_max_gradient.restype = C.c_double
        L.orc_histogram2d.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int,
                                      C.c_uint64, C.c_double, _u64p]
        L.orc_histogram2d.restype = C.c_double
        L.orc_rebrick.argtypes = [C.c_int, _u64p, _u32p, C.c_uint32, C.c_uint32, C.c_void_p,
                                  _u64p, C.POINTER(C.c_double), C.POINTER(C.c_double), _u32p,
                                  C.c_int, C.c_uint64, _u32p, C.POINTER(C.c_float), _u64p,
                                  C.POINTER(C.c_double), C.c_void_p, C.c_uint64, _u64p, _u64p]
        L.orc_rebrick.restype = C.c_int64
        L.orc_render_size.argtypes = [C.POINTER(Scene), _u32p, _u32p]
        L.orc_render_size.restype = None
        L.orc_lod_aspect.argtypes = [_u64p, C.c_uint32, C.POINTER(C.c_double)]
        L.orc_lod_aspect.restype = None
        L.orc_render.argtypes = [C.POINTER(Scene), C.POINTER(C.c_float), _u32p]
        L.orc_render.restype = C.c_uint64
        L.orc_pow01.argtypes = [C.c_float, C.c_float]
        L.orc_pow01.restype = C.c_float
        L.orc_round_half.argtypes = [C.c_float]
        L.orc_round_half.restype = C.c_float
        L.orc_render_timed.argtypes = [C.POINTER(Scene), C.POINTER(C.c_float), _u32p,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_render_timed.restype = C.c_uint64
        L.orc_prepare.argtypes = [C.POINTER(Scene)]
        L.orc_prepare.restype = C.c_void_p
        L.orc_render_prepared.argtypes = [C.c_void_p, C.POINTER(Scene), C.POINTER(C.c_float),
                                          _u32p, C.POINTER(C.c_double)]
        L.orc_render_prepared.restype = C.c_uint64
        L.orc_release.argtypes = [C.c_void_p]
        L.orc_release.restype = None
        L.orc_build_octree.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int,
                                       C.c_int, C.c_void_p, C.c_uint64, _u64p, C.c_uint64]
        L.orc_build_octree.restype = C.c_int64
        L.orc_leaper_render.argtypes = [C.POINTER(Scene), _u32p, C.c_uint64,
                                        C.POINTER(C.c_float), _u32p, _u64p, C.c_uint64, _u64p]
        L.orc_leaper_render.restype = C.c_uint64
        L.orc_generate_volume.argtypes = [C.c_void_p, C.c_int, _u64p, C.POINTER(C.c_float),
                                          C.c_uint32, C.c_float, C.c_uint32, C.c_float,
                                          C.c_uint64, C.c_int, C.c_float, C.c_int]
        L.orc_generate_volume.restype = C.c_int
        L.orc_convert_timed.argtypes = [C.c_void_p, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int,
                                        C.POINTER(C.c_double), _u64p]
        L.orc_convert_timed.restype = C.c_int64
        L.orc_volume_hash.argtypes = [C.c_void_p, C.c_uint64, C.c_int]
        L.orc_volume_hash.restype = C.c_uint64
        _lib = L
    return _lib


def _u64(v):
    return (C.c_uint64 * len(v))(*[int(x) for x in v])


def _u32(v):
    return (C.c_uint32 * len(v))(*[int(x) for x in v])


def _dt(arr):
    """0 = u8, 1 = u16 ([z, y, x]); 2 = RGBA8 colour ([z, y, x, 4] uint8)."""
    if arr.dtype == np.uint8 and arr.ndim == 4:
        return 2
    return 0 if arr.dtype == np.uint8 else 1


def lod_table(dims, brick_size, overlap):
    sizes = (C.c_uint64 * (3 * 64))()
    counts = (C.c_uint64 * (3 * 64))()
    n = lib().orc_lod_table(_u64(dims), _u32(brick_size), overlap, sizes, counts, 64)
    return ([tuple(sizes[3 * i:3 * i + 3]) for i in range(n)],
            [tuple(counts[3 * i:3 * i + 3]) for i in range(n)])


def brick_size(lod_size, brick_count, bsize, overlap, coords):
    out = (C.c_uint64 * 3)()
    lib().orc_brick_size(_u64(lod_size), _u64(brick_count), _u32(bsize), overlap, _u64(coords),
                         out)
    return tuple(out)


def lod0_brick(raw, bsize, overlap, clamp, coords):
    """raw: numpy [z, y, x]; returns the brick as [z, y, x]."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    sizes, counts = lod_table(dims, bsize, overlap)
    bs = brick_size(sizes[0], counts[0], bsize, overlap, coords)
    out = np.zeros((bs[2], bs[1], bs[0]) + raw.shape[3:], dtype=raw.dtype)
    lib().orc_lod0_brick(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims), _u32(bsize),
                         overlap, int(clamp), _u64(coords), out.ctypes.data_as(C.c_void_p))
    return out


def brick_stats(brick):
    mn, mx = C.c_double(), C.c_double()
    b = np.ascontiguousarray(brick)
    lib().orc_brick_stats(b.ctypes.data_as(C.c_void_p), _dt(b), b.size, C.byref(mn), C.byref(mx))
    return mn.value, mx.value


def histogram1d(raw, bsize, overlap):
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    out = np.zeros(1 << (8 * raw.dtype.itemsize), dtype=np.uint64)
    n = lib().orc_histogram1d(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims),
                              _u32(bsize), overlap, out.ctypes.data_as(_u64p))
    return out, int(n)


def brick_hist256(brick, overlap, shift):
    b = np.ascontiguousarray(brick)
    out = np.zeros(256, dtype=np.uint32)
    n = (b.shape[2], b.shape[1], b.shape[0])
    lib().orc_brick_hist256(b.ctypes.data_as(C.c_void_p), _dt(b), _u64(n), overlap, shift,
                            out.ctypes.data_as(_u32p))
    return out


def brick_metadata(lod_size, brick_count, bsize, overlap, aspect=(1.0, 1.0, 1.0)):
    nb = brick_count[0] * brick_count[1] * brick_count[2]
    c = np.zeros((nb, 3), dtype=np.float32)
    e = np.zeros((nb, 3), dtype=np.float32)
    n = np.zeros((nb, 3), dtype=np.uint32)
    lib().orc_brick_metadata(_u64(lod_size), _u64(brick_count), _u32(bsize), overlap,
                             (C.c_double * 3)(*aspect), c.ctypes.data_as(C.POINTER(C.c_float)),
                             e.ctypes.data_as(C.POINTER(C.c_float)), n.ctypes.data_as(_u32p))
    return c, e, n


def max_gradient(raw, bsize, overlap, clamp=False):
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    return lib().orc_max_gradient(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims),
                                  _u32(bsize), overlap, int(clamp))


def histogram2d(raw, bsize, overlap, clamp=False, value_bins=None, max_nonzero=None):
    """[value_bins, 256] value x |gradient| counts and the maximum |gradient|.

    Defaults follow RAWConverter: value_bins = the trimmed 1D histogram's
    length, max_nonzero = the volume's maximum value."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    if value_bins is None:
        value_bins = int(raw.max()) + 1
    if max_nonzero is None:
        max_nonzero = float(raw.max())
    out = np.zeros((value_bins, 256), dtype=np.uint64)
    g = lib().orc_histogram2d(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims), _u32(bsize),
                              overlap, int(clamp), value_bins, max_nonzero,
                              out.ctypes.data_as(_u64p))
    return out, g


def build_octree(raw, bsize, overlap, clamp=False, median=False):
    """Every brick of every LOD in TOC order: list of [z, y, x] arrays."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    sizes, counts = lod_table(dims, bsize, overlap)
    shapes = []
    for l, (ls, lc) in enumerate(zip(sizes, counts)):
        for z in range(lc[2]):
            for y in range(lc[1]):
                for x in range(lc[0]):
                    shapes.append(brick_size(ls, lc, bsize, overlap, (x, y, z)))
    total = sum(s[0] * s[1] * s[2] for s in shapes)
    comps = raw.shape[3:]  # (4,) for RGBA8 colour volumes
    pool = np.zeros((total,) + comps, dtype=raw.dtype)
    offs = np.zeros(len(shapes), dtype=np.uint64)
    n = lib().orc_build_octree(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims),
                               _u32(bsize), overlap, int(clamp), int(median),
                               pool.ctypes.data_as(C.c_void_p), total,
                               offs.ctypes.data_as(_u64p), len(shapes))
    assert n == len(shapes), n
    out = []
    for s, o in zip(shapes, offs):
        out.append(pool[int(o):int(o) + s[0] * s[1] * s[2]].reshape((s[2], s[1], s[0]) + comps))
    return out


def pow01(x, y):
    """The FP32 oracle's GLSL pow(x, y) for x in [0, 1]."""
    return lib().orc_pow01(float(x), float(y))


def generate_volume(dims, dtype, blobs, noise_amp, octaves, cell, seed, int_noise, vmax,
                    threads=0):
    """The seeded volume tvk_generate_volume makes, restated on the host:
    numpy [z, y, x] of dtype (uint8 / uint16), the same bytes."""
    out = np.zeros((dims[2], dims[1], dims[0]), dtype=dtype)
    b = np.ascontiguousarray(np.asarray(blobs, dtype=np.float32).reshape(-1, 7))
    rc = lib().orc_generate_volume(out.ctypes.data_as(C.c_void_p), 0 if dtype == np.uint8 else 1,
                                   _u64(dims), b.ctypes.data_as(C.POINTER(C.c_float)),
                                   b.shape[0], float(noise_amp), int(octaves), float(cell),
                                   int(seed), int(int_noise), float(vmax), int(threads))
    if rc != 0:
        raise ValueError("bad generator arguments")
    return out


def convert_timed(raw, bsize, overlap, clamp=False):
    """The serial CPU bricking of ExtendedOctreeConverter::Convert restated
    (every LOD's bricks with ghost voxels, per-brick min/max, the 1D
    histogram) on one thread: (seconds, bricks, brick-pool bytes)."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    t = C.c_double()
    pb = C.c_uint64()
    n = lib().orc_convert_timed(raw.ctypes.data_as(C.c_void_p), _dt(raw), _u64(dims),
                                _u32(bsize), overlap, int(clamp), C.byref(t), C.byref(pb))
    if n < 0:
        raise ValueError("conversion failed")
    return t.value, int(n), int(pb.value)


def volume_hash(arr, threads=0):
    """FNV-1a of the FNV-1a digests of every 1 MiB chunk of the bytes (hex)."""
    a = np.ascontiguousarray(arr)
    return f"{lib().orc_volume_hash(a.ctypes.data_as(C.c_void_p), a.nbytes, threads):016x}"


def round_half(x):
    return lib().orc_round_half(float(x))


def make_scene(raw, bsize, overlap, tf, *, width=1, height=1, eye=(0, 0, 1.6), at=(0, 0, 0),
               up=(0, 1, 0), fovy=50.0, znear=0.01, zfar=1000.0, srm=1.0, mode=0,
               lighting=False, light_model=0, tf_rgba8=False, clamp=False,
               ambient=(1, 1, 1, 0.1), diffuse=(1, 1, 1, 1), specular=(1, 1, 1, 1),
               light_dir=(0, 0, -1), bp=(0.2, 0.6, 0.2, 32.0), frame_ert=1.0,
               use_double=False, row_stride=1, row_phase=0, threads=0, isovalue=None,
               iso_color=(0.5, 0.5, 0.5), lod=0, median=False, dec_screen=False,
               dec_sampling=False, screen_dec=2.0, sample_dec=2.0, clip_plane=None,
               clearview=None, bias_scale=False):
    """Scene struct for the oracle; returns (scene, arrays that must stay alive).

    clearview: None, or a dict with any of isovalue (default 1.5 x the
    isovalue), color, size, context_scale, border_scale, pos (model space,
    4 components) -- the AbstrRenderer ClearView state."""
    raw = np.ascontiguousarray(raw)
    tf = np.ascontiguousarray(np.asarray(tf, dtype=np.float32))
    s = Scene()
    s.raw = raw.ctypes.data_as(C.c_void_p)
    s.dtype = _dt(raw)
    s.dims[:] = (raw.shape[2], raw.shape[1], raw.shape[0])
    s.brick_size[:] = tuple(bsize)
    s.overlap = overlap
    s.clamp_to_edge = int(clamp)
    s.user_scale[:] = (1.0, 1.0, 1.0)
    s.tf = tf.ctypes.data_as(C.POINTER(C.c_float))
    if tf.ndim == 3:
        s.tf_h, s.tf_w = tf.shape[0], tf.shape[1]
    else:
        s.tf_h, s.tf_w = 1, tf.shape[0]
    s.tf_rgba8 = int(tf_rgba8)
    s.render_mode = int(mode)
    s.lighting = int(bool(lighting))
    s.light_model = int(light_model)
    s.ambient[:] = ambient
    s.diffuse[:] = diffuse
    s.specular[:] = specular
    s.light_dir[:] = light_dir
    s.bp_ka, s.bp_kd, s.bp_ks, s.bp_shininess = bp
    s.sample_rate_modifier = srm
    s.frame_ert = frame_ert
    s.eye[:] = eye
    s.at[:] = at
    s.up[:] = up
    s.fovy_deg, s.znear, s.zfar = fovy, znear, zfar
    s.width, s.height = width, height
    s.use_double = int(use_double)
    s.row_stride, s.row_phase = row_stride, row_phase
    s.lod, s.median = lod, int(median)
    s.decrease_screen_res, s.decrease_sampling_rate = int(dec_screen), int(dec_sampling)
    s.screen_res_dec_factor, s.sample_dec_factor = screen_dec, sample_dec
    s.threads = threads
    # AbstrRenderer.cpp:252-261: half the data range once a dataset is loaded,
    # the ClearView isovalue half as much again above that
    # colour volumes: the 8-bit channel range
    rng = (0.0, 255.0) if raw.ndim == 4 else (float(raw.min()), float(raw.max()))
    default_iso = np.float32(rng[1] - rng[0]) / np.float32(2.0)
    if isovalue is None:
        isovalue = float(default_iso)
    s.isovalue = isovalue
    s.iso_color[:] = iso_color
    if clip_plane is not None:
        s.clip_on = 1
        s.clip_plane[:] = [float(x) for x in clip_plane]
    s.tf_bias_scale = int(bool(bias_scale))
    if clearview is not None:
        cv = dict(clearview)
        s.cv_on = 1
        s.cv_isovalue = cv.get("isovalue",
                               float(default_iso + default_iso / np.float32(2.0)))
        s.cv_color[:] = cv.get("color", (1.0, 0.0, 0.0))
        s.cv_size = cv.get("size", 5.5)
        s.cv_context_scale = cv.get("context_scale", 1.0)
        s.cv_border_scale = cv.get("border_scale", 60.0)
        s.cv_pos[:] = cv.get("pos", (0.0, 0.0, 0.5, 1.0))
    return s, (raw, tf)


def render(raw, bsize, overlap, tf, *, width, height, want_counts=False, **kw):
    """Oracle render of raw ([z, y, x]) -> (image [h, w, 4], samples, counts|None)."""
    s, keep = make_scene(raw, bsize, overlap, tf, width=width, height=height, **kw)
    img = np.zeros((height, width, 4), dtype=np.float32)
    rw, rh = C.c_uint32(), C.c_uint32()
    lib().orc_render_size(C.byref(s), C.byref(rw), C.byref(rh))
    counts = np.zeros((rh.value, rw.value), dtype=np.uint32) if want_counts else None
    n = lib().orc_render(C.byref(s), img.ctypes.data_as(C.POINTER(C.c_float)),
                         counts.ctypes.data_as(_u32p) if want_counts else None)
    del keep
    return img, int(n), counts


class Prepared:
    """Oracle scene bricked once; render() takes a camera each call."""

    def __init__(self, raw, bsize, overlap, tf, **kw):
        self._scene, self._keep = make_scene(raw, bsize, overlap, tf, **kw)
        self._kw = kw
        self._h = lib().orc_prepare(C.byref(self._scene))

    def render(self, *, eye, width, height, at=(0, 0, 0), up=(0, 1, 0), row_stride=1,
               row_phase=0, threads=0, use_double=False, want_counts=False):
        """(image [h, w, 4], samples, march seconds), plus the per-pixel
        sample counts [h, w] with want_counts.  Only the rows py with
        py % row_stride == row_phase are marched; the others stay zero."""
        cam = Scene()
        cam.eye[:] = eye
        cam.at[:] = at
        cam.up[:] = up
        cam.fovy_deg = self._scene.fovy_deg
        cam.znear, cam.zfar = self._scene.znear, self._scene.zfar
        cam.width, cam.height = width, height
        cam.row_stride, cam.row_phase = row_stride, row_phase
        cam.threads = threads
        cam.use_double = int(use_double)
        img = np.zeros((height, width, 4), dtype=np.float32)
        counts = np.zeros((height, width), dtype=np.uint32) if want_counts else None
        t = C.c_double()
        n = lib().orc_render_prepared(self._h, C.byref(cam),
                                      img.ctypes.data_as(C.POINTER(C.c_float)),
                                      counts.ctypes.data_as(_u32p) if want_counts else None,
                                      C.byref(t))
        if want_counts:
            return img, int(n), t.value, counts
        return img, int(n), t.value

    def close(self):
        if self._h:
            lib().orc_release(self._h)
            self._h = None

    def __del__(self):
        self.close()


def leaper_render(raw, bsize, overlap, tf, page, *, width, height, **kw):
    """One GridLeaper pass over the page table `page` (one entry per brick of
    every LOD in TOC order: 0 MISSING, 1 CHILD_EMPTY, 2 EMPTY, >= 3 resident).
    Returns (image [h, w, 4], samples, counts [h, w], missing TOC indices)."""
    raw = np.ascontiguousarray(raw)
    _, cnt = lod_table((raw.shape[2], raw.shape[1], raw.shape[0]), bsize, overlap)
    page = np.ascontiguousarray(page, dtype=np.uint32)
    if page.size != sum(c[0] * c[1] * c[2] for c in cnt):
        raise ValueError("the page table needs one entry per brick of every LOD")
    s, keep = make_scene(raw, bsize, overlap, tf, width=width, height=height, **kw)
    img = np.zeros((height, width, 4), dtype=np.float32)
    counts = np.zeros((height, width), dtype=np.uint32)
    missing = np.zeros(page.size, dtype=np.uint64)
    nm = C.c_uint64()
    n = lib().orc_leaper_render(C.byref(s), page.ctypes.data_as(_u32p), page.size,
                                img.ctypes.data_as(C.POINTER(C.c_float)),
                                counts.ctypes.data_as(_u32p), missing.ctypes.data_as(_u64p),
                                page.size, C.byref(nm))
    del keep
    return img, int(n), counts, missing[:nm.value].astype(np.int64)


def tf_value_limits(tf, range_max):
    """The value range the TF reaches (AbstrRenderer::ContainsData's limits):
    the first and last TF column with a non-zero alpha, times
    range_max / (width - 1) (GLGridLeaper.cpp:650-670)."""
    tf = np.asarray(tf, dtype=np.float32)
    a = tf[..., 3].reshape(-1, tf.shape[-2]) if tf.ndim == 3 else tf[:, 3][None, :]
    cols = np.nonzero((a != 0).any(axis=0))[0]
    w = a.shape[1]
    lo, hi = (int(cols[0]), int(cols[-1])) if cols.size else (w, 0)
    rescale = float(range_max) / float(max(w, 2) - 1)
    return lo * rescale, hi * rescale


def leaper_visibility(raw, bsize, overlap, cached, *, lo=0.0, hi=0.0, isovalue=None,
                      median=False, clamp=False):
    """GLVolumePool::RecomputeVisibility (GLVolumePool.cpp:1580-1700) restated:
    every entry MISSING; the bricks in `cached` (TOC index -> slot entry, the
    cached bricks that hold visible data) keep their entry; every other brick
    that holds nothing visible (ContainsData, :962-989: value range [lo, hi], or
    the isovalue) becomes CHILD_EMPTY when every existing child is CHILD_EMPTY
    (the finest LOD always), else EMPTY (RecomputeVisibilityForOctree,
    :1020-1359).  Returns the page table (uint32)."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    bricks = build_octree(raw, bsize, overlap, clamp=clamp, median=median)
    _, counts = lod_table(dims, bsize, overlap)
    first = np.concatenate([[0], np.cumsum([c[0] * c[1] * c[2] for c in counts])]).astype(int)
    page = np.zeros(first[-1], dtype=np.uint32)
    for i, e in cached.items():
        page[i] = e
    for l, c in enumerate(counts):
        for k in range(c[0] * c[1] * c[2]):
            i = first[l] + k
            if page[i] >= 3:
                continue
            mn, mx = brick_stats(bricks[i])
            has = (isovalue >= mn and isovalue <= mx) if isovalue is not None else \
                (hi >= mn and lo <= mx)
            if has:
                continue
            child_empty = True
            if l > 0:
                cc = counts[l - 1]
                x, y, z = k % c[0], (k // c[0]) % c[1], k // (c[0] * c[1])
                for dz in (0, 1):
                    for dy in (0, 1):
                        for dx in (0, 1):
                            cx, cy, cz = 2 * x + dx, 2 * y + dy, 2 * z + dz
                            if cx < cc[0] and cy < cc[1] and cz < cc[2]:
                                ci = first[l - 1] + cx + cy * cc[0] + cz * cc[0] * cc[1]
                                child_empty &= page[ci] == 1
            page[i] = 1 if child_empty else 2
    return page


class RebrickError(ValueError):
    """The reference's DynamicBrickingDS throws (code -1) or would read outside
    a source brick (code -2)."""

    def __init__(self, code):
        super().__init__("not an integer multiple of the source brick size" if code == -1
                         else "a target brick reads outside its source brick")
        self.code = code


def rebrick(raw, src_bsize, overlap, tgt_bsize, mm_mode=1, clamp=False, median=False,
            lod0_only=False):
    """DynamicBrickingDS over the ExtendedOctree of raw: a list of dicts per
    target brick in TOC order {lod, index, n_voxels, center, extents,
    src_index, min, max, data [z, y, x]}.  mm_mode 0 = MM_SOURCE, 1 =
    MM_PRECOMPUTE, 2 = MM_DYNAMIC."""
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    src = build_octree(raw, src_bsize, overlap, clamp=clamp, median=median)
    sizes, counts = lod_table(dims, src_bsize, overlap)
    n_built = 1 if lod0_only else len(sizes)
    offs = np.zeros(len(src), dtype=np.uint64)
    o = 0
    for i, b in enumerate(src):
        offs[i] = o
        o += b.size
    pool = np.concatenate([b.reshape(-1) for b in src])
    mn = np.array([float(b.min()) for b in src])
    mx = np.array([float(b.max()) for b in src])
    need = C.c_uint64()
    args = [_dt(raw), _u64(dims), _u32(src_bsize), overlap, n_built,
            pool.ctypes.data_as(C.c_void_p), offs.ctypes.data_as(_u64p),
            mn.ctypes.data_as(C.POINTER(C.c_double)), mx.ctypes.data_as(C.POINTER(C.c_double)),
            _u32(tgt_bsize), mm_mode]
    n = lib().orc_rebrick(*args, 0, None, None, None, None, None, 0, None, C.byref(need))
    if n < 0:
        raise RebrickError(int(n))
    info = np.zeros((n, 4), dtype=np.uint32)
    geom = np.zeros((n, 6), dtype=np.float32)
    sidx = np.zeros(n, dtype=np.uint64)
    mm = np.zeros((n, 2), dtype=np.float64)
    out = np.zeros(int(need.value), dtype=raw.dtype)
    ooff = np.zeros(n, dtype=np.uint64)
    n2 = lib().orc_rebrick(*args, n, info.ctypes.data_as(_u32p),
                           geom.ctypes.data_as(C.POINTER(C.c_float)), sidx.ctypes.data_as(_u64p),
                           mm.ctypes.data_as(C.POINTER(C.c_double)),
                           out.ctypes.data_as(C.c_void_p), out.size, ooff.ctypes.data_as(_u64p),
                           C.byref(need))
    assert n2 == n
    res = []
    per_lod = {}
    for t in range(n):
        lod = int(info[t, 0])
        nx, ny, nz = (int(v) for v in info[t, 1:])
        k = per_lod.get(lod, 0)
        per_lod[lod] = k + 1
        o = int(ooff[t])
        res.append({"lod": lod, "index": k, "n_voxels": (nx, ny, nz),
                    "center": tuple(geom[t, :3]), "extents": tuple(geom[t, 3:]),
                    "src_index": int(sidx[t]), "min": mm[t, 0], "max": mm[t, 1],
                    "data": out[o:o + nx * ny * nz].reshape(nz, ny, nx)})
    return res
