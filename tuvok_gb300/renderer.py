"""Python mirror of Tuvok's renderer and dataset interfaces over the C ABI.

``Volume`` stands where Tuvok's bricked dataset (``BrickedDataset`` /
``UVFDataset`` built by ``ExtendedOctreeConverter``) stands; ``Renderer``
keeps ``AbstrRenderer``'s method names (Renderer/AbstrRenderer.h) so callers
and tests read like the reference's.  All compute runs in libtvk.so on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from ._native import check, lib


def _u64(v):
    return (C.c_uint64 * len(v))(*[int(x) for x in v])


def _u32(v):
    return (C.c_uint32 * len(v))(*[int(x) for x in v])


def _f32(v):
    return (C.c_float * len(v))(*[float(x) for x in v])


class Volume:
    """A volume bricked on the GPU (LOD 0 with ghost voxels + statistics).

    ``data`` is a numpy array indexed [z, y, x] (x fastest in memory), or a
    device pointer (int) together with ``dims`` and ``dtype``.
    """

    CLAMP_TO_EDGE, DEVICE_INPUT, MEDIAN, LOD0_ONLY = 1, 2, 4, 8
    MM_SOURCE, MM_PRECOMPUTE, MM_DYNAMIC = N.TVK_MM_SOURCE, N.TVK_MM_PRECOMPUTE, N.TVK_MM_DYNAMIC

    def __init__(self, data, brick_size=(64, 64, 64), overlap=1, clamp_to_edge=False,
                 dims=None, dtype=None, median=False, lod0_only=False, _handle=None):
        if _handle is not None:
            self._h = _handle
            self.info = N.VolumeInfo()
            check(lib().tvk_volume_get_info(self._h, C.byref(self.info)))
            return
        h = C.c_void_p()
        bs = _u32(brick_size)
        flags = ((self.CLAMP_TO_EDGE if clamp_to_edge else 0) | (self.MEDIAN if median else 0) |
                 (self.LOD0_ONLY if lod0_only else 0))
        if isinstance(data, np.ndarray):
            arr = np.ascontiguousarray(data)
            if arr.dtype == np.uint8 and arr.ndim == 4 and arr.shape[3] == 4:
                dt = N.TVK_RGBA8  # colour volume [z, y, x, rgba]
            elif arr.dtype == np.uint8 and arr.ndim == 3:
                dt = N.TVK_U8
            elif arr.dtype == np.uint16 and arr.ndim == 3:
                dt = N.TVK_U16
            else:
                raise TypeError("volumes are uint8 or uint16 [z, y, x], or uint8 [z, y, x, 4] RGBA")
            z, y, x = arr.shape[:3]
            check(lib().tvk_volume_create_ex(arr.ctypes.data_as(C.c_void_p), dt,
                                             _u64((x, y, z)), bs, overlap, flags, C.byref(h)))
        else:
            if dims is None or dtype is None:
                raise ValueError("a device pointer needs dims=(x, y, z) and dtype")
            dt = N.TVK_U8 if np.dtype(dtype) == np.uint8 else N.TVK_U16
            check(lib().tvk_volume_create_ex(C.c_void_p(int(data)), dt, _u64(dims), bs, overlap,
                                             flags | self.DEVICE_INPUT, C.byref(h)))
        self._h = h
        self.info = N.VolumeInfo()
        check(lib().tvk_volume_get_info(self._h, C.byref(self.info)))

    @classmethod
    def FromExtendedOctree(cls, path, offset=0, uvf_version=5, clamp_to_edge=False,
                           median=False, lod0_only=False):
        """ExtendedOctree::Open + GetBrickData: a converter-written brick file
        (uncompressed or LZ4 bricks), rebuilt on the GPU and checked brick by brick."""
        flags = ((cls.CLAMP_TO_EDGE if clamp_to_edge else 0) | (cls.MEDIAN if median else 0) |
                 (cls.LOD0_ONLY if lod0_only else 0))
        h = C.c_void_p()
        check(lib().tvk_volume_open_extended_octree(str(path).encode(), int(offset),
                                                    int(uvf_version), flags, C.byref(h)))
        return cls(None, _handle=h)

    @classmethod
    def FromUVF(cls, path, timestep=0, verify=False, clamp_to_edge=False, median=False,
                lod0_only=False):
        """UVFDataset::Open of a TOC-block UVF file: the ExtendedOctree of
        timestep `timestep`, opened as FromExtendedOctree opens it; `verify`
        checks the file's MD5 checksum first (UVF::VerifyChecksum)."""
        flags = ((cls.CLAMP_TO_EDGE if clamp_to_edge else 0) | (cls.MEDIAN if median else 0) |
                 (cls.LOD0_ONLY if lod0_only else 0) |
                 (N.TVK_UVF_VERIFY_CHECKSUM if verify else 0))
        h = C.c_void_p()
        check(lib().tvk_volume_open_uvf(str(path).encode(), int(timestep), flags, C.byref(h)))
        return cls(None, _handle=h)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            check(lib().tvk_volume_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- dataset interface (IO/Dataset.h, IO/BrickedDataset.h)
    @property
    def np_dtype(self):
        return np.uint16 if self.info.dtype == N.TVK_U16 else np.uint8

    def GetDomainSize(self, lod=0):
        s, b = _u64((0, 0, 0)), _u64((0, 0, 0))
        check(lib().tvk_volume_get_lod(self._h, lod, s, b))
        return tuple(s)

    def GetBrickLayout(self, lod=0):
        s, b = _u64((0, 0, 0)), _u64((0, 0, 0))
        check(lib().tvk_volume_get_lod(self._h, lod, s, b))
        return tuple(b)

    def GetLODLevelCount(self):
        return int(self.info.lod_count)

    def GetRange(self):
        return (self.info.range_min, self.info.range_max)

    def MaxGradientMagnitude(self):
        return self.info.max_gradient

    def GetBrickCount(self, lod=0):
        b = self.GetBrickLayout(lod)
        return b[0] * b[1] * b[2]

    def GetBrickMetadata(self, key):
        ts, lod, idx = key
        md = N.BrickMD()
        check(lib().tvk_volume_get_brick_md(self._h, ts, lod, idx, C.byref(md)))
        return md

    def GetBrick(self, key):
        """Brick voxels (ghost included) as a numpy array [z, y, x] ([z, y, x, 4]
        for a colour volume)."""
        md = self.GetBrickMetadata(key)
        nx, ny, nz = md.n_voxels
        shape = (nz, ny, nx, 4) if self.info.dtype == N.TVK_RGBA8 else (nz, ny, nx)
        out = np.empty(shape, dtype=self.np_dtype)
        ts, lod, idx = key
        check(lib().tvk_volume_get_brick(self._h, ts, lod, idx, out.ctypes.data_as(C.c_void_p),
                                         out.nbytes))
        return out

    def MaxMinForKey(self, key):
        ts, lod, idx = key
        mm = N.MinMax()
        check(lib().tvk_volume_get_minmax(self._h, ts, lod, idx, C.byref(mm)))
        return mm

    def GetCellMinMax(self, index):
        """Macro-cell (min, max) tables of brick `index` (TOC order), each
        [cells z, cells y, cells x] (see tvk_volume_cell_minmax)."""
        dims = (C.c_uint32 * 3)()
        check(lib().tvk_volume_cell_minmax(self._h, index, None, 0, dims))
        out = np.zeros((dims[2], dims[1], dims[0]), dtype=np.uint32)
        check(lib().tvk_volume_cell_minmax(self._h, index, out.ctypes.data_as(N._u32p),
                                           out.size, dims))
        return out & 0xFFFF, out >> 16

    def GetHistogram(self):
        bins = 1 << (8 * (1 if self.info.dtype == N.TVK_U8 else 2))
        out = np.zeros(bins, dtype=np.uint64)
        tl = C.c_uint64()
        check(lib().tvk_volume_get_histogram(self._h, out.ctypes.data_as(N._u64p), bins,
                                             C.byref(tl)))
        return out, int(tl.value)

    def Get2DHistogram(self, value_bins=0):
        """(counts [value_bins, 256] uint64, max gradient magnitude as float32);
        value_bins 0 = the trimmed 1D histogram's length."""
        bins = value_bins or self.GetHistogram()[1]
        out = np.zeros((bins, 256), dtype=np.uint64)
        used = C.c_uint64()
        g = C.c_float()
        check(lib().tvk_volume_get_histogram2d(self._h, out.ctypes.data_as(N._u64p), bins,
                                               out.size, C.byref(used), C.byref(g)))
        return out[:used.value], g.value

    def GetBrickHistograms(self):
        n = int(self.info.lod0_bricks)
        out = np.zeros((n, 256), dtype=np.uint32)
        sh = C.c_uint32()
        check(lib().tvk_volume_get_brick_histograms(self._h, out.ctypes.data_as(N._u32p), n,
                                                    C.byref(sh)))
        return out, int(sh.value)

    def Rebrick(self, brick_size, mm_mode=MM_PRECOMPUTE):
        """DynamicBrickingDS(self, brick_size, mm_mode): a new Volume of smaller
        bricks (ghost included in brick_size) cut from this one's."""
        h = C.c_void_p()
        check(lib().tvk_volume_rebrick(self._h, _u32(brick_size), int(mm_mode), C.byref(h)))
        return Volume(None, _handle=h)

    def GetMaxBrickSize(self):
        return tuple(self.info.brick_size)

    def ReleaseBricks(self):
        """Frees the device brick pool (tvk_volume_release_bricks): afterwards
        only a host-sourced Pool renders the volume."""
        check(lib().tvk_volume_release_bricks(self._h))

    def GetMaxUsedBrickSizes(self):
        out = _u32((0, 0, 0))
        check(lib().tvk_volume_get_max_used_brick_size(self._h, out))
        return tuple(out)

    def IndexFrom4D(self, x, y, z, lod):
        out = C.c_uint64()
        check(lib().tvk_volume_index_from_4d(self._h, _u64((x, y, z, lod)), C.byref(out)))
        return int(out.value)

    def IndexTo4D(self, lod, idx):
        out = _u64((0, 0, 0, 0))
        check(lib().tvk_volume_index_to_4d(self._h, lod, idx, out))
        return tuple(out)


class TransferFunction1D:
    """Tuvok's TransferFunction1D (IO/TransferFunction1D.h:53-101) over the C
    ABI's table functions: an n x 4 float32 RGBA table with the reference's
    methods, each giving its table bit for bit.  Host only.  Hand it to a
    renderer with ``Renderer.Set1DTransFloat(tf.GetColorData())``."""

    def __init__(self, size=0):
        self._t = np.zeros((int(size), 4), dtype=np.float32)
        self._limits = (0, 0)

    @classmethod
    def FromFile(cls, path, target_size=None):
        tf = cls()
        tf.Load(path, target_size)
        return tf

    def _p(self, a=None):
        a = self._t if a is None else a
        return a.ctypes.data_as(N._f32p)

    def GetSize(self):
        return self._t.shape[0]

    def Resize(self, size):
        t = np.zeros((int(size), 4), dtype=np.float32)
        k = min(int(size), self._t.shape[0])
        t[:k] = self._t[:k]
        self._t = t

    def GetColorData(self):
        return self._t

    def GetColor(self, i):
        return tuple(float(x) for x in self._t[i])

    def SetColor(self, i, rgba):
        self._t[i] = rgba

    def SetStdFunction(self, center=0.5, inv_gradient=0.5, component=None, inverted=False):
        """Both overloads: component None sets all four channels (not inverted)."""
        c = -1 if component is None else int(component)
        check(lib().tvk_tf1d_set_std_function(self._p(), self._t.shape[0], float(center),
                                              float(inv_gradient), c, int(bool(inverted))))
        self.ComputeNonZeroLimits()

    def Set(self, rgba_bytes):
        b = np.ascontiguousarray(np.asarray(rgba_bytes, dtype=np.uint8).reshape(-1))
        t = np.zeros((b.size // 4, 4), dtype=np.float32)
        with np.errstate(all="ignore"):
            check(lib().tvk_tf1d_from_bytes(b.ctypes.data_as(C.POINTER(C.c_uint8)), b.size // 4,
                                            self._p(t)))
        self._t = t
        self.ComputeNonZeroLimits()

    def Resample(self, target_size):
        target_size = int(target_size)
        if target_size == self._t.shape[0]:
            return  # the reference returns before recomputing the limits
        t = np.zeros((target_size, 4), dtype=np.float32)
        check(lib().tvk_tf1d_resample(self._p(), self._t.shape[0], self._p(t), target_size))
        self._t = t
        self.ComputeNonZeroLimits()

    def FillOrTruncate(self, target_size):
        t = np.zeros((int(target_size), 4), dtype=np.float32)
        check(lib().tvk_tf1d_fill_or_truncate(self._p(), self._t.shape[0], self._p(t),
                                              t.shape[0]))
        self._t = t
        self.ComputeNonZeroLimits()

    def Clear(self):
        self._t[:] = 0.0
        self._limits = (0, 0)

    def ComputeNonZeroLimits(self):
        lim = (C.c_uint64 * 2)()
        check(lib().tvk_tf1d_nonzero_limits(self._p(), self._t.shape[0], lim))
        self._limits = (int(lim[0]), int(lim[1]))

    def GetNonZeroLimits(self):
        return self._limits

    def GetByteArray(self, used_range=255):
        out = np.zeros(self._t.size, dtype=np.uint8)
        check(lib().tvk_tf1d_byte_array(self._p(), self._t.shape[0], int(used_range),
                                        out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out

    def GetShortArray(self, used_range=4095):
        out = np.zeros(self._t.size, dtype=np.uint16)
        check(lib().tvk_tf1d_short_array(self._p(), self._t.shape[0], int(used_range),
                                         out.ctypes.data_as(C.POINTER(C.c_uint16))))
        return out

    def Load(self, path, target_size=None):
        n = C.c_uint64()
        p = str(path).encode()
        check(lib().tvk_tf1d_load(p, None, 0, C.byref(n)))
        t = np.zeros((n.value, 4), dtype=np.float32)
        check(lib().tvk_tf1d_load(p, self._p(t), n.value, C.byref(n)))
        self._t = t
        self.ComputeNonZeroLimits()
        if target_size is not None:
            self.Resample(target_size)

    def Save(self, path):
        check(lib().tvk_tf1d_save(str(path).encode(), self._p(), self._t.shape[0]))


class Renderer:
    """GLRaycaster-equivalent renderer (AbstrRenderer's API over libtvk.so)."""

    RM_1DTRANS, RM_2DTRANS, RM_ISOSURFACE = (N.TVK_RM_1DTRANS, N.TVK_RM_2DTRANS,
                                              N.TVK_RM_ISOSURFACE)

    def __init__(self):
        h = C.c_void_p()
        check(lib().tvk_renderer_create(C.byref(h)))
        self._h = h
        self._w = self._h_px = 0
        self._vol = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            check(lib().tvk_renderer_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- AbstrRenderer surface
    def RegisterDataset(self, vol: Volume):
        self._vol = vol
        check(lib().tvk_renderer_set_volume(self._h, vol.handle))

    def Set1DTrans(self, rgba_bytes):
        a = np.ascontiguousarray(np.asarray(rgba_bytes, dtype=np.uint8).reshape(-1))
        check(lib().tvk_set_tf1d_rgba8(self._h, a.ctypes.data_as(C.POINTER(C.c_uint8)),
                                       a.size // 4))

    def Set1DTransFloat(self, rgba, rgba8_upload=False):
        a = np.ascontiguousarray(np.asarray(rgba, dtype=np.float32).reshape(-1))
        check(lib().tvk_set_tf1d_float(self._h, a.ctypes.data_as(N._f32p), a.size // 4,
                                       int(rgba8_upload)))

    def Set2DTransFloat(self, rgba, rgba8_upload=False):
        a = np.ascontiguousarray(np.asarray(rgba, dtype=np.float32))
        h, w = a.shape[0], a.shape[1]
        check(lib().tvk_set_tf2d_float(self._h, a.reshape(-1).ctypes.data_as(N._f32p), w, h,
                                       int(rgba8_upload)))

    def SetRendermode(self, mode):
        check(lib().tvk_set_render_mode(self._h, int(mode)))

    def SetUseLighting(self, on):
        check(lib().tvk_set_lighting(self._h, int(bool(on))))

    def SetSampleRateModifier(self, srm):
        check(lib().tvk_set_sample_rate_modifier(self._h, float(srm)))

    def SetIsoValue(self, v):
        check(lib().tvk_set_isovalue(self._h, float(v)))

    def SetIsosurfaceColor(self, rgb):
        check(lib().tvk_set_iso_color(self._h, _f32(rgb)))

    def SetColors(self, ambient, diffuse, specular, light_dir):
        check(lib().tvk_set_colors(self._h, _f32(ambient), _f32(diffuse), _f32(specular),
                                   _f32(light_dir)))

    def SetLightModel(self, model, ka=0.2, kd=0.6, ks=0.2, shininess=32.0):
        check(lib().tvk_set_light_model(self._h, int(model), ka, kd, ks, shininess))

    def SetViewParameters(self, fov, znear, zfar, eye=(0, 0, 1.6), at=(0, 0, 0), up=(0, 1, 0)):
        check(lib().tvk_set_view(self._h, _f32(eye), _f32(at), _f32(up), float(fov),
                                 float(znear), float(zfar)))

    def SetFrameTermination(self, threshold):
        check(lib().tvk_set_frame_termination(self._h, float(threshold)))

    def Resize(self, w, h):
        check(lib().tvk_resize(self._h, int(w), int(h)))
        self._w, self._h_px = int(w), int(h)

    def Paint(self):
        check(lib().tvk_paint(self._h))

    def ReadBackPixels(self, out=None):
        """Last frame as float32 [height, width, 4], row 0 = bottom row."""
        if out is None:
            out = np.empty((self._h_px, self._w, 4), dtype=np.float32)
        check(lib().tvk_read_image(self._h, out.ctypes.data_as(N._f32p), out.size))
        return out

    def ReadBackPixelsAsync(self, out):
        """Starts copying the last frame into `out` (float32 [height, width, 4],
        page-locked for overlap) while later frames render; WaitImage() ends it."""
        check(lib().tvk_read_image_async(self._h, out.ctypes.data_as(N._f32p), out.size))
        return out

    def WaitImage(self):
        """Waits for every asynchronous image copy asked for so far."""
        check(lib().tvk_wait_image(self._h))

    def SetClipPlane(self, plane):
        """AbstrRenderer::SetClipPlane: (a, b, c, d) in world space; n.x + d >= 0 is cut."""
        pl = (C.c_float * 4)(*[float(v) for v in plane])
        check(lib().tvk_set_clip_plane(self._h, pl))

    def EnableClipPlane(self, on=True):
        check(lib().tvk_enable_clip_plane(self._h, int(bool(on))))

    def DisableClipPlane(self):
        self.EnableClipPlane(False)

    SMETH_BIT_WIDTH, SMETH_BIAS_AND_SCALE = 0, 1

    def SetScalingMethod(self, method):
        """AbstrRenderer::SetScalingMethod: the 1D TF coordinate scale
        (SMETH_BIAS_AND_SCALE: value * (|min| + |max|), as GLRaycaster computes it)."""
        check(lib().tvk_set_scaling_method(self._h, int(method)))

    # ClearView (AbstrRenderer::SetCV and its parameters): in iso mode a focus
    # isosurface is revealed behind the context surface around a focus point.
    def SetCV(self, on=True):
        check(lib().tvk_set_clearview(self._h, int(bool(on))))

    def SetCVIsoValue(self, isovalue):
        """Focus isovalue in data units (default 1.5x the initial isovalue)."""
        check(lib().tvk_set_cv_isovalue(self._h, float(isovalue)))

    def SetCVColor(self, rgb):
        check(lib().tvk_set_cv_color(self._h, (C.c_float * 3)(*[float(v) for v in rgb])))

    def SetCVParams(self, size=5.5, context_scale=1.0, border_scale=60.0):
        """SetCVSize / SetCVContextScale / SetCVBorderScale."""
        check(lib().tvk_set_cv_params(self._h, float(size), float(context_scale),
                                      float(border_scale)))

    def SetCVFocusPosFVec(self, pos):
        """Focus point in model space, (x, y, z, w) with w = 1."""
        check(lib().tvk_set_cv_focus_pos(self._h, (C.c_float * 4)(*[float(v) for v in pos])))

    def GetCVFocusPos(self):
        out = (C.c_float * 4)()
        check(lib().tvk_get_cv_focus_pos(self._h, out))
        return tuple(out)

    def SetCVFocusPos(self, x, y):
        """Picks the focus point from the last ClearView frame's context hit at
        pixel (x, y) of the ray-marched image, row 0 at the bottom."""
        check(lib().tvk_set_cv_focus_pixel(self._h, int(x), int(y)))

    def SetLOD(self, lod):
        """m_iCurrentLOD for Paint()."""
        check(lib().tvk_set_lod(self._h, int(lod)))

    def SetReducedQuality(self, decrease_screen_res=False, decrease_sampling_rate=False):
        """decreaseScreenResNow / decreaseSamplingRateNow for Paint()."""
        check(lib().tvk_set_reduced_quality(self._h, int(bool(decrease_screen_res)),
                                            int(bool(decrease_sampling_rate))))

    def SetPerfMeasures(self, min_framerate=0, render_low_res_intermediate=False,
                        screen_res_dec_factor=2.0, sample_dec_factor=2.0):
        check(lib().tvk_set_perf_measures(self._h, int(min_framerate),
                                          int(bool(render_low_res_intermediate)),
                                          float(screen_res_dec_factor), float(sample_dec_factor)))

    def SetLODLimits(self, coarsest_skip, finest):
        check(lib().tvk_set_lod_limits(self._h, int(coarsest_skip), int(finest)))

    def SetCaptureMode(self, on):
        check(lib().tvk_set_capture_mode(self._h, int(bool(on))))

    def ComputeMinLODForCurrentView(self):
        out = C.c_uint32()
        check(lib().tvk_compute_min_lod(self._h, C.byref(out)))
        return out.value

    def PaintProgressive(self, new_frame=False):
        """One subframe of a progressive frame; returns its SubframeInfo."""
        info = N.SubframeInfo()
        check(lib().tvk_paint_progressive(self._h, int(bool(new_frame)), C.byref(info)))
        return info

    def GetRenderSize(self):
        w, h = C.c_uint32(), C.c_uint32()
        check(lib().tvk_get_render_size(self._h, C.byref(w), C.byref(h)))
        return w.value, h.value

    def ReadSampleCounts(self):
        """Per-pixel sample counts of the ray-marched image (GetRenderSize)."""
        w, h = self.GetRenderSize()
        out = np.empty((h, w), dtype=np.uint32)
        check(lib().tvk_read_sample_counts(self._h, out.ctypes.data_as(N._u32p), out.size))
        return out

    def GetStats(self):
        s = N.Stats()
        check(lib().tvk_get_stats(self._h, C.byref(s)))
        return s

    def SetHardwareFiltering(self, on):
        """Texture-unit trilinear lookups instead of the exact ones (see
        tvk_set_hardware_filtering): faster, not bit-exact."""
        check(lib().tvk_set_hardware_filtering(self._h, int(bool(on))))

    def GetCounters(self):
        """The last paint's raw counters (see tvk_get_counters)."""
        out = (C.c_uint64 * 8)()
        check(lib().tvk_get_counters(self._h, out))
        return list(out)

    def GetStream(self):
        s = C.c_void_p()
        check(lib().tvk_renderer_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def GetLastFBO(self):
        p = C.c_void_p()
        w, h = C.c_uint32(), C.c_uint32()
        check(lib().tvk_get_image_device(self._h, C.byref(p), C.byref(w), C.byref(h)))
        return p.value, w.value, h.value


class Batch:
    """Paints several renderers' frames in one persistent launch (tvk_paint_batch)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().tvk_batch_create(C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            check(lib().tvk_batch_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def SetAutotune(self, on=True, ctas_per_sm=0):
        check(lib().tvk_batch_set_autotune(self._h, int(bool(on)), int(ctas_per_sm)))

    def SetRaysPerThread(self, rays=0):
        """1 or 2 rays per thread (16x8 or 32x8 tiles); 0 lets the autotuner pick."""
        check(lib().tvk_batch_set_rays_per_thread(self._h, int(rays)))

    def Paint(self, renderers):
        arr = (C.c_void_p * len(renderers))(*[r._h.value for r in renderers])
        check(lib().tvk_paint_batch(self._h, arr, len(renderers)))

    def GetInfo(self):
        info = N.BatchInfo()
        check(lib().tvk_batch_get_info(self._h, C.byref(info)))
        return info


class Pool:
    """The GridLeaper's brick cache over a bricked volume (GLVolumePool): a
    device pool of brick slots holding at most ``budget_bytes``, a page table of
    every brick of every LOD, and the missing-brick hash table.  With
    ``host_source`` the bricks are paged from a pinned host copy (the
    out-of-core path); otherwise from the volume's device pool."""

    def __init__(self, volume, budget_bytes, host_source=False):
        h = C.c_void_p()
        check(lib().tvk_pool_create(volume.handle, int(budget_bytes), int(bool(host_source)),
                                    C.byref(h)))
        self._h = h
        self._vol = volume  # the pool reads the volume's bricks

    def close(self):
        if self._h:
            check(lib().tvk_pool_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def GetInfo(self):
        info = N.PoolInfo()
        check(lib().tvk_pool_get_info(self._h, C.byref(info)))
        return info

    def GetPageTable(self):
        """Entry per brick in TOC order: 0 MISSING, 1 CHILD_EMPTY, 2 EMPTY, else slot + 3."""
        n = self.GetInfo().bricks
        out = np.empty(n, dtype=np.uint32)
        check(lib().tvk_pool_get_page_table(self._h, out.ctypes.data_as(N._u32p), n))
        return out

    def Reset(self):
        """Empties the cache but for the coarsest brick (GLVolumePool::PH_Reset)."""
        check(lib().tvk_pool_reset(self._h))

    def SetRequestTable(self, size=0, rehash=10):
        """Missing-brick hash table size (0: the reference's) and probe count."""
        check(lib().tvk_pool_set_request_table(self._h, int(size), int(rehash)))

    def GetRequests(self):
        """TOC indices of the bricks the last pass reported missing (ascending)."""
        n = C.c_size_t()
        check(lib().tvk_pool_get_requests(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.uint64)
        if n.value:
            check(lib().tvk_pool_get_requests(self._h, out.ctypes.data_as(N._u64p), n.value,
                                              C.byref(n)))
        return out.astype(np.int64)

    def Paint(self, renderer, max_passes=32):
        """One GridLeaper frame of ``renderer`` (tvk_leaper_paint); returns LeaperInfo."""
        info = N.LeaperInfo()
        check(lib().tvk_leaper_paint(renderer._h, self._h, int(max_passes), C.byref(info)))
        return info


def read_uvf_blocks(path, verify=False):
    """UVF::Open's container walk (tvk_uvf_read_blocks): the global header as a
    dict and one dict per data block (offset, header_bytes, offset_to_next,
    semantics, compression, id), in file order."""
    flags = N.TVK_UVF_VERIFY_CHECKSUM if verify else 0
    info = N.UvfInfo()
    check(lib().tvk_uvf_read_blocks(str(path).encode(), flags, C.byref(info), None, 0))
    blocks = (N.UvfBlock * max(1, info.block_count))()
    check(lib().tvk_uvf_read_blocks(str(path).encode(), flags, C.byref(info), blocks,
                                    info.block_count))
    head = {k: getattr(info, k) for k, _ in N.UvfInfo._fields_}
    rows = [{"offset": b.offset, "header_bytes": b.header_bytes,
             "offset_to_next": b.offset_to_next, "semantics": b.semantics,
             "compression": b.compression, "id": b.id.decode("latin-1")}
            for b in blocks[:info.block_count]]
    return head, rows


def generate_volume_device(ptr, dims, dtype, blobs, noise_amp, octaves, cell, seed, int_noise,
                           vmax):
    """Fills device memory at ``ptr`` with a seeded blob volume (see tvk.h)."""
    b = np.ascontiguousarray(np.asarray(blobs, dtype=np.float32).reshape(-1))
    dt = N.TVK_U8 if np.dtype(dtype) == np.uint8 else N.TVK_U16
    check(lib().tvk_generate_volume(C.c_void_p(int(ptr)), dt, _u64(dims),
                                    b.ctypes.data_as(N._f32p), b.size // 7, float(noise_amp),
                                    int(octaves), float(cell), int(seed), int(int_noise),
                                    float(vmax)))
