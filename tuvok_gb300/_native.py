"""ctypes binding of libtvk.so (the C ABI declared in include/tvk.h).

The library is built in-tree by ``tuvok_gb300.build``.  There is no fallback:
if the shared library is missing or fails to load, importing this module
raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# TVK_LIBRARY selects another build of the same ABI (the counting diagnostic
# build of tuvok_gb300.profile_counts); by default the in-tree libtvk.so
LIB_PATH = Path(os.environ.get("TVK_LIBRARY") or Path(__file__).resolve().parent / "libtvk.so")

TVK_OK = 0
TVK_U8, TVK_U16, TVK_RGBA8 = 0, 1, 2
TVK_RM_1DTRANS, TVK_RM_2DTRANS, TVK_RM_ISOSURFACE = 0, 1, 2
TVK_LIGHT_REFERENCE, TVK_LIGHT_BLINN_PHONG = 0, 1
TVK_MM_SOURCE, TVK_MM_PRECOMPUTE, TVK_MM_DYNAMIC = 0, 1, 2
TVK_UVF_BS_KEY_VALUE_PAIRS, TVK_UVF_BS_1D_HISTOGRAM, TVK_UVF_BS_2D_HISTOGRAM = 4, 5, 6
TVK_UVF_BS_MAXMIN_VALUES, TVK_UVF_BS_TOC_BLOCK = 7, 9
TVK_UVF_CS_NONE, TVK_UVF_CS_CRC32, TVK_UVF_CS_MD5 = 0, 1, 2
TVK_UVF_VERIFY_CHECKSUM = 256

STATUS_NAMES = {0: "TVK_OK", 1: "TVK_ERR_INVALID_ARG", 2: "TVK_ERR_CUDA",
                3: "TVK_ERR_OUT_OF_MEMORY", 4: "TVK_ERR_UNSUPPORTED", 5: "TVK_ERR_STATE",
                6: "TVK_ERR_INTERNAL"}


class TvkError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class BrickMD(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("extents", C.c_float * 3),
                ("n_voxels", C.c_uint32 * 3)]


class MinMax(C.Structure):
    _fields_ = [("min_scalar", C.c_double), ("max_scalar", C.c_double),
                ("min_gradient", C.c_double), ("max_gradient", C.c_double)]


class VolumeInfo(C.Structure):
    _fields_ = [("dims", C.c_uint64 * 3), ("dtype", C.c_int), ("bit_width", C.c_uint32),
                ("brick_size", C.c_uint32 * 3), ("overlap", C.c_uint32),
                ("lod_count", C.c_uint32), ("lod0_bricks", C.c_uint64),
                ("range_min", C.c_double), ("range_max", C.c_double),
                ("max_gradient", C.c_double), ("device_bytes", C.c_uint64)]


class SubframeInfo(C.Structure):
    _fields_ = [("lod", C.c_uint32), ("decreased_screen_res", C.c_int),
                ("decreased_sampling_rate", C.c_int), ("render_width", C.c_uint32),
                ("render_height", C.c_uint32), ("min_lod", C.c_uint32), ("start_lod", C.c_uint32),
                ("ms", C.c_float), ("frame_complete", C.c_int)]


class BatchInfo(C.Structure):
    _fields_ = [("frames", C.c_uint32), ("tiles", C.c_uint32), ("ctas", C.c_uint32),
                ("ctas_per_sm", C.c_uint32), ("launches", C.c_uint32),
                ("graph_reused", C.c_int), ("autotuned", C.c_int), ("ms", C.c_float),
                ("rays_per_thread", C.c_uint32)]


class CnnConv(C.Structure):
    _fields_ = [("x1", C.c_void_p), ("x2", C.c_void_p), ("c1", C.c_int), ("c2", C.c_int),
                ("n", C.c_int), ("h", C.c_int), ("w", C.c_int), ("weights", C.c_void_p),
                ("bias", C.c_void_p), ("cout", C.c_int), ("slope", C.c_float),
                ("y_bf16", C.c_void_p), ("y_f32", C.c_void_p), ("y2_f32", C.c_void_p),
                ("split", C.c_int), ("accumulate", C.c_int), ("upsample1", C.c_int),
                ("h1", C.c_int), ("w1", C.c_int)]


class CnnWgrad(C.Structure):
    _fields_ = [("x1", C.c_void_p), ("x2", C.c_void_p), ("c1", C.c_int), ("c2", C.c_int),
                ("gy", C.c_void_p), ("n", C.c_int), ("h", C.c_int), ("w", C.c_int),
                ("cout", C.c_int), ("dw", C.c_void_p), ("db", C.c_void_p)]


class LearnedInfo(C.Structure):
    _fields_ = [("probe_psnr_db", C.c_float), ("fell_back", C.c_int), ("ms_reduced", C.c_float),
                ("ms_network", C.c_float), ("ms_probe", C.c_float), ("ms_fallback", C.c_float),
                ("reduced_width", C.c_uint32), ("reduced_height", C.c_uint32),
                ("ms_judge", C.c_float), ("ms_frame", C.c_float)]


class PoolInfo(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("slot_bytes", C.c_uint64), ("bricks", C.c_uint64),
                ("hash_size", C.c_uint32), ("host_source", C.c_int),
                ("paged_total", C.c_uint64)]


class LeaperInfo(C.Structure):
    _fields_ = [("passes", C.c_uint32), ("paged", C.c_uint32), ("missing_last", C.c_uint32),
                ("converged", C.c_int), ("resident", C.c_uint32), ("ms", C.c_float),
                ("ms_traversal", C.c_float), ("bytes_paged", C.c_uint64),
                ("samples", C.c_uint64), ("ms_host", C.c_float)]


class UvfBlock(C.Structure):
    _fields_ = [("offset", C.c_uint64), ("header_bytes", C.c_uint64),
                ("offset_to_next", C.c_uint64), ("semantics", C.c_uint64),
                ("compression", C.c_uint64), ("id", C.c_char * 64)]


class UvfInfo(C.Structure):
    _fields_ = [("file_version", C.c_uint64), ("checksum_semantics", C.c_uint64),
                ("checksum_bytes", C.c_uint64), ("data_offset", C.c_uint64),
                ("file_bytes", C.c_uint64), ("big_endian", C.c_uint32),
                ("block_count", C.c_uint32), ("timestep_count", C.c_uint32),
                ("checksum_verified", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("shaded_samples", C.c_uint64),
                ("bricks_visible", C.c_uint64), ("bricks_total", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("last_paint_ms", C.c_float),
                ("gradient_samples", C.c_uint64)]


_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)
_vp = C.c_void_p

# name -> argtypes (every function returns tvk_status unless listed in _RET)
PROTOTYPES = {
    "tvk_status_string": [C.c_int],
    "tvk_last_error": [],
    "tvk_abi_version": [],
    "tvk_volume_create": [_vp, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int, C.POINTER(_vp)],
    "tvk_volume_create_device": [_vp, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int, C.POINTER(_vp)],
    "tvk_volume_create_ex": [_vp, C.c_int, _u64p, _u32p, C.c_uint32, C.c_uint32, C.POINTER(_vp)],
    "tvk_volume_destroy": [_vp],
    "tvk_volume_get_info": [_vp, C.POINTER(VolumeInfo)],
    "tvk_volume_get_lod": [_vp, C.c_uint32, _u64p, _u64p],
    "tvk_volume_get_brick_md": [_vp, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(BrickMD)],
    "tvk_volume_get_brick": [_vp, C.c_uint64, C.c_uint64, C.c_uint64, _vp, C.c_size_t],
    "tvk_volume_get_minmax": [_vp, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(MinMax)],
    "tvk_volume_get_histogram": [_vp, _u64p, C.c_size_t, _u64p],
    "tvk_volume_get_histogram2d": [_vp, _u64p, C.c_size_t, C.c_size_t, _u64p, _f32p],
    "tvk_volume_get_brick_histograms": [_vp, _u32p, C.c_size_t, _u32p],
    "tvk_volume_rebrick": [_vp, _u32p, C.c_int, C.POINTER(_vp)],
    "tvk_volume_get_max_used_brick_size": [_vp, _u32p],
    "tvk_volume_index_from_4d": [_vp, _u64p, _u64p],
    "tvk_volume_index_to_4d": [_vp, C.c_uint64, C.c_uint64, _u64p],
    "tvk_renderer_create": [C.POINTER(_vp)],
    "tvk_renderer_destroy": [_vp],
    "tvk_renderer_set_volume": [_vp, _vp],
    "tvk_set_tf1d_rgba8": [_vp, C.POINTER(C.c_uint8), C.c_uint32],
    "tvk_set_tf1d_float": [_vp, _f32p, C.c_uint32, C.c_int],
    "tvk_set_tf2d_float": [_vp, _f32p, C.c_uint32, C.c_uint32, C.c_int],
    "tvk_tf1d_set_std_function": [_f32p, C.c_uint64, C.c_float, C.c_float, C.c_int, C.c_int],
    "tvk_tf1d_from_bytes": [C.POINTER(C.c_uint8), C.c_uint64, _f32p],
    "tvk_tf1d_resample": [_f32p, C.c_uint64, _f32p, C.c_uint64],
    "tvk_tf1d_fill_or_truncate": [_f32p, C.c_uint64, _f32p, C.c_uint64],
    "tvk_tf1d_nonzero_limits": [_f32p, C.c_uint64, _u64p],
    "tvk_tf1d_byte_array": [_f32p, C.c_uint64, C.c_uint8, C.POINTER(C.c_uint8)],
    "tvk_tf1d_short_array": [_f32p, C.c_uint64, C.c_uint16, C.POINTER(C.c_uint16)],
    "tvk_tf1d_load": [C.c_char_p, _f32p, C.c_uint64, _u64p],
    "tvk_tf1d_save": [C.c_char_p, _f32p, C.c_uint64],
    "tvk_set_render_mode": [_vp, C.c_int],
    "tvk_set_lighting": [_vp, C.c_int],
    "tvk_set_sample_rate_modifier": [_vp, C.c_float],
    "tvk_set_isovalue": [_vp, C.c_float],
    "tvk_set_colors": [_vp, _f32p, _f32p, _f32p, _f32p],
    "tvk_set_iso_color": [_vp, _f32p],
    "tvk_set_light_model": [_vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float],
    "tvk_set_view": [_vp, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_float],
    "tvk_set_model_transform": [_vp, _f32p, _f32p],
    "tvk_resize": [_vp, C.c_uint32, C.c_uint32],
    "tvk_set_frame_termination": [_vp, C.c_float],
    "tvk_paint": [_vp],
    "tvk_set_lod": [_vp, C.c_uint32],
    "tvk_set_reduced_quality": [_vp, C.c_int, C.c_int],
    "tvk_set_perf_measures": [_vp, C.c_uint32, C.c_int, C.c_float, C.c_float],
    "tvk_set_lod_limits": [_vp, C.c_uint32, C.c_uint32],
    "tvk_set_capture_mode": [_vp, C.c_int],
    "tvk_compute_min_lod": [_vp, _u32p],
    "tvk_paint_progressive": [_vp, C.c_int, C.POINTER(SubframeInfo)],
    "tvk_get_render_size": [_vp, _u32p, _u32p],
    "tvk_cnn_conv3x3": [C.POINTER(CnnConv), _vp],
    "tvk_cnn_check": [_vp],
    "tvk_cnn_conv3x3_wgrad": [C.POINTER(CnnWgrad), _vp],
    "tvk_cnn_act_grad": [_vp, _vp, C.c_float, _vp, C.c_size_t, _vp],
    "tvk_cnn_avgpool2": [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_cnn_avgpool2_backward": [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int, _vp],
    "tvk_cnn_upsample2": [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_cnn_upsample2_backward": [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_cnn_head": [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_cnn_head_backward": [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_cnn_mse": [_vp, _vp, C.c_size_t, _vp, _vp, _vp],
    "tvk_cnn_adam": [_vp, _vp, _vp, _vp, C.c_size_t, C.c_float, C.c_float, C.c_float, C.c_float,
                     C.c_int, _vp],
    "tvk_cnn_weights_bf16": [_vp, C.c_int, C.c_int, _vp, _vp, _vp],
    "tvk_cnn_to_bf16": [_vp, C.c_size_t, _vp, _vp],
    "tvk_cnn_prepare_input": [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "tvk_set_clip_plane": [_vp, _f32p],
    "tvk_enable_clip_plane": [_vp, C.c_int],
    "tvk_set_scaling_method": [_vp, C.c_int],
    "tvk_volume_open_extended_octree": [C.c_char_p, C.c_uint64, C.c_uint32, C.c_uint32,
                                        C.POINTER(_vp)],
    "tvk_eo_read_brick": [C.c_char_p, C.c_uint64, C.c_uint32, C.c_uint64, _vp, C.c_size_t,
                          C.POINTER(C.c_size_t)],
    "tvk_uvf_read_blocks": [C.c_char_p, C.c_uint32, C.POINTER(UvfInfo), C.POINTER(UvfBlock),
                            C.c_uint32],
    "tvk_volume_open_uvf": [C.c_char_p, C.c_uint32, C.c_uint32, C.POINTER(_vp)],
    "tvk_set_clearview": [_vp, C.c_int],
    "tvk_set_cv_isovalue": [_vp, C.c_float],
    "tvk_set_cv_color": [_vp, _f32p],
    "tvk_set_cv_params": [_vp, C.c_float, C.c_float, C.c_float],
    "tvk_set_cv_focus_pos": [_vp, _f32p],
    "tvk_get_cv_focus_pos": [_vp, _f32p],
    "tvk_set_cv_focus_pixel": [_vp, C.c_uint32, C.c_uint32],
    "tvk_set_depth_output": [_vp, C.c_int],
    "tvk_copy_depth_device": [_vp, _vp, C.c_size_t],
    "tvk_learned_param_count": [C.POINTER(C.c_size_t)],
    "tvk_learned_create": [_f32p, C.c_size_t, C.POINTER(_vp)],
    "tvk_learned_destroy": [_vp],
    "tvk_paint_learned": [_vp, _vp, C.c_float, C.POINTER(LearnedInfo)],
    "tvk_copy_image_device": [_vp, C.c_int, _vp, C.c_size_t],
    "tvk_batch_create": [C.POINTER(_vp)],
    "tvk_batch_destroy": [_vp],
    "tvk_paint_batch": [_vp, C.POINTER(_vp), C.c_uint32],
    "tvk_batch_set_autotune": [_vp, C.c_int, C.c_uint32],
    "tvk_batch_set_rays_per_thread": [_vp, C.c_uint32],
    "tvk_batch_get_info": [_vp, C.POINTER(BatchInfo)],
    "tvk_volume_release_bricks": [_vp],
    "tvk_pool_create": [_vp, C.c_uint64, C.c_int, C.POINTER(_vp)],
    "tvk_pool_destroy": [_vp],
    "tvk_pool_get_info": [_vp, C.POINTER(PoolInfo)],
    "tvk_pool_get_page_table": [_vp, _u32p, C.c_size_t],
    "tvk_pool_get_requests": [_vp, _u64p, C.c_size_t, C.POINTER(C.c_size_t)],
    "tvk_pool_set_request_table": [_vp, C.c_uint32, C.c_uint32],
    "tvk_pool_reset": [_vp],
    "tvk_leaper_paint": [_vp, _vp, C.c_uint32, C.POINTER(LeaperInfo)],
    "tvk_get_image_device": [_vp, C.POINTER(_vp), _u32p, _u32p],
    "tvk_read_image": [_vp, _f32p, C.c_size_t],
    "tvk_read_image_async": [_vp, _f32p, C.c_size_t],
    "tvk_wait_image": [_vp],
    "tvk_read_sample_counts": [_vp, _u32p, C.c_size_t],
    "tvk_renderer_get_stream": [_vp, C.POINTER(_vp)],
    "tvk_get_stats": [_vp, C.POINTER(Stats)],
    "tvk_get_counters": [_vp, _u64p],
    "tvk_volume_cell_minmax": [_vp, C.c_uint64, _u32p, C.c_uint64, _u32p],
    "tvk_set_hardware_filtering": [_vp, C.c_int],
    "tvk_generate_volume": [_vp, C.c_int, _u64p, _f32p, C.c_uint32, C.c_float, C.c_uint32,
                            C.c_float, C.c_uint64, C.c_int, C.c_float],
    "tvk_brick_lod0_noalloc": [_vp, C.c_int, _u64p, _u32p, C.c_uint32, C.c_int, _u64p,
                               C.c_uint32, C.c_uint32, _vp, C.c_size_t, _vp, _vp, _vp],
}
_RET = {"tvk_status_string": C.c_char_p, "tvk_last_error": C.c_char_p,
        "tvk_abi_version": C.c_int}

_lib = None


def lib():
    """Loads libtvk.so once; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, args in PROTOTYPES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RET.get(name, C.c_int)
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != TVK_OK:
        msg = lib().tvk_last_error().decode(errors="replace")
        raise TvkError(status, msg)
