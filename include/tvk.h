/*
 * tvk.h -- C ABI of tuvok_gb300, a GB300 (sm_103a) implementation of Tuvok's
 * volume-rendering hot path: LOD-0 bricking with ghost voxels, per-brick
 * min/max and histograms, and the brick-by-brick GLRaycaster ray march
 * (1D/2D transfer functions, central-difference lighting, front-to-back
 * compositing with early ray termination, brick-level empty-space skipping).
 *
 * Conventions
 *  - Every entry point returns tvk_status; no C++ exception crosses the ABI.
 *    tvk_last_error() returns a message for the calling thread's last failure.
 *  - One host thread drives one renderer handle.  Each renderer owns one CUDA
 *    stream; all device work of a call is ordered on it.
 *  - Volumes hold their bricks in device memory (HBM); renderers share volumes
 *    read-only.  A volume must outlive the renderers it is attached to.
 *  - Images are RGBA float32, premultiplied colour, row 0 = bottom row
 *    (OpenGL window convention), width*height*4 floats.
 *  - Brick keys are Tuvok's (timestep, lod, 1D index = x + y*bx + z*bx*by).
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the Tuvok source tree).
 */
#ifndef TVK_H
#define TVK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TVK_ABI_VERSION 1

typedef enum tvk_status {
  TVK_OK = 0,
  TVK_ERR_INVALID_ARG = 1,   /* bad pointer, size, key or mode */
  TVK_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  TVK_ERR_OUT_OF_MEMORY = 3, /* device or pinned allocation failed */
  TVK_ERR_UNSUPPORTED = 4,   /* valid request this build does not handle */
  TVK_ERR_STATE = 5,         /* call order: e.g. paint without volume or TF */
  TVK_ERR_INTERNAL = 6
} tvk_status;

/* Voxel types.  TVK_RGBA8: colour volumes, four unsigned 8-bit channels per
 * voxel, x fastest (Dataset::GetComponentCount() == 4, AbstrRenderer::
 * ColorData).  Colour volumes get every LOD, each channel filtered on its own
 * (ExtendedOctreeConverter.inc:39-44), and no statistics
 * (AbstrRenderer::ContainsData never skips colour bricks); they render in 1D
 * mode (the voxel's colour times the TF entry at (r + g + b) / 3,
 * VRender1D-Color.glsl / VRender1DLit-Color.glsl) and iso mode (the alpha
 * channel's isosurface with its colour, GLRaycaster-Color-FS.glsl and
 * Compose-Color-FS.glsl).  A GridLeaper pool over a colour volume renders
 * every mode of GLGridLeaper-Method-*-color.glsl (1D and 2D, lit or not, iso),
 * with every brick's value range taken as [0, 255].  The brick-by-brick 2D
 * mode, ClearView, batches, rebricking, hardware filtering and the histograms
 * refuse them. */
typedef enum tvk_dtype { TVK_U8 = 0, TVK_U16 = 1, TVK_RGBA8 = 2 } tvk_dtype;

/* AbstrRenderer::ERenderMode (Renderer/AbstrRenderer.h:120-126) */
typedef enum tvk_render_mode {
  TVK_RM_1DTRANS = 0,
  TVK_RM_2DTRANS = 1,
  TVK_RM_ISOSURFACE = 2
} tvk_render_mode;

/* Lighting models: the reference model of Shaders/lighting.glsl:33-43 and a
 * selectable Blinn-Phong (ka, kd, ks, shininess). */
typedef enum tvk_light_model {
  TVK_LIGHT_REFERENCE = 0,
  TVK_LIGHT_BLINN_PHONG = 1
} tvk_light_model;

/* AbstrRenderer::ScalingMethod (Renderer/AbstrRenderer.h:156-159): how a
 * 1D-mode sample maps to a TF coordinate.  SMETH_BIT_WIDTH: value * fTransScale
 * with CalculateScaling (GLRenderer.cpp:1813-1819).  SMETH_BIAS_AND_SCALE
 * (MasterController::RequestNewVolumeRenderer's bBiasAndScaleTF): GLRaycaster
 * uploads TFuncBias = -min and fTransScale = |min| + |max| of the data range
 * (TFScaling.cpp scale_bias_and_scale, GLRaycaster.cpp:577-584), but its 1D
 * shaders never receive a ScaleMethod other than 0 (the setter is commented
 * out, GLRenderer.cpp:1820-1833), so the bias goes unused and the coordinate is
 * value * (|min| + |max|).  That is what this renderer computes; 2D and iso
 * modes and the GridLeaper are unaffected. */
typedef enum tvk_scaling_method {
  TVK_SCALE_BIT_WIDTH = 0,
  TVK_SCALE_BIAS_AND_SCALE = 1
} tvk_scaling_method;

typedef struct tvk_volume tvk_volume;
typedef struct tvk_renderer tvk_renderer;

/* BrickMD (IO/Brick.h:58-62): centre and extents in model space (volume
 * normalised to max extent 1, centred at 0) and voxel counts incl. ghost. */
typedef struct tvk_brick_md {
  float center[3];
  float extents[3];
  uint32_t n_voxels[3];
} tvk_brick_md;

/* MinMaxBlock (Basics/MinMaxBlock.h:10-38) */
typedef struct tvk_minmax {
  double min_scalar, max_scalar, min_gradient, max_gradient;
} tvk_minmax;

typedef struct tvk_volume_info {
  uint64_t dims[3];
  tvk_dtype dtype;
  uint32_t bit_width;        /* Dataset::GetBitWidth: 8 or 16 */
  uint32_t brick_size[3];    /* incl. overlap, as Tuvok counts it */
  uint32_t overlap;
  uint32_t lod_count;        /* ExtendedOctree LOD table length */
  uint64_t lod0_bricks;      /* bricks resident on the device (LOD 0) */
  double range_min, range_max;   /* Dataset::GetRange */
  double max_gradient;       /* Dataset::MaxGradientMagnitude */
  uint64_t device_bytes;     /* brick pool + metadata held in HBM */
} tvk_volume_info;

/* Per-frame statistics of the last paint. */
typedef struct tvk_stats {
  uint64_t samples;          /* ray-march steps the reference loop executes */
  uint64_t shaded_samples;   /* of those, steps whose voxels were fetched */
  uint64_t bricks_visible;   /* LOD-0 bricks passing ContainsData */
  uint64_t bricks_total;
  uint64_t kernel_launches;  /* kernels this library launched for the frame */
  float last_paint_ms;       /* device time of the last paint (CUDA events) */
  uint64_t gradient_samples; /* shaded steps that also took the 6 gradient lookups */
} tvk_stats;

/* ---------------------------------------------------------------- misc */

const char* tvk_status_string(tvk_status s);
/* Message of the calling thread's last failing call ("" if none). */
const char* tvk_last_error(void);
int tvk_abi_version(void);

/* ---------------------------------------------------------------- volumes */

/* Bricks a flat volume (x fastest) on the GPU: LOD-0 bricks with `overlap`
 * ghost voxels per side, zero or clamp-to-edge borders, per-brick min/max
 * over the whole brick, the global 1D histogram of inner voxels, a 256-bin
 * histogram per brick and the maximum gradient magnitude.
 * Replaces ExtendedOctreeConverter::Convert's LOD-0 stage
 * (IO/UVF/ExtendedOctree/ExtendedOctreeConverter.cpp:128-280, GetInputBrick
 * :288-373, ClampToEdge :376-462, ComputeBrickStats .inc:408-444),
 * Histogram1DDataBlock::ComputeTemplate (IO/UVF/Histogram1DDataBlock.cpp:120-161)
 * and the max-gradient pass of Histogram2DDataBlock (:349-397).
 * `voxels` is host memory (copied in) for tvk_volume_create and device memory
 * for tvk_volume_create_device.  brick_size includes the overlap. */
tvk_status tvk_volume_create(const void* voxels, tvk_dtype dtype, const uint64_t dims[3],
                             const uint32_t brick_size[3], uint32_t overlap,
                             int clamp_to_edge, tvk_volume** out);
tvk_status tvk_volume_create_device(const void* device_voxels, tvk_dtype dtype,
                                    const uint64_t dims[3], const uint32_t brick_size[3],
                                    uint32_t overlap, int clamp_to_edge, tvk_volume** out);
/* Flags of tvk_volume_create_ex. */
enum {
  TVK_VOLUME_CLAMP_TO_EDGE = 1, /* replicate border voxels into the ghost layer */
  TVK_VOLUME_DEVICE_INPUT = 2,  /* `voxels` is device memory */
  TVK_VOLUME_MEDIAN = 4,        /* coarser LODs by the 7-value median, not the mean */
  TVK_VOLUME_LOD0_ONLY = 8      /* skip the coarser LODs */
};
/* As tvk_volume_create, with every LOD of ExtendedOctreeConverter::Convert:
 * LOD >= 1 bricks come from ComputeHierarchy / DownsampleBrick
 * (ExtendedOctreeConverter.inc:1-398) and FillOverlap (.cpp:1203-1372), and
 * get min/max statistics.  tvk_volume_create and _create_device build every
 * LOD with the mean filter. */
tvk_status tvk_volume_create_ex(const void* voxels, tvk_dtype dtype, const uint64_t dims[3],
                                const uint32_t brick_size[3], uint32_t overlap, uint32_t flags,
                                tvk_volume** out);
/* Opens the ExtendedOctree brick container that Tuvok's converter writes
 * (ExtendedOctreeConverter::Convert) and a UVF file's TOC block holds, at byte
 * `offset` of `path` (ExtendedOctree::Open, IO/UVF/ExtendedOctree/
 * ExtendedOctree.cpp:67-172; headers of UVF version >= 5).  Bricks are read at
 * their table-of-contents offsets in any on-disk layout (scanline, Morton,
 * Hilbert, random) and expanded where stored compressed (GetBrickData,
 * :313-361): zlib, LZMA, LZ4 and bzip2 bricks are decoded (CT_LZHAM is
 * refused, as by the reference).
 * 1-component uint8 / uint16 and 4-component uint8 (TVK_RGBA8) volumes with a
 * 1:1:1 aspect.  The volume is rebuilt on the GPU from the LOD-0 bricks' inner
 * voxels (statistics, histograms, coarser LODs).  The header records neither
 * the border fill nor the LOD filter, so the rebuild starts from `flags`
 * (TVK_VOLUME_CLAMP_TO_EDGE, TVK_VOLUME_MEDIAN, TVK_VOLUME_LOD0_ONLY) and tries
 * the others: the LOD-0 bricks must equal the file's byte for byte (else
 * TVK_ERR_INVALID_ARG), and coarser bricks that no filter reproduces are taken
 * from the file with their min/max recomputed (the converter fills some
 * ghost voxels of coarser bricks before their neighbours are written, so they
 * can keep stale buffer data). */
/* ExtendedOctree::GetBrickData (ExtendedOctree.cpp:313-361) on the host, no
 * GPU involved: brick `index` (table-of-contents order: LODs finest first,
 * x fastest) of the ExtendedOctree at byte `offset` of `path`, expanded from
 * its stored form (uncompressed, zlib, LZMA, LZ4 or bzip2) into `out`, voxels
 * x fastest with the ghost layers.  *n_bytes receives the brick's size; with
 * out == NULL only the size is returned, otherwise capacity must hold it.
 * Corrupt or truncated bricks return TVK_ERR_INVALID_ARG. */
tvk_status tvk_eo_read_brick(const char* path, uint64_t offset, uint32_t uvf_version,
                             uint64_t index, void* out, size_t capacity, size_t* n_bytes);
tvk_status tvk_volume_open_extended_octree(const char* path, uint64_t offset,
                                           uint32_t uvf_version, uint32_t flags,
                                           tvk_volume** out);

/* UVF container (IO/UVF/UVF.cpp:140-158 ParseGlobalHeader, :269-291
 * ParseDataBlocks; GlobalHeader.cpp:37-46; DataBlock.cpp:51-75): the
 * "UVF-DATA" magic, a one-byte big-endian flag, the file version, checksum
 * semantics and bytes, then a chain of data blocks, each an id string, its
 * semantics (UVFTables::BlockSemanticTable), compression and the distance to
 * the next block (0 on the last).  Every value is in the writer's byte order,
 * little-endian, whatever the big-endian flag says: the reference's byte swap
 * (LargeRAWFile::ReadData / WriteData over EndianConvert::Swap, which returns
 * the swapped value and leaves its argument unchanged) never swaps, and this
 * reader does as it does. */
enum {
  TVK_UVF_BS_KEY_VALUE_PAIRS = 4,
  TVK_UVF_BS_1D_HISTOGRAM = 5,
  TVK_UVF_BS_2D_HISTOGRAM = 6,
  TVK_UVF_BS_MAXMIN_VALUES = 7,
  TVK_UVF_BS_TOC_BLOCK = 9,
  TVK_UVF_CS_NONE = 0,
  TVK_UVF_CS_CRC32 = 1,
  TVK_UVF_CS_MD5 = 2,
  /* flag of tvk_uvf_read_blocks and tvk_volume_open_uvf: check the stored
   * MD5 checksum first (UVF::VerifyChecksum, UVF.cpp:232-266; TVK_ERR_INVALID_ARG
   * on a mismatch).  CRC32 checksums are not checked (TVK_ERR_UNSUPPORTED): the
   * reference's CRC32 pass runs over bytes past the end of the file
   * (UVF.cpp:174-198), so a stored CRC32 cannot be reproduced. */
  TVK_UVF_VERIFY_CHECKSUM = 256
};
typedef struct tvk_uvf_block {
  uint64_t offset;         /* file offset of the block header */
  uint64_t header_bytes;   /* 32 + id length: the payload starts at offset + header_bytes */
  uint64_t offset_to_next; /* 0 on the last block */
  uint64_t semantics;      /* UVFTables::BlockSemanticTable */
  uint64_t compression;    /* UVFTables::CompressionSemanticTable */
  char id[64];             /* the block id, truncated, NUL-terminated */
} tvk_uvf_block;
typedef struct tvk_uvf_info {
  uint64_t file_version;       /* GlobalHeader::ulFileVersion */
  uint64_t checksum_semantics; /* TVK_UVF_CS_* */
  uint64_t checksum_bytes;
  uint64_t data_offset;        /* GlobalHeader::GetDataPos: the first block */
  uint64_t file_bytes;
  uint32_t big_endian;         /* the header's flag (recorded, see above) */
  uint32_t block_count;
  /* TOC blocks that UVFDataset::VerifyTOCBlock accepts (1- or 4-component
   * volumes, uvfDataset.cpp:527-542): the dataset's timesteps, in file order */
  uint32_t timestep_count;
  uint32_t checksum_verified;  /* 1 when TVK_UVF_VERIFY_CHECKSUM checked an MD5 */
} tvk_uvf_info;
/* Host only, no GPU: walks the container of `path` and fills *info and up to
 * `capacity` entries of `blocks` (NULL with capacity 0 counts them).  A file
 * that is not UVF, is truncated, or whose block chain leaves the file returns
 * TVK_ERR_INVALID_ARG. */
tvk_status tvk_uvf_read_blocks(const char* path, uint32_t flags, tvk_uvf_info* info,
                               tvk_uvf_block* blocks, uint32_t capacity);
/* UVFDataset::Open for a TOC-block dataset (IO/uvfDataset.cpp:83-216): the
 * volume of timestep `timestep` (the timestep-th TOC block accepted as above),
 * opened as tvk_volume_open_extended_octree opens the ExtendedOctree at the
 * block's payload (TOCBlock::GetHeaderFromFile, TOCBlock.cpp:48-65) with the
 * file's UVF version; `flags` are that call's, plus TVK_UVF_VERIFY_CHECKSUM.
 * Files whose volumes are RasterDataBlocks (UVF before TOC blocks) return
 * TVK_ERR_UNSUPPORTED. */
tvk_status tvk_volume_open_uvf(const char* path, uint32_t timestep, uint32_t flags,
                               tvk_volume** out);
tvk_status tvk_volume_destroy(tvk_volume* v);
tvk_status tvk_volume_get_info(const tvk_volume* v, tvk_volume_info* out);

/* ExtendedOctree::GetLoDSize / GetBrickCount (ExtendedOctree.cpp:241-262). */
tvk_status tvk_volume_get_lod(const tvk_volume* v, uint32_t lod, uint64_t size[3],
                              uint64_t brick_count[3]);

/* BrickedDataset::GetBrickMetadata (IO/BrickedDataset.h:62) for any built LOD;
 * values follow UVFDataset::ComputeMetadataTOC (IO/uvfDataset.cpp:242-288). */
tvk_status tvk_volume_get_brick_md(const tvk_volume* v, uint64_t timestep, uint64_t lod,
                                   uint64_t index, tvk_brick_md* out);

/* MaxMinForKey modes of a rebricked volume (DynamicBrickingDS::MinMaxMode,
 * IO/DynamicBrickingDS.h): the source brick's statistics, or the min/max of
 * the target brick's own voxels (ghost included; computed when rebricking for
 * both PRECOMPUTE and DYNAMIC, which give the same values). */
typedef enum {
  TVK_MM_SOURCE = 0,
  TVK_MM_PRECOMPUTE = 1,
  TVK_MM_DYNAMIC = 2
} tvk_minmax_mode;

/* DynamicBrickingDS::DynamicBrickingDS + Rebrick (IO/DynamicBrickingDS.cpp:133-139,
 * 1090-1180): a new volume whose bricks of brick_size voxels (ghost included)
 * are windows of src's bricks, gathered on the GPU for every built LOD.  Each
 * axis' brick_size - 2*overlap must divide the source's inner brick size
 * (TVK_ERR_INVALID_ARG "x dimension is not an integer multiple of original
 * brick size." where the reference throws std::runtime_error).  The result
 * answers the dataset queries (get_info: brick_size = GetMaxBrickSize; get_lod,
 * get_brick_md, get_brick, get_minmax per minmax_mode, index_*); histograms are
 * the source's (forwarded, as in the reference) and it is not renderable
 * (TVK_ERR_UNSUPPORTED).  The source may be destroyed afterwards. */
tvk_status tvk_volume_rebrick(const tvk_volume* src, const uint32_t brick_size[3], int minmax_mode,
                              tvk_volume** out);

/* BrickedDataset::GetMaxUsedBrickSizes (IO/BrickedDataset.cpp:139-145): the
 * largest n_voxels per axis over every brick. */
tvk_status tvk_volume_get_max_used_brick_size(const tvk_volume* v, uint32_t out[3]);

/* Dataset::GetBrick(key, std::vector<T>&) (IO/Dataset.h:93-100): copies one
 * brick (x fastest, ghost included) to host memory of `bytes` bytes. */
tvk_status tvk_volume_get_brick(const tvk_volume* v, uint64_t timestep, uint64_t lod,
                                uint64_t index, void* host_out, size_t bytes);

/* Frees the volume's device brick pool, keeping its metadata: the out-of-core
 * set-up, where a GridLeaper pool created with host_source = 1 (which holds a
 * pinned host copy of the bricks) is the only renderer of the volume, as
 * GPUMemMan::GetVolumePool keeps only the cache on the GPU (GPUMemMan.cpp:
 * 766-844).  Everything that reads the device bricks afterwards (tvk_paint,
 * tvk_volume_get_brick, rebricking, device-sourced pools) fails with
 * TVK_ERR_STATE.  Blocks until the device is idle. */
tvk_status tvk_volume_release_bricks(tvk_volume* v);

/* BrickedDataset::MaxMinForKey (IO/BrickedDataset.h:73). */
tvk_status tvk_volume_get_minmax(const tvk_volume* v, uint64_t timestep, uint64_t lod,
                                 uint64_t index, tvk_minmax* out);

/* Global histogram, 2^(8*bytes) bins (Histogram1DDataBlock::GetHistogram);
 * *trimmed_len = last non-zero bin + 1.  `bins` may exceed 2^(8*bytes). */
tvk_status tvk_volume_get_histogram(const tvk_volume* v, uint64_t* host_out, size_t bins,
                                    uint64_t* trimmed_len);

/* Value x |gradient| histogram of the LOD-0 inner voxels, computed on the GPU
 * on each call: Histogram2DDataBlock::Compute / ComputeTemplate
 * (IO/UVF/Histogram2DDataBlock.cpp:69-126, 349-438) with the arguments
 * RAWConverter passes (IO/RAWConverter.cpp:655-662).  host_out receives
 * value_bins rows of 256 gradient bins (entries >= value_bins * 256);
 * value_bins = 0 uses the trimmed 1D histogram's length.  The value bin is the
 * raw value, or value * (value_bins - 1) / range_max when range_max exceeds
 * value_bins - 1; the gradient bin is min(255, |g| / max|g| * 255).  A
 * constant volume (max|g| = 0) puts every voxel in gradient bin 0.
 * *max_gradient = Histogram2DDataBlock::GetMaxGradMagnitude (a float).
 * TVK_ERR_UNSUPPORTED for overlap 0 (the reference reads outside the brick). */
tvk_status tvk_volume_get_histogram2d(const tvk_volume* v, uint64_t* host_out, size_t value_bins,
                                      size_t entries, uint64_t* value_bins_used,
                                      float* max_gradient);

/* 256-bin histograms of every LOD-0 brick's inner voxels, brick-major
 * (new: the reference stores only the global histogram); bin = value >> shift
 * with shift = max(0, bits(range_max) - 8). */
tvk_status tvk_volume_get_brick_histograms(const tvk_volume* v, uint32_t* host_out,
                                           size_t n_bricks, uint32_t* shift);

/* LinearIndexDataset::IndexFrom4D / IndexTo4D (IO/LinearIndexDataset.cpp:7-39). */
tvk_status tvk_volume_index_from_4d(const tvk_volume* v, const uint64_t xyzl[4],
                                    uint64_t* index);
tvk_status tvk_volume_index_to_4d(const tvk_volume* v, uint64_t lod, uint64_t index,
                                  uint64_t xyzl[4]);

/* ---------------------------------------------------------------- renderer */

/* MasterController::RequestNewVolumeRenderer (Controller/MasterController.cpp:145-200)
 * for the GLRaycaster type.  Defaults follow AbstrRenderer's constructor
 * (Renderer/AbstrRenderer.cpp:64-170): FOV 50, near 0.01, far 1000, eye
 * (0,0,1.6), sample-rate modifier 1, 1D TF mode, no lighting. */
tvk_status tvk_renderer_create(tvk_renderer** out);
tvk_status tvk_renderer_destroy(tvk_renderer* r);

/* AbstrRenderer::RegisterDataset / LoadDataset (Renderer/AbstrRenderer.h:460). */
tvk_status tvk_renderer_set_volume(tvk_renderer* r, const tvk_volume* v);

/* AbstrRenderer::Set1DTrans + Changed1DTrans (AbstrRenderer.h:189-195) with
 * TransferFunction1D::Set's byte semantics (IO/TransferFunction1D.cpp:146-177):
 * colour channels are stretched to [0,1] by their min/max, alpha is byte/255;
 * the table is then uploaded as GL_RGBA8 (GetByteArray, :311-330). */
tvk_status tvk_set_tf1d_rgba8(tvk_renderer* r, const uint8_t* rgba, uint32_t n);
/* Float RGBA table.  rgba8_upload != 0 reproduces the GL_RGBA8 upload
 * (clamp, x255, truncate); 0 keeps FP32 entries. */
tvk_status tvk_set_tf1d_float(tvk_renderer* r, const float* rgba, uint32_t n, int rgba8_upload);

/* ---- TransferFunction1D (IO/TransferFunction1D.h:53-101) on a caller-held
 * table of n entries of 4 floats (RGBA), host only.  Each function gives the
 * reference method's table bit for bit; none touches the GPU.  The renderer
 * takes the table through tvk_set_tf1d_float. */

/* TransferFunction1D::SetStdFunction (TransferFunction1D.cpp:74-113): a
 * smoothstep ramp centred on center * (n - 1) entries, inv_gradient * (n - 1)
 * entries wide (both clamped to [0, 1]), 0 before and 1 after (reversed when
 * inverted).  component 0..3 sets one channel (the 4-argument overload);
 * -1 sets all four, not inverted (the 2-argument overload, defaults 0.5 and
 * 0.5). */
tvk_status tvk_tf1d_set_std_function(float* rgba, uint64_t n, float center, float inv_gradient,
                                     int component, int inverted);
/* TransferFunction1D::Set (TransferFunction1D.cpp:146-177): n RGBA bytes to
 * floats, colour channels stretched by the per-channel min/max that
 * minmax_component4 finds (:115-144: every channel's range starts from the
 * table's first byte), alpha = byte / 255. */
tvk_status tvk_tf1d_from_bytes(const uint8_t* rgba8, uint64_t n, float* rgba);
/* TransferFunction1D::Resample (TransferFunction1D.cpp:198-238): box average
 * down, linear interpolation up.  dst may equal src only when n_dst == n_src. */
tvk_status tvk_tf1d_resample(const float* src, uint64_t n_src, float* dst, uint64_t n_dst);
/* TransferFunction1D::FillOrTruncate (TransferFunction1D.cpp:188-197). */
tvk_status tvk_tf1d_fill_or_truncate(const float* src, uint64_t n_src, float* dst,
                                     uint64_t n_dst);
/* TransferFunction1D::ComputeNonZeroLimits / GetNonZeroLimits
 * (TransferFunction1D.cpp:362-371): limits = {first, last} entry with a
 * non-zero alpha, {n, 0} when every alpha is 0. */
tvk_status tvk_tf1d_nonzero_limits(const float* rgba, uint64_t n, uint64_t limits[2]);
/* TransferFunction1D::GetByteArray / GetShortArray (TransferFunction1D.cpp:
 * 311-351): each channel clamped to [0, 1], times used_range, truncated;
 * out holds 4 * n values. */
tvk_status tvk_tf1d_byte_array(const float* rgba, uint64_t n, uint8_t used_range, uint8_t* out);
tvk_status tvk_tf1d_short_array(const float* rgba, uint64_t n, uint16_t used_range,
                                uint16_t* out);
/* TransferFunction1D::Load / Save (TransferFunction1D.cpp:240-306): the text
 * format (entry count, then 4 numbers per entry).  Load with rgba == NULL
 * stores the entry count in *n_out only; otherwise capacity must hold it.  A
 * file whose stream is not good after the last number is refused, as
 * Load(istream) refuses it. */
tvk_status tvk_tf1d_load(const char* path, float* rgba, uint64_t capacity, uint64_t* n_out);
tvk_status tvk_tf1d_save(const char* path, const float* rgba, uint64_t n);
/* 2D TF (TransferFunction2D, IO/TransferFunction2D.cpp:222-264) as a float
 * table of h rows (gradient axis, row 0 at t = 0) by w columns (value axis). */
tvk_status tvk_set_tf2d_float(tvk_renderer* r, const float* rgba, uint32_t w, uint32_t h,
                              int rgba8_upload);

/* AbstrRenderer::SetRendermode / SetUseLighting / SetSampleRateModifier /
 * SetIsoValue (AbstrRenderer.h:323, 414-418). */
tvk_status tvk_set_render_mode(tvk_renderer* r, tvk_render_mode mode);
tvk_status tvk_set_lighting(tvk_renderer* r, int enable);
tvk_status tvk_set_sample_rate_modifier(tvk_renderer* r, float srm);
tvk_status tvk_set_isovalue(tvk_renderer* r, float isovalue);

/* AbstrRenderer::SetIsosurfaceColor (AbstrRenderer.h:423); default 0.5 grey.
 * Isosurface mode (GLRaycaster-ISO-FS + RefineIsosurface + Compose-FS) needs
 * no transfer function; tvk_renderer_set_volume resets the isovalue to half
 * the data range (AbstrRenderer.cpp:252-259). */
tvk_status tvk_set_iso_color(tvk_renderer* r, const float rgb[3]);

/* AbstrRenderer::SetColors (AbstrRenderer.h:621): ambient/diffuse/specular
 * RGBA (colour * w is used) and light direction in eye space. */
tvk_status tvk_set_colors(tvk_renderer* r, const float ambient[4], const float diffuse[4],
                          const float specular[4], const float light_dir[3]);
/* AbstrRenderer::SetScalingMethod (AbstrRenderer.h:263-265). */
tvk_status tvk_set_scaling_method(tvk_renderer* r, tvk_scaling_method method);
/* Selects the lighting model; ka/kd/ks/shininess are used by Blinn-Phong. */
tvk_status tvk_set_light_model(tvk_renderer* r, tvk_light_model model, float ka, float kd,
                               float ks, float shininess);

/* AbstrRenderer::SetViewParameters (AbstrRenderer.h:250-261) plus the eye/at/up
 * of GLRenderer::SetViewPort (Renderer/GL/GLRenderer.cpp:905-917). */
tvk_status tvk_set_view(tvk_renderer* r, const float eye[3], const float at[3],
                        const float up[3], float fovy_deg, float znear, float zfar);
/* AbstrRenderer::SetRotation/SetTranslation (AbstrRenderer.h:206-213): 4x4
 * row-vector matrices (Tuvok layout, translation in elements 12..14); must be
 * rigid.  modelview = rotation * translation * view. */
tvk_status tvk_set_model_transform(tvk_renderer* r, const float rotation[16],
                                   const float translation[16]);

/* AbstrRenderer::Resize (AbstrRenderer.h:431). */
tvk_status tvk_resize(tvk_renderer* r, uint32_t width, uint32_t height);

/* Frame-level early termination: stop visiting bricks once the frame alpha
 * reaches `threshold` (1 = never, the reference behaviour; GLRaycaster blends
 * every brick). */
tvk_status tvk_set_frame_termination(tvk_renderer* r, float threshold);

/* AbstrRenderer::Paint (AbstrRenderer.h:433) for one fixed-quality frame:
 * plans the brick list of the current LOD (AbstrRenderer.cpp:999-1100, LOD 0
 * unless tvk_set_lod chose another), then ray marches every pixel on the
 * renderer's stream.  Asynchronous. */
tvk_status tvk_paint(tvk_renderer* r);

/* m_iCurrentLOD for tvk_paint: the bricks of this LOD are rendered, with
 * fStepScale = (1/srm) * max(domain(0) / domain(lod)) and the LOD's brick
 * aspect in the texture coordinates (GLRaycaster.cpp:253-257,
 * uvfDataset.cpp:1747-1774).  TVK_ERR_UNSUPPORTED at paint time for LODs the
 * volume was not built with. */
tvk_status tvk_set_lod(tvk_renderer* r, uint32_t lod);

/* decreaseScreenResNow / decreaseSamplingRateNow for tvk_paint: render at
 * 1/screen_res_dec_factor of the viewport (GLRenderer::SetViewPort,
 * GLRenderer.cpp:864-889) and stretch the result over the viewport with
 * bilinear filtering (CopyOverCompletedRegion, :717-747), and/or divide the
 * sample rate by sample_dec_factor (GLRaycaster.cpp:253-254). */
tvk_status tvk_set_reduced_quality(tvk_renderer* r, int decrease_screen_res,
                                   int decrease_sampling_rate);

/* AbstrRenderer::SetPerfMeasures (AbstrRenderer.cpp:1435-1454): target frame
 * rate (0 = none, 10 s per frame), whether reduced-quality intermediate
 * subframes are allowed, and the two decrease factors (default 2, 2). */
tvk_status tvk_set_perf_measures(tvk_renderer* r, uint32_t min_framerate,
                                 int low_res_intermediate, float screen_res_dec_factor,
                                 float sample_dec_factor);

/* AbstrRenderer::SetLODLimits (AbstrRenderer.cpp:1456-1459): coarsest_skip
 * LODs are never used as the start LOD; finest is the finest LOD used. */
tvk_status tvk_set_lod_limits(tvk_renderer* r, uint32_t coarsest_skip, uint32_t finest);

/* m_eRendererTarget == RT_CAPTURE: progressive frames render LOD 0 only. */
tvk_status tvk_set_capture_mode(tvk_renderer* r, int capture);

/* AbstrRenderer::ComputeMinLODForCurrentView (AbstrRenderer.cpp:789-803) with
 * CullingLOD::GetLODLevel (CullingLOD.cpp:126-138): the finest LOD the
 * current view needs (screen-space error of one pixel). */
tvk_status tvk_compute_min_lod(tvk_renderer* r, uint32_t* lod);

typedef struct tvk_subframe_info {
  uint32_t lod;                  /* LOD the subframe rendered */
  int decreased_screen_res;      /* 1: rendered at reduced resolution, upscaled */
  int decreased_sampling_rate;   /* 1: rendered at the reduced sample rate */
  uint32_t render_width, render_height;
  uint32_t min_lod, start_lod;   /* the frame's plan */
  float ms;                      /* GPU time of the subframe */
  int frame_complete;            /* 1: nothing finer is left for this view */
} tvk_subframe_info;

/* One subframe of Tuvok's progressive frame: AbstrRenderer::PlanFrame
 * (AbstrRenderer.cpp:1125-1212) picks the LOD and quality, the subframe is
 * rendered and timed (blocking), and CompletedASubframe (:651-670) records the
 * time that ComputeMaxLODForCurrentView (:681-787) uses to choose the next
 * frame's start LOD and whether to decrease resolution or sample rate.
 * new_frame = 1 starts a frame for the current view (the reference's blank
 * region).  The sequence is: start LOD (at reduced quality when the planner
 * asks for it), the same LOD at full quality, then one LOD finer per call down
 * to the view's minimum LOD; after that info->frame_complete = 1 and calls
 * render nothing until the next new frame. */
tvk_status tvk_paint_progressive(tvk_renderer* r, int new_frame, tvk_subframe_info* info);

/* ---- Batched frames (no counterpart in the reference, which paints render
 * regions and renderers one after another: GLRenderer.cpp:622-660,
 * MasterController::RequestNewVolumeRenderer MasterController.cpp:145-200) ---- */

typedef struct tvk_batch tvk_batch;

typedef struct tvk_batch_info {
  uint32_t frames;        /* renderers in the last batch */
  uint32_t tiles;         /* work items (tiles) of the persistent launches */
  uint32_t ctas;          /* persistent CTAs launched */
  uint32_t ctas_per_sm;   /* chosen by the autotuner or fixed */
  uint32_t launches;      /* persistent launches: one per kernel variant (voxel
                             type x iso/compositing) and per 64 frames */
  int graph_reused;       /* 1: the captured CUDA graph was replayed */
  int autotuned;          /* 1: this call timed the candidate grid sizes */
  float ms;               /* GPU time of the batch */
  uint32_t rays_per_thread; /* 1: 16x8-pixel tiles; 2: 32x8 tiles, two rays per thread */
} tvk_batch_info;

/* A batch context (its own stream, CUDA graph and autotuning cache) on the
 * current device. */
tvk_status tvk_batch_create(tvk_batch** out);
tvk_status tvk_batch_destroy(tvk_batch* b);

/* Paints the current frame of every renderer (each with its own volume, TF,
 * mode, lighting, sample rate, view, viewport, LOD and reduced-quality
 * switches) in persistent kernel launches -- one per kernel variant present
 * (u8/u16 x iso/compositing) and per 64 frames -- replayed from a CUDA graph
 * while the batch's shape is unchanged.  Every renderer's image, sample counts and
 * statistics are bit-identical to its own tvk_paint.  Results are ordered
 * before later work on each renderer's stream.  The first call for a new
 * shape may render the batch a few extra times to time candidate grid sizes
 * (autotuning, on by default). */
tvk_status tvk_paint_batch(tvk_batch* b, tvk_renderer* const* renderers, uint32_t n);

/* autotune = 0 with ctas_per_sm = 0 uses the occupancy maximum; ctas_per_sm
 * > 0 fixes the persistent grid at that many CTAs per SM. */
tvk_status tvk_batch_set_autotune(tvk_batch* b, int autotune, uint32_t ctas_per_sm);
/* Rays each thread marches (tile width 16 x rays): 0 lets the autotuner pick
 * 1 or 2 per launch shape, together with the grid size. */
tvk_status tvk_batch_set_rays_per_thread(tvk_batch* b, uint32_t rays_per_thread);
tvk_status tvk_batch_get_info(tvk_batch* b, tvk_batch_info* out);

/* ---- Learned reconstruction primitives (no counterpart in the reference; the
 * network replaces its progressive reduced-quality frames, a25 above) ----
 *
 * Device pointers throughout; `stream` is a cudaStream_t (NULL = default).
 * Activations are NHWC BF16; a layer's weights are [tap = ky*3+kx][cout][cin]
 * (FP32 masters, BF16 copies for the kernels).  Convolutions run on the tensor
 * cores with FP32 accumulation. */

typedef struct tvk_cnn_conv {
  const void* x1;        /* BF16 input [n][h][w][c1] */
  const void* x2;        /* optional second input concatenated after x1 [n][h][w][c2] */
  int c1, c2;            /* c1 + c2 a multiple of 16, at most 128 */
  int n, h, w;           /* output size equals input size (padding 1) */
  const void* weights;   /* BF16 [9][cout][c1 + c2] */
  const float* bias;     /* [cout] or NULL */
  int cout;              /* a multiple of 8 in 8..128, 8 | 16 | 32 | 48 | ... */
  float slope;           /* LeakyReLU slope; negative: no activation */
  void* y_bf16;          /* BF16 output [n][h][w][cout] or NULL */
  float* y_f32;          /* FP32 output (channels < split) or NULL */
  float* y2_f32;         /* FP32 output of channels >= split, or NULL (no split) */
  int split;
  int accumulate;        /* FP32 outputs: add to the values there */
  /* 1: x1 is at half resolution, h1 x w1, and is read through a 2x nearest
   * upsampling clamped at its last row and column (x1 pixel (min(y / 2, h1 - 1),
   * min(x / 2, w1 - 1))), so a decoder layer needs no upsampled copy, also when
   * h or w is odd; 0: x1 is h x w. */
  int upsample1;
  int h1, w1;
} tvk_cnn_conv;

typedef struct tvk_cnn_wgrad {
  const void* x1;        /* forward input(s), BF16 */
  const void* x2;
  int c1, c2;
  const void* gy;        /* BF16 gradient at the pre-activation output [n][h][w][cout] */
  int n, h, w, cout;
  float* dw;             /* FP32 [9][cout][c1 + c2], accumulated */
  float* db;             /* FP32 [cout], accumulated, or NULL */
} tvk_cnn_wgrad;

/* y = act(conv3x3(concat(x1, x2), W) + b), zero padding (forward); with the
 * flipped-transposed weights of tvk_cnn_weights_bf16 it is the data gradient. */
tvk_status tvk_cnn_conv3x3(const tvk_cnn_conv* args, void* stream);
/* Waits for `stream` and reports a tensor-core convolution that gave up
 * waiting for its MMAs (bounded at 2 s per patch; TVK_ERR_INTERNAL, output
 * undefined).  Convolutions whose channel counts are multiples of 16 run on
 * tcgen05 with TMEM accumulators, the others on mma.sync. */
tvk_status tvk_cnn_check(void* stream);
/* dW += sum_p G[p] (x) X[p + tap], db += sum_p G[p]. */
tvk_status tvk_cnn_conv3x3_wgrad(const tvk_cnn_wgrad* args, void* stream);
/* G = dY * LeakyReLU'(Y) as BF16 (y = NULL or slope < 0: G = dY). */
tvk_status tvk_cnn_act_grad(const float* dy, const void* y, float slope, void* g_bf16, size_t n,
                            void* stream);
tvk_status tvk_cnn_avgpool2(const void* x, int n, int h, int w, int c, void* y, void* stream);
tvk_status tvk_cnn_avgpool2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                                     int accumulate, void* stream);
tvk_status tvk_cnn_upsample2(const void* x, int n, int h, int w, int c, void* y, void* stream);
tvk_status tvk_cnn_upsample2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                                      void* stream);
/* out [n][2h][2w][4] = base + pixel-shuffled head [n][h][w][16] (FP32). */
tvk_status tvk_cnn_head(const float* head, const float* base, int n, int h, int w, float* out,
                        void* stream);
tvk_status tvk_cnn_head_backward(const float* dout, int n, int h, int w, float* dhead,
                                 void* stream);
/* *loss += mean((out - target)^2); dout = 2 (out - target) / n (dout may be NULL). */
tvk_status tvk_cnn_mse(const float* out, const float* target, size_t n, float* dout, float* loss,
                       void* stream);
/* Adam step `step` (1-based) on FP32 weights. */
tvk_status tvk_cnn_adam(float* w, const float* g, float* m, float* v, size_t n, float lr, float b1,
                        float b2, float eps, int step, void* stream);
/* BF16 copies of a layer's FP32 weights: forward [9][cout][cin] and (if bwd is
 * not NULL) backward-data [9][cin][cout] with flipped taps. */
tvk_status tvk_cnn_weights_bf16(const float* w, int cout, int cin, void* fwd, void* bwd,
                                void* stream);
tvk_status tvk_cnn_to_bf16(const float* x, size_t n, void* y, void* stream);

/* Network input of a reduced frame: RGBA of the w x h image (FP32 [h][w][4]) in
 * channels 0..3, the first-hit depth (FP32 [h][w], as tvk_copy_depth_device
 * gives it; may be null) in channel 4, zero elsewhere and in the padding up to
 * wp x hp, as BF16 [hp][wp][16]. */
tvk_status tvk_cnn_prepare_input(const float* image_rgba, const float* depth, int h, int w, int hp,
                                 int wp, void* out, void* stream);

/* AbstrRenderer::SetClipPlane / EnableClipPlane / DisableClipPlane
 * (AbstrRenderer.h:215-219) for the brick-by-brick ray march: plane (a, b, c, d)
 * in world space; points with n . x + d >= 0, n = normalize(a, b, c) in model
 * space, are cut away (PLANE::clip, Basics/Vectors.h:1455-1457).  Each brick's
 * ray segment is cut at the plane (GLRaycaster.cpp:328-337 caps the brick box)
 * and bricks wholly on the cut side are skipped (AbstrRenderer::Clipped,
 * AbstrRenderer.cpp:923-948).  tvk_leaper_paint refuses a clipping renderer. */
tvk_status tvk_set_clip_plane(tvk_renderer* r, const float plane[4]);
tvk_status tvk_enable_clip_plane(tvk_renderer* r, int on);

/* ClearView (AbstrRenderer::SetCV, AbstrRenderer.cpp:1247-1256; its state
 * :130-136, 171).  In iso mode with ClearView on, tvk_paint marches a second,
 * "focus" isosurface at the ClearView isovalue behind the "context" surface
 * (GLRaycaster-ISO-CV-FS.glsl, driven by GLRaycaster.cpp:421-436) and shades
 * both with Compose-CV-FS.glsl: the context surface fades out near the focus
 * point and where its normals vary little, revealing the focus surface.
 * The isovalue is in data units like tvk_set_isovalue (normalised as
 * GetNormalizedCVIsovalue, AbstrRenderer.cpp:426-438); it starts at 1.5x the
 * isovalue when a volume is set (AbstrRenderer.cpp:261).  Colour, size,
 * context scale and border scale are SetCVColor / SetCVSize /
 * SetCVContextScale / SetCVBorderScale (AbstrRenderer.cpp:1316-1347; defaults
 * (1,0,0), 5.5, 1, 60).  The focus position is model space, w = 1
 * (SetCVFocusPosFVec, :1349-1352; default (0, 0, 0.5, 1));
 * tvk_set_cv_focus_pixel picks it from the context hit of the last ClearView
 * frame at a pixel of the ray-marched image (row 0 at the bottom), or moves it
 * far away (w = 0) where that pixel has no hit (GLRenderer::CVFocusHasChanged,
 * GLRenderer.cpp:2833-2854).  Batches and tvk_paint_learned refuse a ClearView
 * renderer in iso mode; tvk_leaper_paint renders without ClearView
 * (GLGridLeaper::SupportsClearView is false). */
tvk_status tvk_set_clearview(tvk_renderer* r, int on);
tvk_status tvk_set_cv_isovalue(tvk_renderer* r, float isovalue);
tvk_status tvk_set_cv_color(tvk_renderer* r, const float rgb[3]);
tvk_status tvk_set_cv_params(tvk_renderer* r, float size, float context_scale,
                             float border_scale);
tvk_status tvk_set_cv_focus_pos(tvk_renderer* r, const float pos[4]);
tvk_status tvk_get_cv_focus_pos(const tvk_renderer* r, float pos[4]);
tvk_status tvk_set_cv_focus_pixel(tvk_renderer* r, uint32_t x, uint32_t y);

/* First-hit depth of the ray-marched pixels: with `on`, every paint also
 * writes 1 / (1 + t) per pixel of the ray-marched image (render size), t the
 * eye-space distance of the first sample that adds anything (the iso hit in
 * iso mode), 0 where nothing is hit.  tvk_paint_learned writes it for its
 * reduced frame regardless. */
tvk_status tvk_set_depth_output(tvk_renderer* r, int on);
tvk_status tvk_copy_depth_device(tvk_renderer* r, void* dst, size_t bytes);

/* ---- Learned reconstruction (replaces the reference's progressive reduced-
 * quality frames, AbstrRenderer.cpp:681-787 and GLRenderer.cpp:717-747) ----
 *
 * The network: a fixed 4-level U-Net of 11 3x3 convolutions (LeakyReLU 0.1):
 * e0a 16->32, e0b 32->32 | pool | e1a 32->48, e1b 48->48 | pool | e2a 48->64,
 * e2b 64->64 | pool | b 64->64 | up, d2 (64+64)->64 | up, d1 (64+48)->48 | up,
 * d0 (48+32)->32 | head 32->16 (no activation), whose 16 channels are RGBA x
 * 2x2 sub-pixels added to the bilinear upscale of the reduced frame. */

typedef struct tvk_learned tvk_learned;

typedef struct tvk_learned_info {
  float probe_psnr_db;           /* PSNR of the frame at the probe pixels */
  int fell_back;                 /* 1: the plain full-quality frame was rendered */
  float ms_reduced;              /* reduced frame + bilinear upscale */
  float ms_network;              /* input preparation + U-Net */
  float ms_probe;                /* the probe rays (on their own stream, overlapping
                                    the reduced frame and the network) */
  float ms_fallback;             /* the plain frame when falling back, else ~0 */
  uint32_t reduced_width, reduced_height;
  float ms_judge;                /* after the network: waiting for the probes and
                                    comparing them */
  float ms_frame;                /* the whole frame on the renderer's stream */
} tvk_learned_info;

/* Number of FP32 parameters: per layer in the order above, the weights
 * [9][cout][cin] followed by the bias [cout]. */
tvk_status tvk_learned_param_count(size_t* n);
tvk_status tvk_learned_create(const float* host_params, size_t n, tvk_learned** out);
tvk_status tvk_learned_destroy(tvk_learned* net);

/* One learned frame on the renderer (its volume, TF, lighting, view and
 * viewport): the frame at half resolution and half sample rate (as
 * tvk_set_reduced_quality), its bilinear upscale plus the network's residual
 * as the image, then the probe-ray judge: one pixel of every 8x8 block is ray
 * marched at full quality and compared; below threshold_db of probe PSNR the
 * plain full-quality frame replaces the result.  Blocking (the judge reads its
 * error back). */
tvk_status tvk_paint_learned(tvk_renderer* r, tvk_learned* net, float threshold_db,
                             tvk_learned_info* info);

/* Copies the last final image (reduced = 0, width*height*4 floats) or the last
 * ray-marched reduced image (reduced = 1, render size) to device memory, on the
 * renderer's stream. */
tvk_status tvk_copy_image_device(tvk_renderer* r, int reduced, void* dst, size_t bytes);

/* ---- GridLeaper: single-pass LOD traversal over a paged brick cache ----
 *
 * A pool is the GLVolumePool of a volume (GLVolumePool.cpp:119-259): a brick
 * cache of slots in HBM (as many maximum-size bricks as `budget_bytes` holds),
 * a page table over the bricks of every LOD (MISSING / CHILD_EMPTY / EMPTY /
 * slot), the visibility flags for the current TF or isovalue
 * (RecomputeVisibilityForOctree, :1020-1359) and the missing-brick hash table
 * (GLHashTable, size max(15, 509 / (brick voxels / 32768)), 10 probes).  The
 * single brick of the coarsest LOD is pinned in the last slot.  With
 * host_source the volume's bricks are copied once to pinned host memory and
 * paged from there to the device on a side stream, else they are copied from
 * the volume's device pool. */

typedef struct tvk_pool tvk_pool;

typedef struct tvk_pool_info {
  uint32_t slots;
  uint64_t slot_bytes;
  uint64_t bricks;        /* bricks of every LOD (page-table entries) */
  uint32_t hash_size;
  int host_source;
  uint64_t paged_total;   /* bricks paged in so far */
} tvk_pool_info;

typedef struct tvk_leaper_info {
  uint32_t passes;        /* traversal passes run */
  uint32_t paged;         /* bricks paged in during this frame */
  uint32_t missing_last;  /* bricks the last pass reported missing */
  int converged;          /* 1: the last pass found every brick it wanted */
  uint32_t resident;      /* bricks in the cache after the frame */
  float ms;               /* GPU time of the frame, paging included */
  float ms_traversal;     /* of which in the traversal kernels */
  uint64_t bytes_paged;   /* brick bytes copied into the cache this frame */
  uint64_t samples;       /* samples over all passes */
  float ms_host;          /* host time choosing slots and issuing the copies */
} tvk_leaper_info;

tvk_status tvk_pool_create(const tvk_volume* v, uint64_t budget_bytes, int host_source,
                           tvk_pool** out);
tvk_status tvk_pool_destroy(tvk_pool* p);
tvk_status tvk_pool_get_info(const tvk_pool* p, tvk_pool_info* out);
/* The host copy of the page table (one entry per brick in TOC order: 0
 * MISSING, 1 CHILD_EMPTY, 2 EMPTY, else slot + 3). */
tvk_status tvk_pool_get_page_table(const tvk_pool* p, uint32_t* out, size_t n);
/* The bricks (TOC indices, ascending) the last traversal pass reported missing
 * through the hash table (GLHashTable::GetData, GLHashTable.cpp:90-105): the
 * first min(n, *count) are written, *count is the total. */
tvk_status tvk_pool_get_requests(const tvk_pool* p, uint64_t* out, size_t n, size_t* count);

/* GLVolumePool::PH_Reset (GLVolumePool.cpp:261-282): empties the cache except
 * the slot holding the coarsest brick; visibility is recomputed on the next
 * tvk_leaper_paint. */
tvk_status tvk_pool_reset(tvk_pool* p);

/* Size of the missing-brick hash table (GLHashTable, GLGridLeaper.cpp:266-273):
 * 0 restores the reference's max(15, 509 / (brick voxels / 32768)) with 10
 * probes; otherwise `size` entries and `rehash` probes.  A pass reports at
 * most `size` bricks, so with 128^3 bricks the reference's 15 entries bound
 * the bricks paged per pass. */
tvk_status tvk_pool_set_request_table(tvk_pool* p, uint32_t size, uint32_t rehash);

/* One GridLeaper frame with the renderer's TF, mode (1D, 2D, iso), lighting,
 * sample rate and view (GLGridLeaper::Render3DRegion, GLGridLeaper.cpp:914-1154):
 * traversal passes (GLGridLeaper-blend.glsl / -iso.glsl) that resume each ray
 * where it first met a brick coarser than its screen-space error asked for;
 * between passes the reported bricks are paged in, oldest slots first.  Stops
 * when a pass reports nothing missing or after max_passes.  The image is the
 * last pass's (tvk_read_image).  Blocking. */
tvk_status tvk_leaper_paint(tvk_renderer* r, tvk_pool* pool, uint32_t max_passes,
                            tvk_leaper_info* info);

/* Size of the last ray-marched image (the viewport, or the reduced one). */
tvk_status tvk_get_render_size(tvk_renderer* r, uint32_t* width, uint32_t* height);

/* GLRenderer::GetLastFBO + GLFBOTex::ReadBackPixels (GLRenderer.h:105,
 * GLFBOTex.cpp:401): device pointer of the last frame and a blocking copy to
 * host memory (width*height*4 floats). */
tvk_status tvk_get_image_device(tvk_renderer* r, const float** device_rgba, uint32_t* width,
                                uint32_t* height);
tvk_status tvk_read_image(tvk_renderer* r, float* host_rgba, size_t n_floats);

/* The last frame's image copied to host memory asynchronously: the frame is
 * copied once on the device (on the renderer's stream, after the frame), then
 * to host_rgba on a copy stream of the renderer while later frames render.
 * host_rgba must stay valid until tvk_wait_image returns (page-locked memory
 * lets the copy overlap rendering).  Copies complete in the order they were
 * asked for; a new one waits (on the device) for the previous one.  No
 * counterpart in the reference, whose GLRenderer::ReadBackPixels blocks. */
tvk_status tvk_read_image_async(tvk_renderer* r, float* host_rgba, size_t n_floats);
/* Blocks until every asynchronous image copy asked for so far is complete. */
tvk_status tvk_wait_image(tvk_renderer* r);
/* Per-pixel executed sample counts of the last paint (u32 per pixel of the
 * ray-marched image, tvk_get_render_size). */
tvk_status tvk_read_sample_counts(tvk_renderer* r, uint32_t* host_counts, size_t n);

/* The renderer's CUDA stream (cudaStream_t) for callers that order their own
 * work after a paint. */
tvk_status tvk_renderer_get_stream(tvk_renderer* r, void** stream);
/* Blocks until the renderer's stream is idle and fills *out for the last paint. */
tvk_status tvk_get_stats(tvk_renderer* r, tvk_stats* out);
/* The raw counters of the renderer's last paint: [0] reference loop steps
 * (samples), [1] executed samples, [2] rays the march guard stopped, [3]
 * samples that took the gradient; [4..7] are filled only by a library built
 * with TVK_PROFILE_COUNTS=1 (leap iterations, steps they skipped,
 * candidate-brick slab tests, brick marches) and are 0 otherwise.  A
 * diagnostic with no counterpart in the reference. */
tvk_status tvk_get_counters(tvk_renderer* r, uint64_t out[8]);

/* Hardware-filtered lookups (on != 0): the ray march samples each brick
 * through a texture object (a 3D CUDA array copy of every brick, made on the
 * first such frame of the volume) with the texture unit's trilinear filter,
 * instead of the exact eight-texel lookups.  The filter's fixed-point weights
 * make frames differ slightly from the reference restatement; the exact path
 * (the default) is the parity path.  Scalar volumes, 1D / 2D / iso modes;
 * ClearView frames, colour volumes and batches refuse it; the GridLeaper
 * ignores it.  The texture sampling GLSL does (Volume3D.glsl:39-41 texture3D)
 * on the GPU's texture unit, with no separate reference entry point. */
tvk_status tvk_set_hardware_filtering(tvk_renderer* r, int on);

/* The macro-cell table of brick `index` (TOC order, any LOD): cells of 2^3
 * voxel positions, cell c covering voxels c*2 .. c*2 + 2 on each axis
 * (clamped to the brick), each entry min | max << 16 of the raw values there.
 * dims receives the cell counts (x, y, z); with out == NULL only dims is
 * filled, otherwise capacity must hold x*y*z entries, x fastest.  Colour
 * volumes have no cells (TVK_ERR_UNSUPPORTED).  A diagnostic with no
 * counterpart in the reference (the ray march's empty-space tables). */
tvk_status tvk_volume_cell_minmax(const tvk_volume* v, uint64_t index, uint32_t* out,
                                  uint64_t capacity, uint32_t dims[3]);

/* ---------------------------------------------------------------- allocation-free bricking */

/* Most entry points allocate device memory as they go (tvk_volume_create
 * allocates its brick pool and statistics scratch).  Some callers cannot allow
 * that at call time: a host that gives the library a fixed device-memory budget
 * up front, or code that records work into a stream capture or draws only from
 * its own pre-sized pool.  For them this entry point bricks up to
 * TVK_NOALLOC_MAX_BRICKS LOD-0 bricks of a volume that is already in device
 * memory and allocates nothing: the caller passes every input and output, and
 * the per-brick min/max and histogram accumulators live in a fixed array inside
 * the library (about 66 KB on every GPU that loads it, held until the process
 * exits).  It has no counterpart in the reference.
 *
 * The bricks' voxels are the same as tvk_volume_create / tvk_volume_get_brick
 * return (GetInputBrick + ClampToEdge semantics); they are written back to back
 * in the order of brick_coords (x, y, z triples, LOD 0) into device_bricks_out.
 * device_minmax_out receives one tvk_minmax and device_hist_out 256 counts per
 * brick (inner voxels, bin = value >> hist_shift; pass the shift that
 * tvk_volume_get_brick_histograms reports to get the same bins).  Work is
 * queued on `stream` (a cudaStream_t, NULL for the legacy default stream) and
 * the call returns without waiting.
 *   - count above TVK_NOALLOC_MAX_BRICKS, an output smaller than the bricks,
 *     or a pointer not aligned to its element (voxels to the voxel size,
 *     device_minmax_out to 8 bytes, device_hist_out to 4) is rejected with
 *     TVK_ERR_INVALID_ARG and a message before any GPU work is queued;
 *   - the fixed accumulators are shared: each call clears what it uses, and
 *     calls whose GPU work overlaps (different streams or host threads) race;
 *   - the first call on a device looks up the accumulators' device address for
 *     that device (the current device); make that first call before any stream
 *     capture starts.  The address is kept for the life of the process, so the
 *     entry point must not be used after a cudaDeviceReset of that device. */
#define TVK_NOALLOC_MAX_BRICKS 64
tvk_status tvk_brick_lod0_noalloc(const void* device_voxels, tvk_dtype dtype,
                                  const uint64_t dims[3], const uint32_t brick_size[3],
                                  uint32_t overlap, int clamp_to_edge,
                                  const uint64_t* brick_coords, uint32_t count,
                                  uint32_t hist_shift, void* device_bricks_out, size_t out_bytes,
                                  tvk_minmax* device_minmax_out, uint32_t* device_hist_out,
                                  void* stream);

/* ---------------------------------------------------------------- synthetic data */

/* Fills device memory with a seeded volume: the sum of Gaussian blobs (7
 * floats each: cx, cy, cz, sigma, peak, 0, 0; voxel units, centre at voxel
 * centres) plus value noise of `noise_octaves` octaves (cell size halving from
 * noise_cell, amplitude noise_amp) or, with int_noise != 0, uniform integer
 * noise in [-noise_amp, noise_amp]; rounded and clamped to [0, vmax].  The
 * Gaussians are evaluated separably (per-axis factors computed in double on
 * the host) and combined in a fixed order of float operations, so the bytes
 * are a function of the arguments alone on any IEEE machine.  Input creation
 * for tests and benchmarks only. */
tvk_status tvk_generate_volume(void* device_out, tvk_dtype dtype, const uint64_t dims[3],
                               const float* host_blobs, uint32_t n_blobs, float noise_amp,
                               uint32_t noise_octaves, float noise_cell, uint64_t seed,
                               int int_noise, float vmax);

#ifdef __cplusplus
}
#endif

#endif /* TVK_H */
