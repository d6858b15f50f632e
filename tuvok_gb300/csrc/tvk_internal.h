// tvk_internal.h -- shared host/device definitions of the tuvok_gb300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/tvk.h"

namespace tvk {

// ------------------------------------------------------------------ errors

struct Error {
  tvk_status status;
  std::string msg;
};

[[noreturn]] void fail(tvk_status s, const std::string& msg);
void check_cuda(cudaError_t e, const char* what);
// Sets the calling thread's message returned by tvk_last_error().
void set_last_error(const std::string& msg);
#define TVK_CUDA(call) ::tvk::check_cuda((call), #call)

// ------------------------------------------------------------------ bricking

// One LOD of the ExtendedOctree table (IO/UVF/ExtendedOctree/ExtendedOctree.h).
struct LodInfo {
  uint64_t size[3];
  uint64_t bricks[3];
  double aspect[3];
};

// Device-side accumulators of the bricking pass (global scratch memory).
struct BrickScratch {
  uint32_t* bmin;       // per brick
  uint32_t* bmax;       // per brick
  uint32_t* bhist;      // per brick x 256
  unsigned long long* hist;  // global histogram, 2^(8*bytes) bins
  unsigned long long* max_grad_bits;  // IEEE double bits of the max |grad|
  uint32_t* raw_minmax;  // [min, max] of the raw volume
};

// Geometry of the LOD-0 brick grid handed to the bricking kernels.
struct BrickGrid {
  uint64_t dims[3];
  uint32_t B[3];        // max brick size incl. overlap
  uint32_t ov;
  uint32_t cnt[3];      // bricks per axis
  int clamp;
  uint64_t total;       // voxels of the raw volume
};

// RGBA8 colour volumes: LOD-0 bricks with ghost voxels only
void launch_brick_copy4(const void* raw, const BrickGrid& g, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, void* pool, cudaStream_t s,
                        uint64_t* launches);
// LOD-0 bricks + per-brick min/max + global histogram (pass 1), then per-brick
// histograms and largest squared central difference (pass 2), then the exact
// maximum |gradient| at the voxels of the largest one (bricking.cu)
void launch_brick_copy(const void* raw, int bytes, const BrickGrid& g, const uint64_t* d_offsets,
                       const uint32_t* d_sizes, uint64_t n_bricks, void* pool,
                       const BrickScratch& sc, uint32_t global_bins, cudaStream_t s,
                       uint64_t* launches);
void launch_brick_sweep(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, uint32_t ov, uint32_t max_bz,
                        uint32_t shift, uint32_t* bhist, unsigned long long* brick_qmax,
                        cudaStream_t s, uint64_t* launches);
void launch_max_gradient_at(const void* pool, int bytes, const uint64_t* d_offsets,
                            const uint32_t* d_sizes, const uint32_t* d_bricks, uint32_t n_list,
                            uint32_t ov, uint32_t max_bz, long long q_target,
                            unsigned long long* out_bits, cudaStream_t s, uint64_t* launches);

// TransferFunction1D::Set byte semantics (tf1d.cpp)
void tf1d_from_bytes(const uint8_t* bytes, uint64_t n, float* rgba);

// ExtendedOctree tables and UVF metadata (api.cpp)
std::vector<LodInfo> lod_table(const uint64_t dims[3], const uint32_t B[3], uint32_t ov);

// brick decoders (codecs.cpp): the whole stream into exactly out_n bytes
void zlib_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n);
void lzma_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n, uint32_t lc,
                 uint32_t lp, uint32_t pb);
void bzip2_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n);

// ExtendedOctree file (eo.cpp): header and table of contents
struct EoFile {
  std::string path;
  uint64_t base = 0;               // offset of the header in the file
  uint32_t component_type = 0;     // ExtendedOctree::COMPONENT_TYPE (0 = UINT8, 1 = UINT16)
  uint64_t components = 0;
  bool normals = false;
  uint64_t dims[3] = {0, 0, 0};
  double aspect[3] = {1, 1, 1};
  uint64_t brick_size[3] = {0, 0, 0};
  uint32_t overlap = 0, version = 0, compression_level = 0;
  uint64_t size = 0;
  struct Entry {
    uint64_t offset, length;       // from the header's start
    uint32_t compression;          // COMPRESSION_TYPE: 0 none, 3 LZ4
    uint64_t valid_length;
    uint32_t atlas[2];
  };
  std::vector<Entry> toc;          // every LOD's bricks in TOC order
};
void eo_open(const char* path, uint64_t offset, uint32_t uvf_version, EoFile& e);
void eo_read_brick(const EoFile& e, uint64_t index, size_t bytes, std::vector<uint8_t>& out);
size_t lz4_decode_block(const uint8_t* src, size_t src_len, uint8_t* dst, size_t dst_len);

// UVF container (uvf.cpp): global header and the chain of data-block headers
struct UvfFile {
  uint64_t version = 0, checksum_semantics = 0, checksum_bytes = 0;
  uint64_t data_offset = 0, file_bytes = 0;
  bool big_endian = false, checksum_verified = false, has_raster = false;
  std::vector<tvk_uvf_block> blocks;
  std::vector<uint32_t> timesteps;  // indices into blocks of the accepted TOC blocks
};
void uvf_open(const char* path, bool verify_checksum, UvfFile& u);
void brick_size(const LodInfo& l, const uint32_t B[3], uint32_t ov, const uint64_t c[3],
                uint32_t out[3]);
void brick_metadata(const LodInfo& l, const uint32_t B[3], uint32_t ov,
                    std::vector<tvk_brick_md>& md);

// DynamicBrickingDS (rebrick.cu): a new volume whose bricks are windows of the
// source's bricks, gathered on the GPU.  mm_mode: 0 MM_SOURCE, 1 MM_PRECOMPUTE,
// 2 MM_DYNAMIC.
tvk_volume* rebrick_volume(const tvk_volume* src, const uint32_t brick_size[3], int mm_mode);

// value x |gradient| histogram of the LOD-0 inner voxels (Histogram2DDataBlock)
struct Hist2DParams {
  uint32_t ov, z_chunk;
  uint32_t value_bins;    // rows of 256 gradient bins
  uint32_t scale_values;  // 1: bin = value * (value_bins - 1) / max_nonzero
  double max_nonzero;
  double gmax;            // maximum |gradient| (double, as the reference finds it)
  long long qmax;         // its integer squared central-difference sum
  float inv_qmax;
};
void launch_histogram2d(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, uint32_t max_bz,
                        Hist2DParams hp, unsigned long long* hist, cudaStream_t s,
                        uint64_t* launches);
// LODs 1.. of the octree in place in the pool (lod.cu); min/max of every
// LOD>=1 brick into d_min/d_max (indexed by TOC index).
void build_lod_levels(void* pool, int bytes, const uint64_t* d_offsets, const uint64_t* d_voxels,
                      const std::vector<LodInfo>& lods, const std::vector<uint64_t>& lod_first,
                      const uint32_t B[3], uint32_t ov, bool clamp, bool median,
                      uint32_t* d_min, uint32_t* d_max, uint32_t* d_wave, cudaStream_t s,
                      uint64_t* launches);
// seeded synthetic volume (volgen.cu); host_blobs: 7 floats per blob
void launch_generate(void* out, int bytes, const uint64_t dims[3], const float* host_blobs,
                     uint32_t n_blobs, float noise_amp, uint32_t octaves, float cell,
                     uint64_t seed, int int_noise, float vmax, cudaStream_t s);

// ------------------------------------------------------------------ ray march

// Macro cells for empty-space skipping inside a brick: cell c on an axis
// covers sample positions u in [c*kCell, (c+1)*kCell) (voxel coordinates after
// clamping to [0, n-1]); its min/max cover voxels c*kCell .. (c+1)*kCell
// (clamped), every voxel a trilinear lookup from such a position can touch.
#ifndef TVK_CELL_SHIFT
// 2^3 cells with Chebyshev-distance leaps: measured fastest on the 1024^3 lit
// 1080p frame (4.4 ms, against 5.2 ms with 4^3 and 6.3 ms with 8^3 cells)
#define TVK_CELL_SHIFT 1
#endif
constexpr int kCellShift = TVK_CELL_SHIFT;
constexpr int kCell = 1 << kCellShift;
__host__ __device__ inline uint32_t cells_per_axis(uint32_t n) {
  return ((n - 1) >> kCellShift) + 1;
}

// Per-brick record of one frame (host-computed, uploaded per paint).
struct alignas(16) DevBrick {
  float pmin[3];
  float step;           // fRayStepsize
  float pmax[3];
  uint32_t cells;       // cells per axis, packed x | y << 10 | z << 20
  float tex[3][4];      // eye -> brick texture coordinates
  uint32_t n[3];        // voxels incl. ghost
  uint32_t id;          // TOC index of the brick (its texture, when filtering in hardware)
  unsigned long long off;        // voxel offset of the brick in the pool
  unsigned long long cell_off;   // offset of the brick's first macro cell
};

// Per-cell min/max of every LOD-0 brick (volume creation); packed min | max << 16.
// macro-cell min/max of every listed brick; max_cell_rows = the largest
// number of cells along y of a brick
void launch_cell_minmax(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, const uint64_t* d_cell_offsets,
                        uint64_t n_bricks, uint32_t max_cell_rows, uint32_t* cells,
                        cudaStream_t s, uint64_t* launches);

// Empty-cell bits for the current transfer function (1 = every reachable TF
// entry has zero corrected alpha).
struct EmptyCellParams {
  const uint32_t* cell_minmax;         // volume cells
  const uint64_t* cell_offsets;        // per brick, first cell
  const uint32_t* cell_counts;         // per brick, cells in total
  const uint64_t* word_offsets;        // per brick, first word of its bits
  uint64_t n_bricks;
  const uint32_t* nz_prefix;           // prefix count of non-zero TF entries / columns
  uint32_t tf_w;
  float inv_max_raw, trans_scale;
  int iso_mode;                        // 1: empty = cell maximum below iso_norm
  float iso_norm;
  uint32_t* bits;
};
void launch_empty_cells(const EmptyCellParams& p, uint32_t max_words_per_brick, cudaStream_t s,
                        uint64_t* launches);

// Chebyshev distance, in cells and capped at kCellDistCap, from every macro
// cell to the nearest non-empty cell of its brick (0: the cell is not empty):
// every cell within distance d - 1 of a cell at distance d is empty, so a ray
// may leap over that whole cube.  Three separable passes (x from the empty
// bits, then y, then z) over all bricks.
#ifndef TVK_CELL_DIST_CAP
#define TVK_CELL_DIST_CAP 15  // 15, 31 and 63 measure the same with 2^3 cells; 15 halves the passes
#endif
constexpr int kCellDistCap = TVK_CELL_DIST_CAP;
struct CellDistParams {
  const uint32_t* bits;           // empty-cell bits (pass x)
  const uint64_t* word_offsets;   // per brick, first word of its bits
  const uint64_t* cell_offsets;   // per brick, first cell
  const uint32_t* cell_dims;      // per brick, cells per axis packed x | y << 10 | z << 20
  const uint8_t* in;              // passes y and z: the previous pass
  uint8_t* out;
  uint64_t n_bricks;
};
void launch_cell_dist(const CellDistParams& p, const uint32_t max_lines[3], uint8_t* tmp_a,
                      uint8_t* tmp_b, uint8_t* dist, cudaStream_t s, uint64_t* launches);

struct RenderParams {
  const void* pool;
  int bytes;                 // 1 or 2 (scalar), 4 (RGBA8 colour volume)
  const DevBrick* bricks;    // visible bricks only, compact
  uint32_t n_bricks;
  const uint8_t* cell_dist;    // macro-cell distances (null: no skipping inside bricks)
  const float4* tf;          // rgb + opacity-corrected alpha
  const uint8_t* tf_col_nonzero;  // 2D: per value column, any alpha > 0
  uint32_t tf_w, tf_h;
  int mode;                  // tvk_render_mode
  int lighting;
  int light_model;
  float trans_scale, grad_scale;
  float inv_max_raw;
  float light_a[3], light_d[3], light_s[3], light_dir[3];
  float bp_ka, bp_kd, bp_ks, bp_shininess;
  float norm_mat[3][3];
  float domain_scale[3];
  float inv[3][4];           // eye -> model (rigid)
  float mv[3][4];            // model -> eye
  float kx, ky, inv_w2, inv_h2;
  float znear, zfar;
  float frame_ert;
  float iso_norm;            // fIsoval
  float proj_x, proj_y;      // vProjParam
  float iso_diffuse[3];      // diffuse colour * iso colour
  float max_q;               // guard on len/step
  uint32_t width, height;     // the frame the camera projects to
  // pixels actually marched: (x * stride + off_x, y * stride + off_y) for x <
  // out_w, y < out_h, written densely to out (stride 1, offset 0: every pixel)
  uint32_t out_w, out_h, stride, off_x, off_y;
  float4* out;
  uint32_t* spp;             // per-pixel sample counts (may be null)
  float* depth;              // per pixel 1 / (1 + first-hit distance), 0: no hit (may be null)
  int clip_on;               // clip plane: keep eye-space points p with
  float clip_eye[4];         //   clip_eye . (p, 1) <= 0
  // ClearView (iso mode): the march writes, per pixel, the context surface's
  // hit and normal and the focus surface's hit and normal to cv_hits (four
  // float4 per pixel) instead of shading; cv_compose shades them.
  int cv_on;
  float cv_iso;              // the focus surface's fIsoval (GetNormalizedCVIsovalue)
  int cv_cell_skip;          // cell distances hold for cv_iso too (cv_iso >= iso_norm)
  float4* cv_hits;
  float step_scale;          // fStepScale (colour volumes correct opacity per sample)
  unsigned long long* counters;  // [samples, shaded, errors, gradient samples]
  // hardware-filtered lookups: the texture object of every brick (TOC order),
  // null for the exact lookups from the pool
  const cudaTextureObject_t* tex;
};

void launch_raycast(const RenderParams& p, cudaStream_t s, uint64_t* launches);

// Compose-CV-FS.glsl:49-108 over the hit records of a ClearView frame of
// w x h pixels drawn at the lower left of a fbo_w x fbo_h target: context
// lighting, curvature from the four neighbours' normals, distance to the focus
// point, focus lighting, blend and border darkening.
struct CvComposeParams {
  const float4* hits;        // four float4 per pixel (see RenderParams::cv_hits)
  float4* out;
  uint32_t w, h, fbo_w, fbo_h;
  float light_a[3], diffuse_context[3], diffuse_focus[3], light_s[3], light_dir[3];
  float size, context_scale, border_scale;  // vCVParam
  float pick[3];                             // vCVPickPos (eye space)
};
void launch_cv_compose(const CvComposeParams& p, cudaStream_t s, uint64_t* launches);
// Frames of one persistent batched launch, passed whole as a kernel parameter
// (it lives in the constant bank; no staging copy).  All frames of a launch
// share the kernel variant: voxel type and iso or compositing mode.
constexpr uint32_t kBatchFrames = 64;
struct BatchLaunch {
  uint32_t n_frames;
  uint32_t tile_first[kBatchFrames + 1];  // prefix sum of 16x8 tiles per frame
  RenderParams frames[kBatchFrames];
};
static_assert(sizeof(BatchLaunch) <= 32000, "kernel parameters are limited to 32 KB");
// variant = (bytes == 2 ? 2 : 0) + (iso ? 1 : 0); *d_next_item must start at 0
void launch_raycast_batch(const BatchLaunch& L, int variant, uint32_t* d_next_item,
                          uint32_t ctas, cudaStream_t s, uint64_t* launches);
int batch_ctas_per_sm_max(int variant);
const void* batch_kernel_function(int variant);
// ------------------------------------------------------------------ GridLeaper

// Page-table entries (GLVolumePool.cpp:25-30): flags, or the slot + kBiFlagCount
constexpr uint32_t kBiMissing = 0, kBiChildEmpty = 1, kBiEmpty = 2, kBiFlagCount = 3;
constexpr uint32_t kLeaperMaxLods = 20;

// One GridLeaper pass (GLGridLeaper-blend.glsl / -iso.glsl over the functions
// GLVolumePool.cpp:484-656 generates).  Shading, TF and camera fields come from
// the renderer's RenderParams.
struct LeaperParams {
  RenderParams R;
  const void* slots;           // brick cache: slot s at slots + s * slot_voxels
  uint64_t slot_voxels;
  const uint32_t* page;        // page table over the bricks of every LOD
  const uint32_t* brick_dims;  // per brick n_voxels x | y << 10 | z << 20
  uint32_t max_lod;            // iMaxLOD
  float layout[kLeaperMaxLods][3];  // GetFloatBrickLayout per LOD
  uint32_t lod_offset[kLeaperMaxLods], lod_lx[kLeaperMaxLods], lod_lxy[kLeaperMaxLods];
  float vol_size[3];           // LOD-0 voxels (volumeSize)
  float max_inner[3];          // inner brick size (maxInnerBrickSize)
  float ghost;                 // overlap voxels per side
  float lod_factor, lod0_err;  // fLoDFactor, fLevelZeroWorldSpaceError
  float eye2norm[3][4];        // eye space -> normalised volume coordinates
  float norm2eye[3][4];
  float norm_to_eye_n[3][3];   // normals (mModelViewIT)
  float light_dir_model[3], eye_model[3];
  float srm;
  uint32_t* hash;              // missing-brick hash table (GLHashTable)
  uint32_t hash_size, rehash;
  uint32_t ser_x, ser_xy, ser_xyz;  // Serialize: LOD-0 layout x, x*y, x*y*z
  float4* resume_pos;          // xyz = normalised position, w = depth (1000: done)
  float4* resume_col;
  uint32_t first_pass;
  const uint8_t* cell_dist;    // macro-cell distances of every brick (null: none)
  const uint64_t* cell_off;    // per brick, first macro cell
};
void launch_leaper(const LeaperParams& p, cudaStream_t s, uint64_t* launches);

// Bilinear stretch of a reduced-resolution image over the viewport
// (GLRenderer::CopyOverCompletedRegion with GL_LINEAR).
void launch_upscale(const float4* low, uint32_t lw, uint32_t lh, float4* out, uint32_t w,
                    uint32_t h, float rescale, cudaStream_t s, uint64_t* launches);

// ------------------------------------------------------------------ CNN (cnn.cu)

using CnnConv = tvk_cnn_conv;
using CnnWgrad = tvk_cnn_wgrad;
void cnn_conv3x3(const CnnConv& c, cudaStream_t s);
// c's convolution (16 output channels) with the head's pixel shuffle fused:
// out[oh][ow][4] += shuffle(conv); c.y_f32 is the buffer of the unfused fallback.
void cnn_conv3x3_shuffle(const CnnConv& c, float* out, int oh, int ow, cudaStream_t s);
// Tensor-core convolutions that gave up waiting for their MMAs since the last
// reset (0 normally).
uint32_t cnn_tc_timeouts(bool reset);
void cnn_conv3x3_wgrad(const CnnWgrad& c, cudaStream_t s);
void cnn_act_grad(const float* dy, const void* y, float slope, void* g, size_t n, cudaStream_t s);
void cnn_avgpool2(const void* x, int n, int h, int w, int c, void* y, cudaStream_t s);
void cnn_avgpool2_backward(const float* dy, int n, int h, int w, int c, float* dx, int accumulate,
                           cudaStream_t s);
void cnn_upsample2(const void* x, int n, int h, int w, int c, void* y, cudaStream_t s);
void cnn_upsample2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                            cudaStream_t s);
void cnn_head(const float* head, const float* base, int n, int h, int w, int oh, int ow,
              float* out, cudaStream_t s);
void cnn_prepare_input(const float* img, const float* depth, int h, int w, int hp, int wp,
                       void* out, cudaStream_t s);
void cnn_probe_mse(const float* frame, int w, const float* probe, int pw, int ph, int stride,
                   int ox, int oy, float* sum, cudaStream_t s);
void cnn_head_backward(const float* dout, int n, int h, int w, float* dhead, cudaStream_t s);
void cnn_mse(const float* out, const float* target, size_t n, float* dout, float* loss,
             cudaStream_t s);
void cnn_adam(float* w, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2,
              float eps, int step, cudaStream_t s);
void cnn_weights_bf16(const float* w, int cout, int cin, void* fwd, void* bwd, cudaStream_t s);
void cnn_to_bf16(const float* x, size_t n, void* y, cudaStream_t s);

}  // namespace tvk

// ------------------------------------------------------------------ handles

struct tvk_volume {
  int device = 0;
  tvk_dtype dtype = TVK_U8;
  int bytes = 1;
  uint64_t dims[3] = {0, 0, 0};
  uint32_t brick_size[3] = {0, 0, 0};
  uint32_t overlap = 0;
  bool clamp = false;
  std::vector<tvk::LodInfo> lods;
  bool build_lods = true;   // coarser LODs too (ComputeHierarchy)
  bool median = false;      // 7-value median instead of the mean
  std::vector<uint64_t> lod_first;  // TOC index of each built LOD's first brick (+ end)
  uint64_t total_bricks = 0;  // all built LODs
  uint64_t n_bricks = 0;  // LOD 0
  std::vector<tvk_brick_md> md;
  std::vector<uint64_t> offsets;  // voxels, per brick
  std::vector<uint32_t> sizes;    // 3 per brick
  std::vector<double> bmin, bmax;
  std::vector<unsigned long long> hist;
  std::vector<uint32_t> bhist;
  uint32_t hist_shift = 0;
  uint64_t hist_trimmed = 0;
  double range_min = 0, range_max = 0, max_grad = 0;
  void* d_pool = nullptr;
  size_t pool_bytes = 0;
  // macro cells of the LOD-0 bricks
  std::vector<uint64_t> cell_offsets;   // per brick, first cell
  std::vector<uint32_t> cell_counts;    // per brick
  std::vector<uint32_t> cell_dims;      // packed x | y << 10 | z << 20
  uint64_t total_cells = 0;
  void* d_cells = nullptr;              // uint32 per cell
  void* d_cell_meta = nullptr;          // cell offsets (u64) + counts (u32) per brick
  // DynamicBrickingDS volumes: bricks cut from a source volume's bricks
  bool rebricked = false;
  int mm_mode = 0;
  std::vector<uint64_t> src_index;      // source TOC index per brick
  // hardware-filtered copies of every brick (3D CUDA arrays with texture
  // objects), made on a renderer's first frame with hardware filtering on
  mutable std::vector<cudaArray_t> tex_arrays;
  mutable std::vector<cudaTextureObject_t> tex_objs;
  mutable void* d_tex = nullptr;        // the texture objects, TOC order
};

struct tvk_renderer;

namespace tvk {
// The volume's device brick pool; an error once tvk_volume_release_bricks
// moved the bricks to host memory (only a GridLeaper pool paging from its
// pinned host copy renders such a volume).
inline const void* device_bricks(const tvk_volume* V) {
  if (!V->d_pool)
    fail(TVK_ERR_STATE, "the volume's bricks were released from device memory");
  return V->d_pool;
}
}  // namespace tvk

static_assert(sizeof(tvk::DevBrick) == 112, "DevBrick layout is part of the per-frame upload size");
