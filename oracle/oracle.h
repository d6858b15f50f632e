/*
 * oracle.h -- CPU restatement of Tuvok's volume-rendering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path of
 * tuvok_gb300 is compared against.  Only the test suite, the smoke check and the
 * CPU-baseline leg of bench.py load it; the product library never links or calls
 * it, and nothing it computes is ever shipped as a result.
 *
 * Every function states the reference file:line it restates (paths are relative
 * to the Tuvok source tree).  Parity of the bricking/statistics half is pinned
 * against the reference's own ExtendedOctreeConverter (built from the reference
 * sources by oracle/ref/Makefile) and the golden vectors of IO/test/rebricking.h.
 * The rendering half restates GLSL that can only run through OpenGL; no golden
 * images exist in the reference, so its parity is pinned only by this
 * restatement (stated in the test headers).
 */
#ifndef TVK_ORACLE_H
#define TVK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- LOD table / brick geometry (IO/UVF/ExtendedOctree/ExtendedOctree.cpp) ---- */

/* ExtendedOctree::ComputeMetadata (ExtendedOctree.cpp:188-243).  Writes up to
 * max_lods entries of per-LOD voxel sizes (3 x u64) and brick counts (3 x u64).
 * Returns the LOD count. */
int orc_lod_table(const uint64_t dims[3], const uint32_t brick_size[3],
                  uint32_t overlap, uint64_t* lod_sizes, uint64_t* brick_counts,
                  int max_lods);

/* The aspect of LOD `lod` as ExtendedOctree::ComputeMetadata accumulates it
 * (ExtendedOctree.cpp:188-243; GetBrickAspect :292-294). */
void orc_lod_aspect(const uint64_t dims[3], uint32_t lod, double out[3]);

/* ExtendedOctree::ComputeBrickSize (ExtendedOctree.cpp:276-285). */
void orc_brick_size(const uint64_t lod_size[3], const uint64_t brick_count[3],
                    const uint32_t brick_size[3], uint32_t overlap,
                    const uint64_t coords[3], uint64_t out[3]);

/* ExtendedOctreeConverter::GetInputBrick + ClampToEdge
 * (ExtendedOctreeConverter.cpp:288-373, 376-462): one LOD-0 brick including its
 * overlap, x fastest.  dtype 0 = u8, 1 = u16.  `out` holds the brick's voxels. */
void orc_lod0_brick(const void* raw, int dtype, const uint64_t dims[3],
                    const uint32_t brick_size[3], uint32_t overlap,
                    int clamp_to_edge, const uint64_t coords[3], void* out);

/* ExtendedOctreeConverter::ComputeBrickStats<T> (ExtendedOctreeConverter.inc:408-444). */
void orc_brick_stats(const void* brick, int dtype, uint64_t n_voxels,
                     double* min_out, double* max_out);

/* Histogram1DDataBlock::ComputeTemplate<T> (Histogram1DDataBlock.cpp:120-161):
 * histogram of the inner voxels of every LOD-0 brick.  `hist` has 2^(8*bytes)
 * bins.  Returns the trimmed length (last non-zero bin + 1). */
uint64_t orc_histogram1d(const void* raw, int dtype, const uint64_t dims[3],
                         const uint32_t brick_size[3], uint32_t overlap,
                         uint64_t* hist);

/* Per-brick 256-bin histogram of a brick's inner voxels (new in this build:
 * the reference keeps only the global histogram).  bin = value >> shift. */
void orc_brick_hist256(const void* brick, int dtype, const uint64_t n[3],
                       uint32_t overlap, uint32_t shift, uint32_t* hist);

/* UVFDataset::ComputeMetadataTOC (uvfDataset.cpp:242-288) for LOD `lod`:
 * per-brick centre/extents (float, model space) and n_voxels, in brick index
 * order z*bx*by + y*bx + x.  aspect = per-axis LOD aspect (1 at LOD 0). */
void orc_brick_metadata(const uint64_t lod_size[3], const uint64_t brick_count[3],
                        const uint32_t brick_size[3], uint32_t overlap,
                        const double aspect[3], float* centers, float* extents,
                        uint32_t* n_voxels);

/* ExtendedOctreeConverter::Convert's whole octree (ExtendedOctreeConverter.cpp:
 * 128-280): LOD 0 by orc_lod0_brick, every coarser LOD by DownsampleBrick /
 * DownsampleBricktoBrick (.inc:1-356; mean in double truncated to T, or the
 * 7-value median network of VolumeTools::Filter) followed by FillOverlap
 * (.cpp:1203-1372) in the reference's sequential order.  Bricks are written
 * back to back in TOC order (LOD-major, then z, y, x) into `pool`;
 * brick_offsets (voxels) gets one entry per brick.  Ghost voxels the reference
 * leaves holding a previous brick's bytes (clamp mode only) are zero here.
 * Returns the brick count, or -1 if pool_voxels or max_bricks is too small. */
int64_t orc_build_octree(const void* raw, int dtype, const uint64_t dims[3],
                         const uint32_t brick_size[3], uint32_t overlap, int clamp_to_edge,
                         int median, void* pool, uint64_t pool_voxels,
                         uint64_t* brick_offsets, uint64_t max_bricks);

/* MaxGradientMagnitude as Histogram2DDataBlock::ComputeTemplate<T> finds it
 * (Histogram2DDataBlock.cpp:327-345, 363-397). */
double orc_max_gradient(const void* raw, int dtype, const uint64_t dims[3],
                        const uint32_t brick_size[3], uint32_t overlap,
                        int clamp_to_edge);

/* The 2D value x |gradient| histogram of Histogram2DDataBlock::ComputeTemplate<T>
 * (Histogram2DDataBlock.cpp:349-438): `hist` holds value_bins rows of 256
 * gradient bins.  Returns the maximum gradient magnitude. */
double orc_histogram2d(const void* raw, int dtype, const uint64_t dims[3],
                       const uint32_t brick_size[3], uint32_t overlap, int clamp_to_edge,
                       uint64_t value_bins, double max_nonzero, uint64_t* hist);

/* ---- DynamicBrickingDS (IO/DynamicBrickingDS.cpp) ---- */

/* Re-cuts a bricked source (pool + TOC offsets as orc_build_octree writes them,
 * n_built_lods LODs present, per-brick min/max) into bricks of tgt_brick voxels
 * (ghost included).  Per target brick t in TOC order: info[4t..] = lod,
 * n_voxels x/y/z; geom[6t..] = centre xyz, extents xyz; src_index[t] = source
 * TOC index; minmax[2t..] = MaxMinForKey for mm_mode (0 MM_SOURCE, 1
 * MM_PRECOMPUTE, 2 MM_DYNAMIC); voxels at out_pool + out_offsets[t].  Only
 * bricks that fit max_out / pool_cap are written.  Returns the target brick
 * count (*pool_needed = voxels of all of them), -1 where the reference throws
 * (not an integer multiple), -2 where its copy would read outside a source
 * brick. */
int64_t orc_rebrick(int dtype, const uint64_t dims[3], const uint32_t src_brick[3],
                    uint32_t overlap, uint32_t n_built_lods, const void* src_pool,
                    const uint64_t* src_offsets, const double* src_min, const double* src_max,
                    const uint32_t tgt_brick[3], int mm_mode, uint64_t max_out, uint32_t* info,
                    float* geom, uint64_t* src_index, double* minmax, void* out_pool,
                    uint64_t pool_cap, uint64_t* out_offsets, uint64_t* pool_needed);

/* ---- Ray march (Shaders/GLRaycaster-*.glsl) ---- */

enum { ORC_RM_1D = 0, ORC_RM_2D = 1, ORC_RM_ISO = 2 };
enum { ORC_LIGHT_REFERENCE = 0, ORC_LIGHT_BLINN_PHONG = 1 };

typedef struct orc_scene {
  /* volume, bricked by the oracle itself */
  const void* raw;
  int dtype;                /* 0 = u8, 1 = u16, 2 = RGBA8 colour (LOD 0 only) */
  uint64_t dims[3];
  uint32_t brick_size[3];   /* including overlap, as Tuvok counts it */
  uint32_t overlap;
  int clamp_to_edge;
  double user_scale[3];     /* Dataset::GetScale, normally 1 */
  /* transfer function: RGBA float table; tf_rgba8 != 0 reproduces the GL_RGBA8
   * upload (truncate x255, /255 on lookup) */
  const float* tf;
  uint32_t tf_w, tf_h;      /* tf_h = 1 for 1D */
  int tf_rgba8;
  int render_mode;          /* ORC_RM_* */
  int lighting;
  int light_model;          /* ORC_LIGHT_* */
  float ambient[4], diffuse[4], specular[4], light_dir[3];
  float bp_ka, bp_kd, bp_ks, bp_shininess;
  float isovalue;           /* iso mode: data units */
  float sample_rate_modifier;
  float frame_ert;          /* stop visiting bricks once frame alpha >= this; 1 = never */
  /* camera: Tuvok's SetViewParameters + BuildLookAt + Perspective */
  float eye[3], at[3], up[3];
  float fovy_deg, znear, zfar;
  uint32_t width, height;
  int use_double;           /* 1: evaluate the march in FP64 (error reporting) */
  /* optional: render only rows with y % row_stride == row_phase (CPU baseline) */
  uint32_t row_stride, row_phase;
  int threads;              /* OpenMP threads, 0 = default */
  float iso_color[3];       /* AbstrRenderer m_vIsoColor (default 0.5 grey) */
  /* level of detail and reduced quality (AbstrRenderer m_iCurrentLOD,
   * decreaseScreenResNow / decreaseSamplingRateNow and their factors) */
  uint32_t lod;             /* LOD >= 1 bricks come from orc_build_octree */
  int median;               /* ComputeHierarchy filter of those LODs */
  int decrease_screen_res, decrease_sampling_rate;
  float screen_res_dec_factor, sample_dec_factor;
  /* AbstrRenderer's clip plane (SetClipPlane / EnableClipPlane): a, b, c, d
   * in world (= model) space; points with n.x + d >= 0, n = normalize(a, b, c),
   * are cut away (PLANE::clip, Basics/Vectors.h:1455-1457) */
  int clip_on;
  float clip_plane[4];
  /* ClearView in iso mode (AbstrRenderer SetCV and its m_fCVIsovalue,
   * m_vCVColor, m_fCVSize, m_fCVContextScale, m_fCVBorderScale, m_vCVPos):
   * the focus isosurface behind the context surface, composed by
   * Compose-CV-FS.glsl.  cv_pos is model space (w = 0: a direction) */
  int cv_on;
  float cv_isovalue;        /* data units */
  float cv_color[3];
  float cv_size, cv_context_scale, cv_border_scale;
  float cv_pos[4];
  /* AbstrRenderer SMETH_BIAS_AND_SCALE in 1D mode: fTransScale = |min| + |max|
   * of the data range (GLRaycaster.cpp:577-584; the bias is never applied) */
  int tf_bias_scale;
} orc_scene;

/* Renders the scene; out_rgba is width*height*4 floats, row 0 = bottom row
 * (gl_FragCoord.y = 0.5).  Returns the number of executed samples; the sample
 * count of each pixel goes to samples_per_pixel when it is not NULL.  With
 * decrease_screen_res the march runs at the reduced size (the counts are of
 * that image, orc_render_size) and is stretched bilinearly over the viewport. */
void orc_render_size(const orc_scene* scene, uint32_t* width, uint32_t* height);

uint64_t orc_render(const orc_scene* scene, float* out_rgba,
                    uint32_t* samples_per_pixel);

/* orc_render with the wall time of the set-up (bricking, statistics) and of
 * the march itself. */
uint64_t orc_render_timed(const orc_scene* scene, float* out_rgba,
                          uint32_t* samples_per_pixel, double* setup_s, double* march_s);

/* Bricks the scene's volume once (returns a handle) so that several cameras
 * can be rendered without repeating the set-up; orc_render_prepared takes the
 * camera, viewport, row selection, threads and precision from `cam`. */
void* orc_prepare(const orc_scene* scene);
uint64_t orc_render_prepared(void* prepared, const orc_scene* cam, float* out_rgba,
                             uint32_t* samples_per_pixel, double* march_s);
void orc_release(void* prepared);

/* One GridLeaper pass (GLGridLeaper-blend.glsl / -iso.glsl) of the scene over a
 * page table with one entry per brick of every LOD in TOC order (0 MISSING,
 * 1 CHILD_EMPTY, 2 EMPTY, >= 3 resident), the bricks built by
 * orc_build_octree.  Writes the image and per-pixel samples; the bricks the
 * rays reported missing go to `missing` (ascending TOC index).  Returns the
 * number of samples. */
uint64_t orc_leaper_render(const orc_scene* scene, const uint32_t* page, uint64_t n_page,
                           float* out_rgba, uint32_t* samples_per_pixel, uint64_t* missing,
                           uint64_t max_missing, uint64_t* n_missing);

/* IEEE binary16 round-to-nearest-even of a float, returned as float (the
 * RGBA16F ray-entry buffer of GLRaycaster.cpp:97). */
float orc_round_half(float x);

/* ---- Synthetic inputs (CPU twin of the GPU generator; input creation only) ---- */
void orc_generate_blobs(void* out, int dtype, const uint64_t dims[3],
                        const float* blobs, uint32_t n_blobs, float noise_amp,
                        uint32_t noise_octaves, float noise_cell, uint64_t seed,
                        int int_noise, float vmax, int threads);

#ifdef __cplusplus
}
#endif

#endif
