// tvk_renderer.hpp -- header-only C++ shim over the C ABI (tvk.h) that keeps
// Tuvok's renderer and dataset method names, so code written against
// AbstrRenderer (Renderer/AbstrRenderer.h:112-881) and BrickedDataset
// (IO/BrickedDataset.h:46-96) ports by changing the class names.  Errors throw
// tvk::Exception (the reference throws tuvok::Exception / std::runtime_error
// or returns false with a T_ERROR log).
#ifndef TVK_RENDERER_HPP
#define TVK_RENDERER_HPP

#include <algorithm>
#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "tvk.h"

namespace tvk {

struct Exception : std::runtime_error {
  tvk_status status;
  Exception(tvk_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(tvk_status s) {
  if (s != TVK_OK)
    throw Exception(s, std::string(tvk_status_string(s)) + ": " + tvk_last_error());
}

// IO/Brick.h:57: BrickKey = (timestep, LOD, 1D index)
using BrickKey = std::tuple<uint64_t, uint64_t, uint64_t>;

// A volume bricked on the GPU (the LOD-0 level of what
// ExtendedOctreeConverter::Convert produces, with per-brick statistics).
// UVF::Open's container walk (tvk_uvf_read_blocks): the data blocks in file
// order; *info (optional) receives the global header.
inline std::vector<tvk_uvf_block> ReadUVFBlocks(const std::string& path, uint32_t flags = 0,
                                                tvk_uvf_info* info = nullptr) {
  tvk_uvf_info i;
  check(tvk_uvf_read_blocks(path.c_str(), flags, &i, nullptr, 0));
  std::vector<tvk_uvf_block> blocks(i.block_count);
  check(tvk_uvf_read_blocks(path.c_str(), flags, &i, blocks.data(), i.block_count));
  if (info) *info = i;
  return blocks;
}

class BrickedVolume {
 public:
  BrickedVolume(const void* host_voxels, tvk_dtype dtype, std::array<uint64_t, 3> dims,
                std::array<uint32_t, 3> brick_size, uint32_t overlap, bool clamp_to_edge = false) {
    check(tvk_volume_create(host_voxels, dtype, dims.data(), brick_size.data(), overlap,
                            clamp_to_edge ? 1 : 0, &v_));
  }
  ~BrickedVolume() { tvk_volume_destroy(v_); }
  // tvk_volume_create_ex: TVK_VOLUME_* flags (device input, median LODs, LOD 0 only)
  static std::unique_ptr<BrickedVolume> Create(const void* voxels, tvk_dtype dtype,
                                               std::array<uint64_t, 3> dims,
                                               std::array<uint32_t, 3> brick_size,
                                               uint32_t overlap, uint32_t flags) {
    std::unique_ptr<BrickedVolume> v(new BrickedVolume());
    check(tvk_volume_create_ex(voxels, dtype, dims.data(), brick_size.data(), overlap, flags,
                               &v->v_));
    return v;
  }
  // ExtendedOctree::Open over a converter-written brick file (uncompressed,
  // zlib, LZMA, LZ4 or bzip2 bricks; tvk_volume_open_extended_octree)
  static std::unique_ptr<BrickedVolume> OpenExtendedOctree(const std::string& path,
                                                           uint64_t offset = 0,
                                                           uint32_t uvf_version = 5,
                                                           uint32_t flags = 0) {
    std::unique_ptr<BrickedVolume> v(new BrickedVolume());
    check(tvk_volume_open_extended_octree(path.c_str(), offset, uvf_version, flags, &v->v_));
    return v;
  }
  // UVFDataset::Open of a TOC-block UVF file, timestep `timestep`
  // (tvk_volume_open_uvf; flags as above plus TVK_UVF_VERIFY_CHECKSUM)
  static std::unique_ptr<BrickedVolume> OpenUVF(const std::string& path, uint32_t timestep = 0,
                                                uint32_t flags = 0) {
    std::unique_ptr<BrickedVolume> v(new BrickedVolume());
    check(tvk_volume_open_uvf(path.c_str(), timestep, flags, &v->v_));
    return v;
  }
  // DynamicBrickingDS over this volume (tvk_volume_rebrick)
  static std::unique_ptr<BrickedVolume> Rebrick(const BrickedVolume& src,
                                                std::array<uint32_t, 3> brick_size,
                                                tvk_minmax_mode mode) {
    std::unique_ptr<BrickedVolume> v(new BrickedVolume());
    check(tvk_volume_rebrick(src.v_, brick_size.data(), mode, &v->v_));
    return v;
  }
  std::vector<uint64_t> GetHistogram(size_t bins) const {
    std::vector<uint64_t> h(bins);
    uint64_t used = 0;
    check(tvk_volume_get_histogram(v_, h.data(), bins, &used));
    h.resize(used);
    return h;
  }
  // Out-of-core: frees the device bricks (a host-sourced VolumePool keeps rendering)
  void ReleaseBricks() { check(tvk_volume_release_bricks(v_)); }
  BrickedVolume(const BrickedVolume&) = delete;
  BrickedVolume& operator=(const BrickedVolume&) = delete;

  tvk_volume* handle() const { return v_; }

  tvk_volume_info Info() const {
    tvk_volume_info i;
    check(tvk_volume_get_info(v_, &i));
    return i;
  }
  std::pair<double, double> GetRange() const {
    const tvk_volume_info i = Info();
    return {i.range_min, i.range_max};
  }
  float MaxGradientMagnitude() const { return float(Info().max_gradient); }
  uint64_t GetLODLevelCount() const { return Info().lod_count; }
  std::array<uint64_t, 3> GetDomainSize(uint32_t lod = 0) const {
    std::array<uint64_t, 3> s, b;
    check(tvk_volume_get_lod(v_, lod, s.data(), b.data()));
    return s;
  }
  std::array<uint64_t, 3> GetBrickLayout(uint32_t lod = 0) const {
    std::array<uint64_t, 3> s, b;
    check(tvk_volume_get_lod(v_, lod, s.data(), b.data()));
    return b;
  }
  tvk_brick_md GetBrickMetadata(const BrickKey& k) const {
    tvk_brick_md m;
    check(tvk_volume_get_brick_md(v_, std::get<0>(k), std::get<1>(k), std::get<2>(k), &m));
    return m;
  }
  template <class T>
  bool GetBrick(const BrickKey& k, std::vector<T>& out) const {
    const tvk_brick_md m = GetBrickMetadata(k);
    out.resize(size_t(m.n_voxels[0]) * m.n_voxels[1] * m.n_voxels[2]);
    check(tvk_volume_get_brick(v_, std::get<0>(k), std::get<1>(k), std::get<2>(k), out.data(),
                               out.size() * sizeof(T)));
    return true;
  }
  tvk_minmax MaxMinForKey(const BrickKey& k) const {
    tvk_minmax m;
    check(tvk_volume_get_minmax(v_, std::get<0>(k), std::get<1>(k), std::get<2>(k), &m));
    return m;
  }
  BrickKey IndexFrom4D(uint64_t x, uint64_t y, uint64_t z, uint64_t lod,
                       uint64_t timestep = 0) const {
    const uint64_t xyzl[4] = {x, y, z, lod};
    uint64_t idx = 0;
    check(tvk_volume_index_from_4d(v_, xyzl, &idx));
    return BrickKey(timestep, lod, idx);
  }

 private:
  BrickedVolume() = default;
  tvk_volume* v_ = nullptr;
};

// The renderer, named after AbstrRenderer's methods.
// IO/TransferFunction1D.h:53-101 over the C ABI's table functions: the same
// methods, each giving the reference's table bit for bit.
class TransferFunction1D {
 public:
  explicit TransferFunction1D(size_t iSize = 0) : data_(4 * iSize, 0.0f) {}
  explicit TransferFunction1D(const std::string& filename) { Load(filename); }

  size_t GetSize() const { return data_.size() / 4; }
  void Resize(size_t iSize) { data_.resize(4 * iSize, 0.0f); }
  void SetStdFunction(float fCenterPoint = 0.5f, float fInvGradient = 0.5f) {
    check(tvk_tf1d_set_std_function(data_.data(), GetSize(), fCenterPoint, fInvGradient, -1, 0));
    ComputeNonZeroLimits();
  }
  void SetStdFunction(float fCenterPoint, float fInvGradient, int iComponent, bool bInvertedStep) {
    check(tvk_tf1d_set_std_function(data_.data(), GetSize(), fCenterPoint, fInvGradient,
                                    iComponent, bInvertedStep ? 1 : 0));
    ComputeNonZeroLimits();
  }
  void Set(const std::vector<unsigned char>& tf) {
    std::vector<float> t(tf.size() / 4 * 4);
    check(tvk_tf1d_from_bytes(tf.data(), tf.size() / 4, t.data()));
    data_.swap(t);
    ComputeNonZeroLimits();
  }
  void Resample(size_t iTargetSize) {
    if (iTargetSize == GetSize()) return;  // the reference returns before recomputing the limits
    std::vector<float> t(4 * iTargetSize);
    check(tvk_tf1d_resample(data_.data(), GetSize(), t.data(), iTargetSize));
    data_.swap(t);
    ComputeNonZeroLimits();
  }
  void FillOrTruncate(size_t iTargetSize) {
    std::vector<float> t(4 * iTargetSize);
    check(tvk_tf1d_fill_or_truncate(data_.data(), GetSize(), t.data(), iTargetSize));
    data_.swap(t);
    ComputeNonZeroLimits();
  }
  void Clear() {
    std::fill(data_.begin(), data_.end(), 0.0f);
    limits_ = {0, 0};
  }
  void ComputeNonZeroLimits() {
    uint64_t l[2];
    check(tvk_tf1d_nonzero_limits(data_.data(), GetSize(), l));
    limits_ = {l[0], l[1]};
  }
  const std::array<uint64_t, 2>& GetNonZeroLimits() const { return limits_; }
  std::array<float, 4> GetColor(size_t i) const {
    return {data_[4 * i], data_[4 * i + 1], data_[4 * i + 2], data_[4 * i + 3]};
  }
  void SetColor(size_t i, const std::array<float, 4>& c) {
    for (int k = 0; k < 4; ++k) data_[4 * i + k] = c[k];
  }
  const std::vector<float>& GetColorData() const { return data_; }
  void GetByteArray(std::vector<unsigned char>& v, unsigned char cUsedRange = 255) const {
    v.resize(data_.size());
    check(tvk_tf1d_byte_array(data_.data(), GetSize(), cUsedRange, v.data()));
  }
  bool Load(const std::string& filename) {
    uint64_t n = 0;
    if (tvk_tf1d_load(filename.c_str(), nullptr, 0, &n) != TVK_OK) return false;
    std::vector<float> t(4 * n);
    if (tvk_tf1d_load(filename.c_str(), t.data(), n, &n) != TVK_OK) return false;
    data_.swap(t);
    ComputeNonZeroLimits();
    return true;
  }
  bool Load(const std::string& filename, size_t iTargetSize) {
    if (!Load(filename)) return false;
    Resample(iTargetSize);
    return true;
  }
  bool Save(const std::string& filename) const {
    return tvk_tf1d_save(filename.c_str(), data_.data(), GetSize()) == TVK_OK;
  }

 private:
  std::vector<float> data_;
  std::array<uint64_t, 2> limits_{{0, 0}};
};

class Renderer {
 public:
  enum ERenderMode { RM_1DTRANS = TVK_RM_1DTRANS, RM_2DTRANS = TVK_RM_2DTRANS,
                     RM_ISOSURFACE = TVK_RM_ISOSURFACE };

  Renderer() { check(tvk_renderer_create(&r_)); }
  ~Renderer() { tvk_renderer_destroy(r_); }
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;

  bool RegisterDataset(const BrickedVolume& v) {
    check(tvk_renderer_set_volume(r_, v.handle()));
    return true;
  }
  // AbstrRenderer::Set1DTrans(const std::vector<unsigned char>&)
  void Set1DTrans(const std::vector<unsigned char>& rgba) {
    check(tvk_set_tf1d_rgba8(r_, rgba.data(), uint32_t(rgba.size() / 4)));
  }
  void Set1DTransFloat(const std::vector<float>& rgba, bool rgba8_upload = false) {
    check(tvk_set_tf1d_float(r_, rgba.data(), uint32_t(rgba.size() / 4), rgba8_upload));
  }
  // AbstrRenderer::Changed1DTrans after editing the TransferFunction1D: the
  // reference uploads its bytes (GetByteArray) as GL_RGBA8
  void Set1DTrans(const TransferFunction1D& tf) { Set1DTransFloat(tf.GetColorData(), true); }
  void Set2DTransFloat(const std::vector<float>& rgba, uint32_t w, uint32_t h) {
    check(tvk_set_tf2d_float(r_, rgba.data(), w, h, 0));
  }
  void SetRendermode(ERenderMode m) { check(tvk_set_render_mode(r_, tvk_render_mode(m))); }
  void SetUseLighting(bool on) { check(tvk_set_lighting(r_, on ? 1 : 0)); }
  void SetSampleRateModifier(float f) { check(tvk_set_sample_rate_modifier(r_, f)); }
  // texture-unit trilinear lookups instead of the exact ones (faster, not bit-exact)
  void SetHardwareFiltering(bool on) { check(tvk_set_hardware_filtering(r_, on ? 1 : 0)); }
  void SetIsoValue(float v) { check(tvk_set_isovalue(r_, v)); }
  void SetColors(const float ambient[4], const float diffuse[4], const float specular[4],
                 const float light_dir[3]) {
    check(tvk_set_colors(r_, ambient, diffuse, specular, light_dir));
  }
  void SetViewParameters(float fov, float znear, float zfar, const float eye[3],
                         const float at[3], const float up[3]) {
    check(tvk_set_view(r_, eye, at, up, fov, znear, zfar));
  }
  void Resize(uint32_t w, uint32_t h) {
    check(tvk_resize(r_, w, h));
    w_ = w;
    h_ = h;
  }
  bool Paint() {
    check(tvk_paint(r_));
    return true;
  }
  // GLRenderer::GetLastFBO + GLFBOTex::ReadBackPixels
  std::vector<float> ReadBackPixels() {
    std::vector<float> img(size_t(w_) * h_ * 4);
    check(tvk_read_image(r_, img.data(), img.size()));
    return img;
  }
  // copies the last frame into rgba (w x h x 4 floats, valid until WaitImage)
  // while later frames render
  void ReadBackPixelsAsync(float* rgba, size_t n_floats) {
    check(tvk_read_image_async(r_, rgba, n_floats));
  }
  void WaitImage() { check(tvk_wait_image(r_)); }
  tvk_stats Stats() {
    tvk_stats s;
    check(tvk_get_stats(r_, &s));
    return s;
  }
  // AbstrRenderer::SetClipPlane / EnableClipPlane / DisableClipPlane (world space)
  void SetClipPlane(const float plane[4]) { check(tvk_set_clip_plane(r_, plane)); }
  void EnableClipPlane() { check(tvk_enable_clip_plane(r_, 1)); }
  void DisableClipPlane() { check(tvk_enable_clip_plane(r_, 0)); }
  // AbstrRenderer::SetScalingMethod
  void SetScalingMethod(tvk_scaling_method m) { check(tvk_set_scaling_method(r_, m)); }
  // AbstrRenderer::SetCV, SetCVIsoValue, SetCVColor, SetCVSize /
  // SetCVContextScale / SetCVBorderScale, SetCVFocusPosFVec, SetCVFocusPos
  void SetCV(bool enable) { check(tvk_set_clearview(r_, enable ? 1 : 0)); }
  void SetCVIsoValue(float isovalue) { check(tvk_set_cv_isovalue(r_, isovalue)); }
  void SetCVColor(const float rgb[3]) { check(tvk_set_cv_color(r_, rgb)); }
  void SetCVParams(float size, float context_scale, float border_scale) {
    check(tvk_set_cv_params(r_, size, context_scale, border_scale));
  }
  void SetCVFocusPosFVec(const float pos[4]) { check(tvk_set_cv_focus_pos(r_, pos)); }
  void SetCVFocusPos(uint32_t x, uint32_t y) { check(tvk_set_cv_focus_pixel(r_, x, y)); }
  // m_iCurrentLOD, decreaseScreenResNow / decreaseSamplingRateNow
  void SetLOD(uint32_t lod) { check(tvk_set_lod(r_, lod)); }
  void SetReducedQuality(bool screen, bool sampling) {
    check(tvk_set_reduced_quality(r_, screen ? 1 : 0, sampling ? 1 : 0));
  }
  // AbstrRenderer::SetPerfMeasures / SetLODLimits / ComputeMinLODForCurrentView
  void SetPerfMeasures(uint32_t min_framerate, bool low_res_intermediate,
                       float screen_res_dec_factor = 2.0f, float sample_dec_factor = 2.0f) {
    check(tvk_set_perf_measures(r_, min_framerate, low_res_intermediate ? 1 : 0,
                                screen_res_dec_factor, sample_dec_factor));
  }
  void SetLODLimits(uint32_t coarsest_skip, uint32_t finest) {
    check(tvk_set_lod_limits(r_, coarsest_skip, finest));
  }
  uint32_t ComputeMinLODForCurrentView() {
    uint32_t l = 0;
    check(tvk_compute_min_lod(r_, &l));
    return l;
  }
  // One subframe of the progressive frame (PlanFrame)
  tvk_subframe_info PaintProgressive(bool new_frame) {
    tvk_subframe_info i;
    check(tvk_paint_progressive(r_, new_frame ? 1 : 0, &i));
    return i;
  }
  tvk_renderer* handle() const { return r_; }

 private:
  tvk_renderer* r_ = nullptr;
  uint32_t w_ = 0, h_ = 0;
};

// Several renderers' frames in one persistent launch replayed from a CUDA
// graph (the reference paints render regions one after another,
// GLRenderer.cpp:622-660).
class BatchPainter {
 public:
  BatchPainter() { check(tvk_batch_create(&b_)); }
  ~BatchPainter() { tvk_batch_destroy(b_); }
  BatchPainter(const BatchPainter&) = delete;
  BatchPainter& operator=(const BatchPainter&) = delete;
  void SetAutotune(bool on, uint32_t ctas_per_sm = 0) {
    check(tvk_batch_set_autotune(b_, on ? 1 : 0, ctas_per_sm));
  }
  void SetRaysPerThread(uint32_t rays) { check(tvk_batch_set_rays_per_thread(b_, rays)); }
  void Paint(const std::vector<Renderer*>& rs) {
    std::vector<tvk_renderer*> h;
    for (Renderer* r : rs) h.push_back(r->handle());
    check(tvk_paint_batch(b_, h.data(), uint32_t(h.size())));
  }
  tvk_batch_info Info() {
    tvk_batch_info i;
    check(tvk_batch_get_info(b_, &i));
    return i;
  }

 private:
  tvk_batch* b_ = nullptr;
};

// The learned reconstruction: reduced frame + tensor-core U-Net + probe judge
// with fallback to the plain frame.
class LearnedReconstruction {
 public:
  explicit LearnedReconstruction(const std::vector<float>& params) {
    check(tvk_learned_create(params.data(), params.size(), &n_));
  }
  ~LearnedReconstruction() { tvk_learned_destroy(n_); }
  LearnedReconstruction(const LearnedReconstruction&) = delete;
  LearnedReconstruction& operator=(const LearnedReconstruction&) = delete;
  static size_t ParamCount() {
    size_t n = 0;
    check(tvk_learned_param_count(&n));
    return n;
  }
  tvk_learned_info Paint(Renderer& r, float threshold_db) {
    tvk_learned_info i;
    check(tvk_paint_learned(r.handle(), n_, threshold_db, &i));
    return i;
  }

 private:
  tvk_learned* n_ = nullptr;
};

// GLVolumePool + GLHashTable + GLGridLeaper::Render3DRegion: the LOD brick
// cache of a volume and the GridLeaper frame over it.
class VolumePool {
 public:
  VolumePool(const BrickedVolume& v, uint64_t budget_bytes, bool host_source) {
    check(tvk_pool_create(v.handle(), budget_bytes, host_source ? 1 : 0, &p_));
  }
  ~VolumePool() { tvk_pool_destroy(p_); }
  VolumePool(const VolumePool&) = delete;
  VolumePool& operator=(const VolumePool&) = delete;
  tvk_pool_info Info() const {
    tvk_pool_info i;
    check(tvk_pool_get_info(p_, &i));
    return i;
  }
  std::vector<uint32_t> PageTable() const {
    std::vector<uint32_t> t(Info().bricks);
    check(tvk_pool_get_page_table(p_, t.data(), t.size()));
    return t;
  }
  void Reset() { check(tvk_pool_reset(p_)); }  // PH_Reset
  void SetRequestTable(uint32_t size, uint32_t rehash) {
    check(tvk_pool_set_request_table(p_, size, rehash));
  }
  // Render3DRegion's subframes until converged or max_passes
  tvk_leaper_info Paint(Renderer& r, uint32_t max_passes) {
    tvk_leaper_info i;
    check(tvk_leaper_paint(r.handle(), p_, max_passes, &i));
    return i;
  }

 private:
  tvk_pool* p_ = nullptr;
};

}  // namespace tvk

#endif  // TVK_RENDERER_HPP
