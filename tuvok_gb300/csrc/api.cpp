// api.cpp -- C ABI of tuvok_gb300: volumes (GPU bricking) and renderers (GPU
// ray march) with the host-side planning of Tuvok's AbstrRenderer.
//
// Host arithmetic that feeds the kernels (brick metadata, texture matrices, step
// sizes, transfer-function tables) follows the reference's own evaluation order
// and is compiled with -ffp-contract=off, so the values handed to the GPU do not
// depend on the host compiler or CPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "tvk_internal.h"

namespace tvk {

namespace {
thread_local std::string g_last_error;
}

void fail(tvk_status s, const std::string& msg) { throw Error{s, msg}; }

void set_last_error(const std::string& msg) { g_last_error = msg; }

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  const tvk_status s = (e == cudaErrorMemoryAllocation) ? TVK_ERR_OUT_OF_MEMORY : TVK_ERR_CUDA;
  fail(s, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class F>
tvk_status guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return TVK_OK;
  } catch (const Error& e) {
    g_last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return TVK_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return TVK_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown failure";
    return TVK_ERR_INTERNAL;
  }
}

#define REQUIRE(cond, msg) \
  do {                     \
    if (!(cond)) ::tvk::fail(TVK_ERR_INVALID_ARG, msg); \
  } while (0)

// Device buffer owned by RAII.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void ensure(size_t n) {
    if (n <= bytes && p) return;
    release();
    TVK_CUDA(cudaMalloc(&p, n ? n : 1));
    bytes = n;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { if (p) cudaFreeHost(p); }
  void ensure(size_t n) {
    if (n <= bytes && p) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    TVK_CUDA(cudaMallocHost(&p, n ? n : 1));
    bytes = n;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// ------------------------------------------------------------ LOD / metadata

// ExtendedOctree::ComputeMetadata (IO/UVF/ExtendedOctree/ExtendedOctree.cpp:188-243).
std::vector<LodInfo> lod_table(const uint64_t dims[3], const uint32_t B[3], uint32_t ov) {
  std::vector<LodInfo> t;
  uint64_t v[3] = {dims[0], dims[1], dims[2]};
  double asp[3] = {1, 1, 1};
  const uint64_t usable[3] = {B[0] - 2ull * ov, B[1] - 2ull * ov, B[2] - 2ull * ov};
  do {
    LodInfo l;
    if (!t.empty()) {
      for (int a = 0; a < 3; ++a) {
        if (v[a] > 1) {
          const uint64_t h = uint64_t(std::ceil(v[a] / 2.0));
          asp[a] *= (v[a] % 2) ? double(float(v[a]) / float(h)) : 2.0;
          v[a] = h;
        }
      }
      const double m = std::max(asp[0], std::max(asp[1], asp[2]));
      for (int a = 0; a < 3; ++a) asp[a] /= m;
    }
    for (int a = 0; a < 3; ++a) {
      l.size[a] = v[a];
      l.bricks[a] = uint64_t(std::ceil(v[a] / double(usable[a])));
      l.aspect[a] = asp[a];
    }
    t.push_back(l);
  } while (v[0] > 1 || v[1] > 1 || v[2] > 1);
  return t;
}

// ExtendedOctree::ComputeBrickSize (ExtendedOctree.cpp:276-285).
void brick_size(const LodInfo& l, const uint32_t B[3], uint32_t ov, const uint64_t c[3],
                uint32_t out[3]) {
  for (int a = 0; a < 3; ++a) {
    const uint64_t core = B[a] - 2ull * ov;
    const bool last = c[a] == l.bricks[a] - 1;
    out[a] = uint32_t((last && (l.size[a] % core)) ? (2ull * ov + l.size[a] % core) : B[a]);
  }
}

// UVFDataset::ComputeMetadataTOC (IO/uvfDataset.cpp:242-288): x, y, z loop
// order, corner accumulated in float.
void brick_metadata(const LodInfo& l, const uint32_t B[3], uint32_t ov,
                    std::vector<tvk_brick_md>& md) {
  md.assign(l.bricks[0] * l.bricks[1] * l.bricks[2], tvk_brick_md{});
  const float asp[3] = {float(l.aspect[0]), float(l.aspect[1]), float(l.aspect[2])};
  float nd[3] = {float(l.size[0]) * asp[0], float(l.size[1]) * asp[1], float(l.size[2]) * asp[2]};
  const float maxv = std::max(nd[0], std::max(nd[1], nd[2]));
  for (int a = 0; a < 3; ++a) nd[a] /= maxv;
  float corner[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
  for (uint64_t x = 0; x < l.bricks[0]; ++x) {
    corner[1] = 0;
    for (uint64_t y = 0; y < l.bricks[1]; ++y) {
      corner[2] = 0;
      for (uint64_t z = 0; z < l.bricks[2]; ++z) {
        const uint64_t c[3] = {x, y, z};
        uint32_t bs[3];
        brick_size(l, B, ov, c, bs);
        tvk_brick_md& m = md[z * l.bricks[0] * l.bricks[1] + y * l.bricks[0] + x];
        for (int a = 0; a < 3; ++a) {
          ext[a] = float(bs[a] - 2u * ov) * asp[a] / maxv;
          m.center[a] = (corner[a] + ext[a] / 2.0f) - nd[a] * 0.5f;
          m.extents[a] = ext[a];
          m.n_voxels[a] = bs[a];
        }
        corner[2] += ext[2];
      }
      corner[1] += ext[1];
    }
    corner[0] += ext[0];
  }
}

uint32_t bits_of(uint64_t v) {
  uint32_t b = 0;
  while (v) { ++b; v >>= 1; }
  return b;
}

// ------------------------------------------------------------ volume build

void build_volume(tvk_volume* V, const void* d_raw, cudaStream_t s) {
  const uint64_t nvox = V->dims[0] * V->dims[1] * V->dims[2];
  uint64_t launches = 0;
  V->lods = lod_table(V->dims, V->brick_size, V->overlap);
  const LodInfo& l0 = V->lods[0];
  V->n_bricks = l0.bricks[0] * l0.bricks[1] * l0.bricks[2];
  REQUIRE(V->n_bricks < (1ull << 31), "too many bricks");
  // bricks of every LOD in TOC order (LOD-major, then z, y, x); LOD 0 first
  const size_t n_lods = V->build_lods ? V->lods.size() : 1;
  V->lod_first.assign(1, 0);
  V->md.clear();
  for (size_t l = 0; l < n_lods; ++l) {
    std::vector<tvk_brick_md> m;
    brick_metadata(V->lods[l], V->brick_size, V->overlap, m);
    V->md.insert(V->md.end(), m.begin(), m.end());
    V->lod_first.push_back(V->md.size());
  }
  V->total_bricks = V->md.size();
  V->offsets.resize(V->total_bricks);
  V->sizes.resize(3 * V->total_bricks);
  std::vector<uint64_t> voxels(V->total_bricks);
  const uint64_t align = 256 / V->bytes;  // brick starts on 256-byte boundaries
  uint64_t off = 0;
  uint32_t max_bz = 0;
  for (uint64_t b = 0; b < V->total_bricks; ++b) {
    for (int a = 0; a < 3; ++a) V->sizes[3 * b + a] = V->md[b].n_voxels[a];
    if (b < V->n_bricks) max_bz = std::max(max_bz, V->md[b].n_voxels[2]);
    V->offsets[b] = off;
    voxels[b] = uint64_t(V->sizes[3 * b]) * V->sizes[3 * b + 1] * V->sizes[3 * b + 2];
    off += (voxels[b] + align - 1) / align * align;
  }
  V->pool_bytes = off * V->bytes;
  TVK_CUDA(cudaMalloc(&V->d_pool, V->pool_bytes));

  DevBuf d_off, d_sizes, d_scratch, d_vox;
  d_off.ensure(V->total_bricks * sizeof(uint64_t));
  d_sizes.ensure(V->total_bricks * 3 * sizeof(uint32_t));
  d_vox.ensure(V->total_bricks * sizeof(uint64_t));
  TVK_CUDA(cudaMemcpyAsync(d_off.p, V->offsets.data(), V->total_bricks * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemcpyAsync(d_sizes.p, V->sizes.data(), V->total_bricks * 3 * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemcpyAsync(d_vox.p, voxels.data(), V->total_bricks * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));
  if (V->dtype == TVK_RGBA8) {
    // colour volumes: the bricks of every LOD, each channel filtered on its
    // own.  Channel range of 8-bit data; no histograms, gradients or macro
    // cells (colour bricks are never empty).
    BrickGrid g;
    for (int a = 0; a < 3; ++a) {
      g.dims[a] = V->dims[a];
      g.B[a] = V->brick_size[a];
      g.cnt[a] = uint32_t(l0.bricks[a]);
    }
    g.ov = V->overlap;
    g.clamp = V->clamp ? 1 : 0;
    g.total = nvox;
    launch_brick_copy4(d_raw, g, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(), V->n_bricks,
                       V->d_pool, s, &launches);
    if (V->total_bricks > V->n_bricks) {
      DevBuf d_wave;
      uint64_t max_lod_bricks = 0;
      for (size_t l = 1; l < n_lods; ++l)
        max_lod_bricks = std::max<uint64_t>(max_lod_bricks, V->lod_first[l + 1] - V->lod_first[l]);
      d_wave.ensure(max_lod_bricks * sizeof(uint32_t));
      std::vector<LodInfo> built(V->lods.begin(), V->lods.begin() + n_lods);
      build_lod_levels(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_vox.as<uint64_t>(), built,
                       V->lod_first, V->brick_size, V->overlap, V->clamp, V->median, nullptr,
                       nullptr, d_wave.as<uint32_t>(), s, &launches);
    }
    TVK_CUDA(cudaStreamSynchronize(s));
    V->range_min = 0;
    V->range_max = 255;
    V->bmin.assign(V->total_bricks, 0.0);
    V->bmax.assign(V->total_bricks, 255.0);
    V->hist.clear();
    V->bhist.clear();
    V->hist_trimmed = 0;
    V->max_grad = 0;
    V->cell_offsets.assign(V->total_bricks, 0);
    V->cell_counts.assign(V->total_bricks, 0);
    V->cell_dims.assign(V->total_bricks, 0);
    V->total_cells = 0;
    return;
  }
  // scratch: bmin, bmax, bhist, hist, max_grad bits, per-brick largest Q
  const uint64_t gbins = uint64_t(1) << (8 * V->bytes);
  const size_t sz_bmin = V->n_bricks * 4, sz_bh = V->n_bricks * 256 * 4, sz_h = gbins * 8;
  const size_t sz_q = V->n_bricks * 8;
  const size_t total = sz_h + 8 + 8 + sz_q + 2 * sz_bmin + sz_bh + 64;
  d_scratch.ensure(total);
  uint8_t* base = d_scratch.as<uint8_t>();
  BrickScratch sc;
  sc.hist = reinterpret_cast<unsigned long long*>(base);
  sc.max_grad_bits = reinterpret_cast<unsigned long long*>(base + sz_h);
  sc.raw_minmax = nullptr;
  unsigned long long* d_qmax = reinterpret_cast<unsigned long long*>(base + sz_h + 16);
  sc.bmin = reinterpret_cast<uint32_t*>(base + sz_h + 16 + sz_q);
  sc.bmax = sc.bmin + V->n_bricks;
  sc.bhist = sc.bmax + V->n_bricks;
  TVK_CUDA(cudaMemsetAsync(base, 0, sz_h + 16 + sz_q, s));
  TVK_CUDA(cudaMemsetAsync(sc.bmin, 0xff, sz_bmin, s));
  TVK_CUDA(cudaMemsetAsync(sc.bmax, 0, sz_bmin, s));
  TVK_CUDA(cudaMemsetAsync(sc.bhist, 0, sz_bh, s));

  // pass 1: the LOD-0 bricks, their min/max and the global histogram of the
  // inner voxels -- every voxel once, so it also gives the data range
  // (Dataset::GetRange) that sets the per-brick bin shift
  BrickGrid g;
  for (int a = 0; a < 3; ++a) {
    g.dims[a] = V->dims[a];
    g.B[a] = V->brick_size[a];
    g.cnt[a] = uint32_t(l0.bricks[a]);
  }
  g.ov = V->overlap;
  g.clamp = V->clamp ? 1 : 0;
  g.total = nvox;
  launch_brick_copy(d_raw, V->bytes, g, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                    V->n_bricks, V->d_pool, sc, uint32_t(gbins), s, &launches);
  V->hist.resize(gbins);
  TVK_CUDA(cudaMemcpyAsync(V->hist.data(), sc.hist, sz_h, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaStreamSynchronize(s));
  {
    uint64_t lo = 0, hi = gbins - 1;
    while (lo < gbins && V->hist[lo] == 0) ++lo;
    while (hi > 0 && V->hist[hi] == 0) --hi;
    REQUIRE(lo < gbins, "empty volume");
    V->range_min = double(lo);
    V->range_max = double(hi);
    const uint32_t b = bits_of(hi);
    V->hist_shift = b > 8 ? b - 8 : 0;
  }
  // pass 2: per-brick 256-bin histograms and the largest squared central
  // difference per brick; the maximum |gradient| is then evaluated in the
  // reference's double arithmetic at the voxels of the largest one only
  launch_brick_sweep(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                     V->n_bricks, V->overlap, max_bz, V->hist_shift, sc.bhist, d_qmax, s,
                     &launches);
  std::vector<unsigned long long> qmax(V->n_bricks);
  TVK_CUDA(cudaMemcpyAsync(qmax.data(), d_qmax, sz_q, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaStreamSynchronize(s));
  {
    unsigned long long qm = 0;
    for (unsigned long long q : qmax) qm = std::max(qm, q);
    if (qm > 0) {  // stored as Q + 1; 0 = no inner voxel with neighbours
      std::vector<uint32_t> list;
      for (uint64_t b = 0; b < V->n_bricks; ++b)
        if (qmax[b] == qm) list.push_back(uint32_t(b));
      DevBuf d_list;
      d_list.ensure(list.size() * sizeof(uint32_t));
      TVK_CUDA(cudaMemcpyAsync(d_list.p, list.data(), list.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, s));
      launch_max_gradient_at(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                             d_list.as<uint32_t>(), uint32_t(list.size()), V->overlap, max_bz,
                             (long long)(qm - 1), sc.max_grad_bits, s, &launches);
      TVK_CUDA(cudaStreamSynchronize(s));  // d_list is released here
    }
  }
  // pass 4: the coarser LODs (ComputeHierarchy + FillOverlap) and their min/max
  DevBuf d_lmm, d_wave;
  std::vector<uint32_t> lmin, lmax;
  if (V->total_bricks > V->n_bricks) {
    d_lmm.ensure(2 * V->total_bricks * sizeof(uint32_t));
    uint64_t max_lod_bricks = 0;
    for (size_t l = 1; l < n_lods; ++l)
      max_lod_bricks = std::max<uint64_t>(max_lod_bricks, V->lod_first[l + 1] - V->lod_first[l]);
    d_wave.ensure(max_lod_bricks * sizeof(uint32_t));
    std::vector<LodInfo> built(V->lods.begin(), V->lods.begin() + n_lods);
    build_lod_levels(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_vox.as<uint64_t>(), built,
                     V->lod_first, V->brick_size, V->overlap, V->clamp, V->median,
                     d_lmm.as<uint32_t>(), d_lmm.as<uint32_t>() + V->total_bricks,
                     d_wave.as<uint32_t>(), s, &launches);
    lmin.resize(V->total_bricks);
    lmax.resize(V->total_bricks);
    TVK_CUDA(cudaMemcpyAsync(lmin.data(), d_lmm.p, V->total_bricks * 4, cudaMemcpyDeviceToHost, s));
    TVK_CUDA(cudaMemcpyAsync(lmax.data(), d_lmm.as<uint32_t>() + V->total_bricks,
                             V->total_bricks * 4, cudaMemcpyDeviceToHost, s));
  }
  // pass 5: macro-cell min/max for empty-space skipping inside the bricks of
  // every built LOD (after the coarser LODs exist)
  const uint64_t nb_all = V->total_bricks;
  V->cell_offsets.resize(nb_all);
  V->cell_counts.resize(nb_all);
  V->cell_dims.resize(nb_all);
  uint32_t max_cell_rows = 0;
  V->total_cells = 0;
  for (uint64_t k = 0; k < nb_all; ++k) {
    const uint32_t cx = cells_per_axis(V->sizes[3 * k]), cy = cells_per_axis(V->sizes[3 * k + 1]),
                   cz = cells_per_axis(V->sizes[3 * k + 2]);
    if (cx > 1023 || cy > 1023 || cz > 1023)
      fail(TVK_ERR_UNSUPPORTED, "bricks above 2046 voxels per axis (macro-cell table limit)");
    V->cell_dims[k] = cx | (cy << 10) | (cz << 20);
    V->cell_counts[k] = cx * cy * cz;
    V->cell_offsets[k] = V->total_cells;
    V->total_cells += V->cell_counts[k];
    max_cell_rows = std::max(max_cell_rows, cy);
  }
  TVK_CUDA(cudaMalloc(&V->d_cells, V->total_cells * sizeof(uint32_t)));
  TVK_CUDA(cudaMalloc(&V->d_cell_meta, nb_all * (sizeof(uint64_t) + sizeof(uint32_t))));
  uint64_t* d_cell_off = static_cast<uint64_t*>(V->d_cell_meta);
  uint32_t* d_cell_cnt = reinterpret_cast<uint32_t*>(d_cell_off + nb_all);
  TVK_CUDA(cudaMemcpyAsync(d_cell_off, V->cell_offsets.data(), nb_all * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemcpyAsync(d_cell_cnt, V->cell_counts.data(), nb_all * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, s));
  launch_cell_minmax(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                     d_cell_off, nb_all, max_cell_rows, static_cast<uint32_t*>(V->d_cells), s,
                     &launches);

  std::vector<uint32_t> bmin(V->n_bricks), bmax(V->n_bricks);
  V->bhist.resize(V->n_bricks * 256);
  unsigned long long mg = 0;
  TVK_CUDA(cudaMemcpyAsync(bmin.data(), sc.bmin, sz_bmin, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaMemcpyAsync(bmax.data(), sc.bmax, sz_bmin, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaMemcpyAsync(V->bhist.data(), sc.bhist, sz_bh, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaMemcpyAsync(&mg, sc.max_grad_bits, 8, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaStreamSynchronize(s));
  V->bmin.resize(V->total_bricks);
  V->bmax.resize(V->total_bricks);
  for (uint64_t i = 0; i < V->total_bricks; ++i) {
    V->bmin[i] = i < V->n_bricks ? bmin[i] : lmin[i];
    V->bmax[i] = i < V->n_bricks ? bmax[i] : lmax[i];
  }
  double mgd;
  std::memcpy(&mgd, &mg, 8);
  V->max_grad = mgd;
  uint64_t len = gbins;
  while (len > 0 && V->hist[len - 1] == 0) --len;
  V->hist_trimmed = len;
}

// Histogram2DDataBlock::ComputeTemplate<T> second pass (Histogram2DDataBlock.cpp:399-435)
// over the LOD-0 bricks already in the pool, with the maximum gradient of the
// first pass that build_volume ran.  `bins` rows of 256 gradient bins.
void compute_histogram2d(const tvk_volume* V, uint64_t bins, uint64_t* host_out) {
  uint32_t max_bz = 0;
  for (uint64_t b = 0; b < V->n_bricks; ++b) max_bz = std::max(max_bz, V->sizes[3 * b + 2]);
  const double nf2 = double(V->bytes == 1 ? 255 : 65535) * 2.0;
  Hist2DParams hp{};
  hp.ov = V->overlap;
  hp.value_bins = uint32_t(bins);
  hp.max_nonzero = V->range_max;
  hp.scale_values = V->range_max > double(bins - 1) ? 1u : 0u;
  hp.gmax = V->max_grad;
  // |g| = sqrt(Q) / (2 max(T)) up to double rounding, so Q is recovered exactly
  const double qr = V->max_grad * nf2;
  hp.qmax = (long long)std::llround(qr * qr);
  hp.inv_qmax = hp.qmax > 0 ? 1.0f / float(hp.qmax) : 0.0f;
  const size_t out_bytes = bins * 256 * sizeof(uint64_t);
  DevBuf d_off, d_sizes, d_hist;
  d_off.ensure(V->n_bricks * sizeof(uint64_t));
  d_sizes.ensure(V->n_bricks * 3 * sizeof(uint32_t));
  d_hist.ensure(out_bytes);
  cudaStream_t s;
  TVK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  TVK_CUDA(cudaMemcpyAsync(d_off.p, V->offsets.data(), V->n_bricks * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemcpyAsync(d_sizes.p, V->sizes.data(), V->n_bricks * 3 * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemsetAsync(d_hist.p, 0, out_bytes, s));
  uint64_t launches = 0;
  launch_histogram2d(device_bricks(V), V->bytes, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                     V->n_bricks, max_bz, hp, d_hist.as<unsigned long long>(), s, &launches);
  TVK_CUDA(cudaMemcpyAsync(host_out, d_hist.p, out_bytes, cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaStreamSynchronize(s));
}

// Paths built for scalar (one-component) volumes only.
void require_scalar(const tvk_volume* V, const char* what) {
  if (V->dtype == TVK_RGBA8)
    fail(TVK_ERR_UNSUPPORTED, std::string(what) + " take scalar volumes, not colour volumes");
}

void free_brick_textures(const tvk_volume* V) {
  for (cudaTextureObject_t t : V->tex_objs)
    if (t) cudaDestroyTextureObject(t);
  for (cudaArray_t a : V->tex_arrays)
    if (a) cudaFreeArray(a);
  V->tex_objs.clear();
  V->tex_arrays.clear();
  if (V->d_tex) cudaFree(V->d_tex);
  V->d_tex = nullptr;
}

void free_volume_device(tvk_volume* V) {
  free_brick_textures(V);
  for (void** p : {&V->d_pool, &V->d_cells, &V->d_cell_meta}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
}

// Every brick of every LOD copied into a 3D CUDA array of its own size, read
// through a texture object with linear filtering, clamp to edge and
// normalised reads (the hardware-filtered lookups of the ray march's texture
// variant).  Made once per volume, on first use; 2.6 GB more for the
// 1024^3 u16 volume.
void ensure_brick_textures(const tvk_volume* V) {
  if (V->d_tex) return;
  if (V->dtype == TVK_RGBA8 || V->rebricked)
    fail(TVK_ERR_UNSUPPORTED, "hardware filtering takes bricked scalar volumes");
  const uint8_t* pool = static_cast<const uint8_t*>(device_bricks(V));
  const cudaChannelFormatDesc cd = V->bytes == 1 ? cudaCreateChannelDesc<unsigned char>()
                                                 : cudaCreateChannelDesc<unsigned short>();
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof(td));
  for (int a = 0; a < 3; ++a) td.addressMode[a] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeNormalizedFloat;
  td.normalizedCoords = 0;
  V->tex_arrays.assign(V->total_bricks, nullptr);
  V->tex_objs.assign(V->total_bricks, 0);
  try {
    for (uint64_t k = 0; k < V->total_bricks; ++k) {
      const uint32_t* n = &V->sizes[3 * k];
      const cudaExtent ext = make_cudaExtent(n[0], n[1], n[2]);
      TVK_CUDA(cudaMalloc3DArray(&V->tex_arrays[k], &cd, ext));
      cudaMemcpy3DParms cp;
      std::memset(&cp, 0, sizeof(cp));
      cp.srcPtr = make_cudaPitchedPtr(const_cast<uint8_t*>(pool + V->offsets[k] * V->bytes),
                                      size_t(n[0]) * V->bytes, n[0], n[1]);
      cp.dstArray = V->tex_arrays[k];
      cp.extent = ext;
      cp.kind = cudaMemcpyDeviceToDevice;
      TVK_CUDA(cudaMemcpy3D(&cp));
      cudaResourceDesc rd;
      std::memset(&rd, 0, sizeof(rd));
      rd.resType = cudaResourceTypeArray;
      rd.res.array.array = V->tex_arrays[k];
      TVK_CUDA(cudaCreateTextureObject(&V->tex_objs[k], &rd, &td, nullptr));
    }
    TVK_CUDA(cudaMalloc(&V->d_tex, V->total_bricks * sizeof(cudaTextureObject_t)));
    TVK_CUDA(cudaMemcpy(V->d_tex, V->tex_objs.data(),
                        V->total_bricks * sizeof(cudaTextureObject_t), cudaMemcpyHostToDevice));
  } catch (...) {
    free_brick_textures(V);
    throw;
  }
}

tvk_volume* create_volume(const void* src, bool on_device, tvk_dtype dtype, const uint64_t dims[3],
                          const uint32_t bsz[3], uint32_t ov, int clamp, bool median = false,
                          bool build_lods = true) {
  REQUIRE(src && dims && bsz, "null argument");
  REQUIRE(dtype == TVK_U8 || dtype == TVK_U16 || dtype == TVK_RGBA8,
          "dtype must be TVK_U8, TVK_U16 or TVK_RGBA8");

  for (int a = 0; a < 3; ++a) {
    REQUIRE(dims[a] >= 1, "volume dimensions must be >= 1");
    REQUIRE(bsz[a] > 2 * ov, "brick size must exceed twice the overlap (ExtendedOctree.cpp:196)");
    REQUIRE(bsz[a] <= 4096, "brick size above 4096");
  }
  REQUIRE(dims[0] * dims[1] * dims[2] < (1ull << 40), "volume too large");
  std::unique_ptr<tvk_volume> V(new tvk_volume());
  TVK_CUDA(cudaGetDevice(&V->device));
  V->dtype = dtype;
  V->bytes = dtype == TVK_U8 ? 1 : (dtype == TVK_U16 ? 2 : 4);
  for (int a = 0; a < 3; ++a) {
    V->dims[a] = dims[a];
    V->brick_size[a] = bsz[a];
  }
  V->overlap = ov;
  V->clamp = clamp != 0;
  V->median = median;
  V->build_lods = build_lods;
  cudaStream_t s;
  TVK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  const size_t raw_bytes = size_t(dims[0] * dims[1] * dims[2]) * V->bytes;
  try {
    if (on_device) {
      build_volume(V.get(), src, s);
    } else {
      DevBuf d_raw;
      d_raw.ensure(raw_bytes);
      TVK_CUDA(cudaMemcpyAsync(d_raw.p, src, raw_bytes, cudaMemcpyHostToDevice, s));
      build_volume(V.get(), d_raw.p, s);
      TVK_CUDA(cudaStreamSynchronize(s));
    }
  } catch (...) {
    cudaStreamSynchronize(s);
    free_volume_device(V.get());
    throw;
  }
  return V.release();
}

// Global (TOC) index of a brick key (timestep, LOD, 1D index within the LOD).
uint64_t key_check(const tvk_volume* v, uint64_t ts, uint64_t lod, uint64_t idx) {
  REQUIRE(v, "null volume");
  REQUIRE(ts == 0, "only timestep 0 exists");
  REQUIRE(lod < v->lods.size(), "LOD out of range");
  if (lod + 1 >= v->lod_first.size())
    fail(TVK_ERR_UNSUPPORTED, "the volume was created with LOD 0 only");
  REQUIRE(idx < v->lod_first[lod + 1] - v->lod_first[lod], "brick index out of range");
  return v->lod_first[lod] + idx;
}

// ------------------------------------------------------------ view math

struct View {
  double mv[3][4];   // model -> eye
  double inv[3][4];  // eye -> model
  float kx, ky, inv_w2, inv_h2;
};

// Basics/Vectors.h:1250-1263 (BuildLookAt) and :1265-1276 (Perspective), in
// double, rounded to float where the kernel consumes them.
View make_view(const float eye_f[3], const float at[3], const float up[3], float fovy,
               uint32_t w, uint32_t h, const double model[3][4]) {
  const double eye[3] = {eye_f[0], eye_f[1], eye_f[2]};
  double F[3] = {double(at[0]) - eye[0], double(at[1]) - eye[1], double(at[2]) - eye[2]};
  double U[3] = {up[0], up[1], up[2]};
  auto cross = [](const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  auto norm = [](double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; ++i) v[i] /= l;
  };
  double S[3], U2[3];
  cross(F, U, S);
  cross(S, F, U2);
  norm(F);
  norm(U2);
  norm(S);
  double view[3][4];
  const double* rows[3] = {S, U2, F};
  for (int r = 0; r < 3; ++r) {
    const double sg = (r == 2) ? -1.0 : 1.0;
    double d = 0;
    for (int c = 0; c < 3; ++c) {
      view[r][c] = sg * rows[r][c];
      d += rows[r][c] * eye[c];
    }
    view[r][3] = -sg * d;
  }
  View v;
  // modelview = view o model (column-vector form); model is identity unless set
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) {
      double acc = (c == 3) ? view[r][3] : 0.0;
      for (int k = 0; k < 3; ++k) acc += view[r][k] * model[k][c];
      v.mv[r][c] = acc;
    }
  }
  for (int r = 0; r < 3; ++r) {
    double t = 0;
    for (int c = 0; c < 3; ++c) {
      v.inv[r][c] = v.mv[c][r];
      t += v.mv[c][r] * v.mv[c][3];
    }
    v.inv[r][3] = -t;
  }
  const double th = std::tan(double(fovy) * (3.14159265358979323846 / 180.0) / 2.0);
  const double aspect = double(w) / double(h);
  v.kx = float(aspect * th);
  v.ky = float(th);
  v.inv_w2 = float(2.0 / double(w));
  v.inv_h2 = float(2.0 / double(h));
  return v;
}

}  // namespace tvk

// ------------------------------------------------------------ renderer state

struct tvk_renderer {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_staged = nullptr;
  cudaEvent_t ev_ready = nullptr;  // a planned frame's uploads are queued (batch paints)
  // asynchronous image readback: the frame is copied to d_img_ro on the render
  // stream, then to the host on copy_stream while the next frame renders
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_img_ready = nullptr, ev_img_copied = nullptr;
  bool img_pending = false;
  const tvk_volume* vol = nullptr;
  // transfer function (effective RGBA as the GPU samples it)
  std::vector<float> tf;
  uint32_t tf_w = 0, tf_h = 0;
  bool tf_2d = false;
  bool tf_dirty = true;
  tvk_render_mode mode = TVK_RM_1DTRANS;
  bool lighting = false;
  tvk_light_model light_model = TVK_LIGHT_REFERENCE;
  float bp[4] = {0.2f, 0.6f, 0.2f, 32.0f};
  // AbstrRenderer.cpp:162-168 defaults
  float ambient[4] = {1, 1, 1, 0.1f}, diffuse[4] = {1, 1, 1, 1}, specular[4] = {1, 1, 1, 1};
  float light_dir[3] = {0, 0, -1};
  float srm = 1.0f;
  float isovalue = 0.5f;
  float frame_ert = 1.0f;
  // AbstrRenderer.cpp:64-69 defaults
  float eye[3] = {0, 0, 1.6f}, at[3] = {0, 0, 0}, up[3] = {0, 1, 0};
  float fovy = 50.0f, znear = 0.01f, zfar = 1000.0f;
  double model[3][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}};
  uint32_t width = 0, height = 0;
  // device buffers
  tvk::DevBuf d_img, d_spp, d_bricks, d_counters;
  tvk::DevBuf d_img_ro;  // the image being read back asynchronously
  tvk::PinnedBuf h_bricks, h_counters;
  tvk::PinnedBuf h_tf;
  // empty-cell bits for the current TF and volume
  // Device TF tables (opacity-corrected for one step scale) and the empty-cell
  // bits made from them; two slots, so frames that alternate sample rates
  // (reduced and full quality) rebuild nothing
  struct TfSlot {
    float step_scale = -1.0f;
    bool raw_alpha = false;
    bool valid = false;
    uint64_t used = 0;
    tvk::DevBuf d_tf, d_tfcol, d_tfpfx, d_empty, d_empty_meta;
    tvk::DevBuf d_dist, d_dist_tmp, d_cell_dims;  // macro-cell distances (+ scratch)
    std::vector<uint64_t> empty_word_off;
    bool empty_valid = false;
    bool empty_iso = false;
    float empty_iso_norm = 0.0f;
    float empty_trans_scale = 0.0f;
  };
  TfSlot slots[2];
  int slot = 0;
  uint64_t slot_clock = 0;
  float iso_color[3] = {0.5f, 0.5f, 0.5f};  // AbstrRenderer.cpp:86 m_vIsoColor
  bool cell_skip = true;
  bool hw_filter = false;  // texture lookups instead of the exact ones (tvk_set_hardware_filtering)
  bool depth_out = false;            // write the first-hit depth of ray-marched pixels
  bool clip_on = false;              // AbstrRenderer m_bClipPlaneOn
  float clip_plane[4] = {0, 0, 1, 0};  // m_ClipPlane, world space
  // ClearView (AbstrRenderer.cpp:130-136, 171 defaults; m_fCVIsovalue follows
  // the isovalue when a dataset is set, AbstrRenderer.cpp:261)
  tvk_scaling_method tf_scaling = TVK_SCALE_BIT_WIDTH;  // m_TFScalingMethod
  bool cv_on = false;
  float cv_iso = 0.8f;
  float cv_color[3] = {1, 0, 0};
  float cv_size = 5.5f, cv_context_scale = 1.0f, cv_border_scale = 60.0f;
  float cv_pos[4] = {0, 0, 0.5f, 1};   // m_vCVPos, model space
  tvk::DevBuf d_cvhits;                // the last ClearView frame's hit records
  double cv_last_inv[3][4] = {};       // its eye -> model transform (picking)
  bool cv_painted = false;
  tvk::DevBuf d_depth;
  tvk_stats stats{};
  uint64_t launches = 0;
  bool painted = false;
  // level of detail and reduced-quality rendering (AbstrRenderer m_iCurrentLOD,
  // decreaseScreenResNow / decreaseSamplingRateNow, SetPerfMeasures factors)
  uint32_t lod = 0;
  bool dec_screen = false, dec_sampling = false;
  float screen_dec = 2.0f, sample_dec = 2.0f;
  uint32_t render_w = 0, render_h = 0;  // size of the last ray-marched image
  tvk::DevBuf d_lowimg;
  // progressive frames (AbstrRenderer::PlanFrame, ComputeMin/MaxLODForCurrentView,
  // CompletedASubframe); names follow the reference's members
  float max_ms_per_frame = 10000.0f;    // SetPerfMeasures, 0 fps -> 10 s
  bool low_res_intermediate = false;    // m_bRenderLowResIntermediateResults
  uint32_t lod_limits[2] = {0, 0};      // m_iLODLimits
  bool capture = false;                 // m_eRendererTarget == RT_CAPTURE
  bool decrease_screen_res = false, decrease_sampling_rate = false;
  bool decrease_screen_res_now = false, decrease_sampling_rate_now = false;
  bool another_redraw_low_res = false;  // doAnotherRedrawDueToLowResOutput
  float msec_passed[2] = {-1.0f, -1.0f};
  float msec_current_frame = -1.0f;
  uint32_t lod_not_ok = 0;
  uint64_t perf_lod_skip = 0;
  uint64_t max_lod_index = 0, min_lod_view = 0, start_lod_offset = 0, current_lod_offset = 0;
  uint64_t current_lod = 0;
  bool frame_started = false;
};

// Several renderers' frames in one persistent launch (replaces the reference's
// sequential per-region / per-renderer paints, GLRenderer.cpp:622-660).
struct tvk_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_done = nullptr;
  tvk::DevBuf d_next;                        // one work counter per launch
  std::vector<tvk::BatchLaunch> launch;      // frame tables of the launches
  std::vector<int> variant;                  // kernel variant of each launch
  bool autotune = true;
  uint32_t fixed_ctas_per_sm = 0;           // 0: tuned or the occupancy maximum
  uint32_t fixed_rays_per_thread = 0;       // 0: tuned (1 or 2), else fixed
  // launch shapes -> (CTAs per SM, rays per thread)
  std::map<std::vector<uint64_t>, std::pair<uint32_t, uint32_t>> tuned;
  uint32_t rpt = 1;                         // rays per thread of the current launches
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> graph_sig;
  std::vector<cudaGraphNode_t> kernel_nodes;  // graph node of each launch
  // launches 1.. run on their own streams, forked from and joined back into
  // `stream`, so that one launch's tail overlaps the next launch's work
  std::vector<cudaStream_t> aux;
  std::vector<cudaEvent_t> fork_join;         // [0]: fork; [1 + k]: join of aux[k]
  tvk_batch_info info{};
};

// The reconstruction network: a fixed 4-level U-Net over the reduced frame.
namespace tvk {
struct UNetLayer {
  const char* name;
  int c1, c2, cout;
  float slope;  // LeakyReLU slope, < 0: none
};
// e*: encoder (two convolutions per level, 2x2 average pooling between levels),
// b: bottleneck, d*: decoder (2x nearest upsampling, then one convolution over
// the upsampled tensor concatenated with the encoder's skip tensor), head: 16
// channels = RGBA x 2x2 sub-pixels added to the bilinear upscale.
constexpr UNetLayer kUNet[] = {
    {"e0a", 16, 0, 32, 0.1f}, {"e0b", 32, 0, 32, 0.1f}, {"e1a", 32, 0, 48, 0.1f},
    {"e1b", 48, 0, 48, 0.1f}, {"e2a", 48, 0, 64, 0.1f}, {"e2b", 64, 0, 64, 0.1f},
    {"b", 64, 0, 64, 0.1f},   {"d2", 64, 64, 64, 0.1f}, {"d1", 64, 48, 48, 0.1f},
    {"d0", 48, 32, 32, 0.1f}, {"head", 32, 0, 16, -1.0f}};
constexpr int kUNetLayers = int(sizeof(kUNet) / sizeof(kUNet[0]));
inline size_t unet_param_count() {
  size_t n = 0;
  for (const UNetLayer& l : kUNet) n += size_t(9) * l.cout * (l.c1 + l.c2) + l.cout;
  return n;
}
}  // namespace tvk

struct tvk_learned {
  int device = 0;
  tvk::DevBuf d_w, d_b;                    // BF16 weights, FP32 biases (all layers)
  size_t w_off[tvk::kUNetLayers] = {}, b_off[tvk::kUNetLayers] = {};
  tvk::DevBuf d_act, d_head, d_input, d_sum;
  int hp = 0, wp = 0;
  tvk::PinnedBuf h_sum;
  cudaEvent_t ev[5] = {};
  uint32_t frame = 0;
  // the probe rays run on their own stream with their own brick list
  cudaStream_t probe_stream = nullptr;
  tvk::DevBuf p_bricks, p_counters;
  tvk::PinnedBuf p_hbricks;
  cudaEvent_t ev_pstaged = nullptr, ev_planned = nullptr, ev_pstart = nullptr,
              ev_pdone = nullptr;
};

// LOD-octree brick cache for the GridLeaper (GLVolumePool + GLHashTable).
struct tvk_pool {
  const tvk_volume* vol = nullptr;
  int device = 0;
  uint32_t n_slots = 0;
  uint64_t slot_voxels = 0;
  tvk::DevBuf d_slots;
  bool host_source = false;          // bricks paged from pinned host memory
  tvk::PinnedBuf h_bricks;           // host brick store (the volume's pool layout)
  std::vector<uint32_t> page;        // page table per brick (all LODs)
  tvk::PinnedBuf h_page;
  tvk::DevBuf d_page, d_dims;
  struct Slot {                      // PoolSlotData (GLVolumePool.h:24-60)
    int64_t brick = -1;
    uint64_t time = 0;                 // 0 never used, 1 flagged empty, else creation time
    uint64_t orig_time = 0;
  };
  std::vector<Slot> slots;           // the coarsest brick starts in the last slot
  uint64_t clock = 2;
  uint32_t coarsest = 0;
  tvk::DevBuf d_hash;
  tvk::PinnedBuf h_hash;
  uint32_t hash_size = 0, rehash = 10;
  tvk::DevBuf d_resume_pos, d_resume_col;
  cudaStream_t page_stream = nullptr;
  cudaEvent_t ev_paged = nullptr;
  cudaEvent_t ev_pass[2] = {nullptr, nullptr};  // brackets each traversal launch
  // visibility flags were computed for this state
  bool vis_valid = false;
  int vis_mode = -1;
  double vis_lo = 0, vis_hi = 0;
  float vis_iso = 0;
  uint64_t paged_total = 0;
  std::vector<uint64_t> requests;    // bricks the last pass reported missing
};

namespace tvk {
namespace {

// raw_alpha: the entries keep their alpha (colour volumes correct the opacity
// of each sample's product with the voxel alpha instead).
void upload_tf(tvk_renderer* R, float step_scale, bool raw_alpha = false) {
  if (R->tf_dirty) {
    for (auto& sl : R->slots) sl.valid = false;
    R->tf_dirty = false;
  }
  for (int i = 0; i < 2; ++i)
    if (R->slots[i].valid && R->slots[i].step_scale == step_scale &&
        R->slots[i].raw_alpha == raw_alpha) {
      R->slot = i;
      R->slots[i].used = ++R->slot_clock;
      return;
    }
  // rebuild the least recently used slot
  const int si = (!R->slots[0].valid || (R->slots[1].valid && R->slots[0].used <= R->slots[1].used))
                     ? 0 : 1;
  R->slot = si;
  tvk_renderer::TfSlot& S = R->slots[si];
  const size_t n = size_t(R->tf_w) * R->tf_h;
  // the previous upload may still be reading the staging buffer
  TVK_CUDA(cudaStreamSynchronize(R->stream));
  R->h_tf.ensure(n * sizeof(float4) + R->tf_w);
  float* t = R->h_tf.as<float>();
  uint8_t* col = reinterpret_cast<uint8_t*>(t + 4 * n);
  std::fill(col, col + R->tf_w, uint8_t(0));
  for (size_t i = 0; i < n; ++i) {
    t[4 * i + 0] = R->tf[4 * i + 0];
    t[4 * i + 1] = R->tf[4 * i + 1];
    t[4 * i + 2] = R->tf[4 * i + 2];
    // VRender1D.glsl:53 opacity correction, evaluated per table entry
    const float a = R->tf[4 * i + 3];
    t[4 * i + 3] = raw_alpha ? a : 1.0f - std::pow(1.0f - a, step_scale);
    // a sample whose corrected alpha is exactly 0 adds exactly nothing
    if (t[4 * i + 3] != 0.0f) col[i % R->tf_w] = 1;
  }
  S.d_tf.ensure(n * sizeof(float4));
  S.d_tfcol.ensure(R->tf_w);
  TVK_CUDA(cudaMemcpyAsync(S.d_tf.p, t, n * sizeof(float4), cudaMemcpyHostToDevice, R->stream));
  TVK_CUDA(cudaMemcpyAsync(S.d_tfcol.p, col, R->tf_w, cudaMemcpyHostToDevice, R->stream));
  // prefix counts of value columns with any non-zero corrected alpha
  std::vector<uint32_t> pfx(R->tf_w + 1, 0);
  for (uint32_t x = 0; x < R->tf_w; ++x) pfx[x + 1] = pfx[x] + (col[x] ? 1u : 0u);
  S.d_tfpfx.ensure(pfx.size() * sizeof(uint32_t));
  TVK_CUDA(cudaMemcpy(S.d_tfpfx.p, pfx.data(), pfx.size() * sizeof(uint32_t),
                      cudaMemcpyHostToDevice));
  S.valid = true;
  S.step_scale = step_scale;
  S.raw_alpha = raw_alpha;
  S.used = ++R->slot_clock;
  S.empty_valid = false;
}

// Empty-cell bits of every brick of every built LOD for the current TF (re-run
// when the TF, the opacity correction or the volume changes).
void update_empty_cells(tvk_renderer* R, const tvk_volume* V, float trans_scale, bool iso_mode,
                        float iso_norm) {
  tvk_renderer::TfSlot& S = R->slots[R->slot];
  if (S.empty_valid && S.empty_iso == iso_mode &&
      (iso_mode ? S.empty_iso_norm == iso_norm : S.empty_trans_scale == trans_scale))
    return;
  // every built LOD's bricks, indexed by TOC position
  const uint64_t nb = V->total_bricks;
  S.empty_word_off.resize(nb);
  uint64_t words = 0;
  uint32_t max_words = 0;
  for (uint64_t k = 0; k < nb; ++k) {
    S.empty_word_off[k] = words;
    const uint32_t w = (V->cell_counts[k] + 31) / 32;
    words += w;
    max_words = std::max(max_words, w);
  }
  S.d_empty.ensure(std::max<uint64_t>(1, words) * sizeof(uint32_t));
  S.d_empty_meta.ensure(nb * sizeof(uint64_t));
  TVK_CUDA(cudaMemcpyAsync(S.d_empty_meta.p, S.empty_word_off.data(), nb * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, R->stream));
  EmptyCellParams p;
  p.cell_minmax = static_cast<const uint32_t*>(V->d_cells);
  p.cell_offsets = static_cast<const uint64_t*>(V->d_cell_meta);
  p.cell_counts = reinterpret_cast<const uint32_t*>(p.cell_offsets + nb);
  p.word_offsets = S.d_empty_meta.as<uint64_t>();
  p.n_bricks = nb;
  p.nz_prefix = S.d_tfpfx.as<uint32_t>();
  p.tf_w = R->tf_w;
  p.inv_max_raw = V->bytes == 1 ? 1.0f / 255.0f : 1.0f / 65535.0f;
  p.trans_scale = trans_scale;
  p.iso_mode = iso_mode ? 1 : 0;
  p.iso_norm = iso_norm;
  p.bits = S.d_empty.as<uint32_t>();
  launch_empty_cells(p, max_words, R->stream, &R->launches);
  // Chebyshev distances of the cells to the nearest non-empty cell
  const uint64_t ncells = std::max<uint64_t>(1, V->total_cells);
  S.d_dist.ensure(ncells);
  S.d_dist_tmp.ensure(2 * ncells);
  S.d_cell_dims.ensure(nb * sizeof(uint32_t));
  TVK_CUDA(cudaMemcpyAsync(S.d_cell_dims.p, V->cell_dims.data(), nb * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, R->stream));
  uint32_t max_lines[3] = {0, 0, 0};
  for (uint64_t k = 0; k < nb; ++k) {
    const uint32_t d = V->cell_dims[k];
    const uint32_t cx = d & 1023u, cy = (d >> 10) & 1023u, cz = d >> 20;
    max_lines[0] = std::max(max_lines[0], cy * cz);
    max_lines[1] = std::max(max_lines[1], cx * cz);
    max_lines[2] = std::max(max_lines[2], cx * cy);
  }
  CellDistParams cd;
  cd.bits = S.d_empty.as<uint32_t>();
  cd.word_offsets = S.d_empty_meta.as<uint64_t>();
  cd.cell_offsets = static_cast<const uint64_t*>(V->d_cell_meta);
  cd.cell_dims = S.d_cell_dims.as<uint32_t>();
  cd.in = nullptr;
  cd.out = nullptr;
  cd.n_bricks = nb;
  uint8_t* tmp = S.d_dist_tmp.as<uint8_t>();
  launch_cell_dist(cd, max_lines, tmp, tmp + ncells, S.d_dist.as<uint8_t>(), R->stream,
                   &R->launches);
  // the word offsets above were copied from pageable memory; keep them alive
  TVK_CUDA(cudaStreamSynchronize(R->stream));
  S.empty_valid = true;
  S.empty_iso = iso_mode;
  S.empty_iso_norm = iso_norm;
  S.empty_trans_scale = trans_scale;
}

void set_tf(tvk_renderer* R, const float* rgba, uint32_t w, uint32_t h, bool rgba8) {
  R->tf.assign(rgba, rgba + size_t(4) * w * h);
  if (rgba8) {
    // TransferFunction1D.cpp:311-330 GetByteArray, sampled back as UNORM8
    for (float& x : R->tf) {
      const unsigned char b = (unsigned char)(std::max(0.0f, std::min(x, 1.0f)) * 255);
      x = float(b) / 255.0f;
    }
  }
  R->tf_w = w;
  R->tf_h = h;
  R->tf_2d = h > 1;
  R->tf_dirty = true;
}

// What one (sub)frame renders: the LOD and the two reduced-quality switches.
struct Subframe {
  uint32_t lod;
  bool dec_screen, dec_sampling;
};

// A frame planned on the host and ready to launch.
struct PlannedFrame {
  RenderParams P;
  uint32_t rw, rh;   // ray-marched size (smaller than the viewport when reduced)
  bool upscale;
  uint64_t launches0;
  CvComposeParams cv;  // ClearView frames (P.cv_on): the compose pass
};

// Where a planned frame's brick list and counters go: the renderer's own
// buffers and stream, or a second set so that two frames of one renderer can
// be in flight on two streams (the learned frame's probe rays).
struct Stage {
  DevBuf* d_bricks;
  PinnedBuf* h_bricks;
  cudaEvent_t ev_staged;   // the last brick-list upload from h_bricks
  DevBuf* d_counters;
  cudaStream_t stream;     // brick-list upload and counter clear
};

Stage renderer_stage(tvk_renderer* R) {
  return Stage{&R->d_bricks, &R->h_bricks, R->ev_staged, &R->d_counters, R->stream};
}

// Everything of a paint up to the kernel launch: TF table and empty-cell bits
// (on the renderer's stream), the brick list of the LOD (uploaded on the
// stage's stream), the counters cleared, and the frame's parameters.
PlannedFrame plan_frame(tvk_renderer* R, const Subframe& sf, const Stage* stage = nullptr) {
  const Stage st = stage ? *stage : renderer_stage(R);
  const tvk_volume* V = R->vol;
  if (!V) fail(TVK_ERR_STATE, "no volume attached (tvk_renderer_set_volume)");
  const bool iso_mode = R->mode == TVK_RM_ISOSURFACE;
  if (!iso_mode && R->tf.empty()) fail(TVK_ERR_STATE, "no transfer function set");
  if (R->width == 0 || R->height == 0) fail(TVK_ERR_STATE, "no viewport (tvk_resize)");
  if (R->mode == TVK_RM_2DTRANS && !R->tf_2d) fail(TVK_ERR_STATE, "2D mode needs a 2D TF");
  if (R->mode == TVK_RM_1DTRANS && R->tf_2d) fail(TVK_ERR_STATE, "1D mode needs a 1D TF");
  if (V->dtype == TVK_RGBA8 && R->mode == TVK_RM_2DTRANS)
    fail(TVK_ERR_UNSUPPORTED, "colour volumes render in 1D or iso mode only");
  const uint32_t L = sf.lod;
  if (L >= V->lods.size()) fail(TVK_ERR_INVALID_ARG, "LOD out of range");
  if (L + 1 >= V->lod_first.size())
    fail(TVK_ERR_UNSUPPORTED, "the volume was created with LOD 0 only");
  TVK_CUDA(cudaSetDevice(R->device));
  const uint64_t launches0 = R->launches;

  // GLRaycaster.cpp:253-257: the sample rate divided by m_fSampleDecFactor while
  // decreasing the sampling rate; fStepScale grows with the LOD's voxel size
  const float srm = R->srm / (sf.dec_sampling ? R->sample_dec : 1.0f);
  float dom = 0.0f;
  for (int a = 0; a < 3; ++a)
    dom = std::max(dom, float(V->lods[0].size[a]) / float(V->lods[L].size[a]));
  const float step_scale = 1.0f / srm * dom;
  // GLRenderer.cpp:864-889 SetViewPort: 1/m_fScreenResDecFactor of the viewport,
  // rounded to the nearest pixel
  uint32_t rw = R->width, rh = R->height;
  if (sf.dec_screen) {
    const float rescale = 1.0f / R->screen_dec;
    rw = std::max(1u, uint32_t(float(R->width) * rescale + 0.5f));
    rh = std::max(1u, uint32_t(float(R->height) * rescale + 0.5f));
  }
  if (!R->tf.empty()) upload_tf(R, step_scale, V->dtype == TVK_RGBA8);
  // GLRenderer.cpp:1813-1819 CalculateScaling, or in 1D mode with bias and
  // scale the fTransScale of GLRaycaster.cpp:577-584 (|min| + |max|)
  const bool color = V->dtype == TVK_RGBA8;
  const uint32_t cbits = color ? 8 : 8 * V->bytes;  // Dataset::GetBitWidth
  const uint32_t imax = (1u << cbits) - 1;
  const float trans_scale =
      (R->mode == TVK_RM_1DTRANS && R->tf_scaling == TVK_SCALE_BIAS_AND_SCALE)
          ? std::fabs(float(V->range_min)) + std::fabs(float(V->range_max))
          : float(double(imax) / V->range_max);
  // AbstrRenderer.cpp:412-424 GetNormalizedIsovalue: isovalue / 2^bits
  const float iso_norm = float(double(R->isovalue) / double(1u << cbits));
  if (R->cell_skip && !color) update_empty_cells(R, V, trans_scale, iso_mode, iso_norm);

  const View view = make_view(R->eye, R->at, R->up, R->fovy, rw, rh, R->model);

  // AbstrRenderer.cpp:1003-1012: scale of the brick boxes
  const double user_scale[3] = {1, 1, 1};
  const float us[3] = {float(user_scale[0]), float(user_scale[1]), float(user_scale[2])};
  const float dmax = float(std::max(V->dims[0], std::max(V->dims[1], V->dims[2])));
  float dcs[3];
  for (int a = 0; a < 3; ++a) dcs[a] = us[a] * float(V->dims[a]) / dmax;
  const float dcmax = std::max(dcs[0], std::max(dcs[1], dcs[2]));
  float vs[3];
  for (int a = 0; a < 3; ++a) vs[a] = us[a] / dcmax;

  // AbstrRenderer.cpp:953-997 ContainsData with TF non-zero limits
  // (TransferFunction1D.cpp:362-371; TF2D's value axis for 2D)
  uint64_t nz_lo = R->tf_w, nz_hi = 0;
  for (uint32_t y = 0; y < R->tf_h; ++y)
    for (uint32_t x = 0; x < R->tf_w; ++x)
      if (R->tf[4 * (size_t(y) * R->tf_w + x) + 3] != 0) {
        nz_lo = std::min<uint64_t>(nz_lo, x);
        nz_hi = std::max<uint64_t>(nz_hi, x);
      }
  const double rmax = V->range_max;
  const double rescale = rmax / double(R->tf_w - 1);
  const double lo = double(nz_lo) * rescale, hi = double(nz_hi) * rescale;

  // per-brick records of the visible bricks of LOD L (BuildSubFrameBrickList)
  const uint64_t first = V->lod_first[L], nbl = V->lod_first[L + 1] - first;
  TVK_CUDA(cudaEventSynchronize(st.ev_staged));
  st.h_bricks->ensure(nbl * sizeof(DevBrick));
  DevBrick* hb = st.h_bricks->as<DevBrick>();
  uint32_t nvis = 0;
  // Front-to-back order valid for every ray: bricks sorted by L1 distance of
  // their grid coordinates from the eye's brick cell.  Along a ray that
  // distance grows at every crossing into the next brick, so this order
  // restates the per-ray entry-distance order of the brick loop
  // (AbstrRenderer.cpp:1097 sorts by corner distance instead).
  const LodInfo& ll = V->lods[L];
  int64_t eye_cell[3];
  for (int a = 0; a < 3; ++a) {
    const double o = view.inv[a][3];
    const uint64_t stride = a == 0 ? 1 : (a == 1 ? ll.bricks[0] : ll.bricks[0] * ll.bricks[1]);
    int64_t e = int64_t(ll.bricks[a]);
    for (uint64_t i = 0; i < ll.bricks[a]; ++i) {
      const tvk_brick_md& m = V->md[first + i * stride];
      const double lo_b = double(m.center[a] * vs[a] - m.extents[a] * vs[a] / 2.0f);
      const double hi_b = double(m.center[a] * vs[a] + m.extents[a] * vs[a] / 2.0f);
      if (i == 0 && o < lo_b) { e = -1; break; }
      if (o < hi_b) { e = int64_t(i); break; }
    }
    eye_cell[a] = e;
  }
  // The clip plane in model space (GLRaycaster.cpp:328-337: the world plane
  // through the inverse model transform, the normal normalised, d kept) and
  // in eye space for the rays
  float clip_m[4] = {0, 0, 0, 0}, clip_e[4] = {0, 0, 0, 0};
  if (R->clip_on) {
    double nm[3], dm = double(R->clip_plane[3]);
    for (int j = 0; j < 3; ++j) {
      nm[j] = 0;
      for (int i = 0; i < 3; ++i) nm[j] += double(R->clip_plane[i]) * R->model[i][j];
    }
    for (int i = 0; i < 3; ++i) dm += double(R->clip_plane[i]) * R->model[i][3];
    const float n0 = float(nm[0]), n1 = float(nm[1]), n2 = float(nm[2]);
    const float len = std::sqrt((n0 * n0 + n1 * n1) + n2 * n2);
    clip_m[0] = n0 / len;
    clip_m[1] = n1 / len;
    clip_m[2] = n2 / len;
    clip_m[3] = float(dm);
    double de = double(clip_m[3]);
    for (int j = 0; j < 3; ++j) {
      double ne = 0;
      for (int i = 0; i < 3; ++i) ne += double(clip_m[i]) * view.inv[i][j];
      clip_e[j] = float(ne);
    }
    for (int i = 0; i < 3; ++i) de += double(clip_m[i]) * view.inv[i][3];
    clip_e[3] = float(de);
  }
  // AbstrRenderer::Clipped (AbstrRenderer.cpp:923-948): every corner cut away
  auto clipped = [&](const float pmin[3], const float pmax[3]) {
    for (int c = 0; c < 8; ++c) {
      const float x = (c & 4) ? pmax[0] : pmin[0];
      const float y = (c & 2) ? pmax[1] : pmin[1];
      const float z = (c & 1) ? pmax[2] : pmin[2];
      if (!(((clip_m[0] * x + clip_m[1] * y) + clip_m[2] * z) + clip_m[3] >= 0.0f)) return false;
    }
    return true;
  };
  std::vector<std::pair<uint64_t, uint64_t>> order;  // (L1 distance, brick)
  order.reserve(nbl);
  for (uint64_t j = 0; j < nbl; ++j) {
    const uint64_t k = first + j;
    // ContainsData (uvfDataset.cpp:1201-1215): TF value limits, or the
    // isovalue; colour bricks always (AbstrRenderer.cpp:955-959)
    if (!color &&
        (iso_mode ? !(double(R->isovalue) <= V->bmax[k]) : !(hi >= V->bmin[k] && lo <= V->bmax[k])))
      continue;
    const int64_t c[3] = {int64_t(j % ll.bricks[0]), int64_t((j / ll.bricks[0]) % ll.bricks[1]),
                          int64_t(j / (ll.bricks[0] * ll.bricks[1]))};
    uint64_t d = 0;
    for (int a = 0; a < 3; ++a) d += uint64_t(std::llabs(c[a] - eye_cell[a]));
    order.emplace_back(d, k);
  }
  std::sort(order.begin(), order.end());
  for (const auto& ok : order) {
    const uint64_t k = ok.second;
    const tvk_brick_md& m = V->md[k];
    DevBrick& b = hb[nvis];
    std::memset(&b, 0, sizeof(b));
    float e[3], c[3], tmin[3], tmax[3];
    for (int a = 0; a < 3; ++a) {
      b.n[a] = m.n_voxels[a];
      e[a] = m.extents[a] * vs[a];
      c[a] = m.center[a] * vs[a];
      b.pmin[a] = c[a] - e[a] / 2.0f;
      b.pmax[a] = c[a] + e[a] / 2.0f;
      // UVFDataset::GetTextCoords (uvfDataset.cpp:1747-1774): the upper corner
      // is scaled by the LOD's brick aspect (ExtendedOctree::GetBrickAspect)
      tmin[a] = float(V->overlap) / float(b.n[a]);
      tmax[a] = (1.0f - tmin[a]) * float(ll.aspect[a]);
    }
    // GLRaycaster.cpp:589-612 ComputeEyeToTextureMatrix
    for (int a = 0; a < 3; ++a) {
      const double sc = double((tmin[a] - tmax[a]) / (b.pmin[a] - b.pmax[a]));
      for (int j = 0; j < 3; ++j) b.tex[a][j] = float(sc * view.inv[a][j]);
      b.tex[a][3] = float(sc * (view.inv[a][3] - double(b.pmax[a])) + double(tmax[a]));
    }
    // GLRaycaster.cpp:255 fRayStepsize
    float stp = std::numeric_limits<float>::infinity();
    for (int a = 0; a < 3; ++a) {
      const float vsz = 1.0f / float(b.n[a]);
      stp = std::min(stp, e[a] * vsz * 0.5f * 1.0f / srm);
    }
    b.step = stp;
    b.off = V->offsets[k];
    b.id = uint32_t(k);
    b.cells = V->cell_dims[k];
    b.cell_off = V->cell_offsets[k];
    if (R->clip_on && clipped(b.pmin, b.pmax)) continue;  // the slot is reused
    ++nvis;
  }
  st.d_bricks->ensure(std::max<size_t>(1, nbl) * sizeof(DevBrick));
  if (nvis)
    TVK_CUDA(cudaMemcpyAsync(st.d_bricks->p, hb, nvis * sizeof(DevBrick), cudaMemcpyHostToDevice,
                             st.stream));
  TVK_CUDA(cudaEventRecord(st.ev_staged, st.stream));

  RenderParams P;
  std::memset(&P, 0, sizeof(P));
  P.pool = device_bricks(V);
  P.bytes = V->bytes;
  P.bricks = st.d_bricks->as<DevBrick>();
  P.n_bricks = nvis;
  P.tf = R->slots[R->slot].d_tf.as<float4>();
  P.tf_col_nonzero = R->slots[R->slot].d_tfcol.as<uint8_t>();
  P.tf_w = R->tf_w;
  P.tf_h = R->tf_h;
  P.mode = R->mode;
  P.lighting = R->lighting ? 1 : 0;
  P.light_model = R->light_model;
  P.cell_dist = (R->cell_skip && !color) ? R->slots[R->slot].d_dist.as<uint8_t>() : nullptr;
  if (R->hw_filter) {
    if (color) fail(TVK_ERR_UNSUPPORTED, "hardware filtering takes scalar volumes");
    if (iso_mode && R->cv_on)
      fail(TVK_ERR_UNSUPPORTED, "hardware filtering does not run ClearView frames");
    ensure_brick_textures(V);
    P.tex = static_cast<const cudaTextureObject_t*>(V->d_tex);
  }
  P.trans_scale = trans_scale;
  P.step_scale = step_scale;
  const float mg = float(V->max_grad);
  P.grad_scale = (mg == 0) ? 1.0f : 1.0f / mg;  // GLRenderer.cpp:1840-1841
  P.inv_max_raw = V->bytes == 2 ? 1.0f / 65535.0f : 1.0f / 255.0f;
  for (int a = 0; a < 3; ++a) {
    // GLRenderer.cpp:2890-2893: colour.xyz * colour.w
    P.light_a[a] = R->ambient[a] * R->ambient[3];
    P.light_d[a] = R->diffuse[a] * R->diffuse[3];
    P.light_s[a] = R->specular[a] * R->specular[3];
    P.light_dir[a] = R->light_dir[a];
    P.domain_scale[a] = 1.0f / float(user_scale[a]);
    for (int j = 0; j < 3; ++j) P.norm_mat[a][j] = float(view.mv[a][j]);
    for (int j = 0; j < 4; ++j) P.inv[a][j] = float(view.inv[a][j]);
    for (int j = 0; j < 4; ++j) P.mv[a][j] = float(view.mv[a][j]);
  }
  P.clip_on = R->clip_on ? 1 : 0;
  for (int a = 0; a < 4; ++a) P.clip_eye[a] = clip_e[a];
  P.bp_ka = R->bp[0];
  P.bp_kd = R->bp[1];
  P.bp_ks = R->bp[2];
  P.bp_shininess = R->bp[3];
  P.kx = view.kx;
  P.ky = view.ky;
  P.inv_w2 = view.inv_w2;
  P.inv_h2 = view.inv_h2;
  P.znear = R->znear;
  P.zfar = R->zfar;
  P.frame_ert = R->frame_ert;
  P.iso_norm = iso_norm;
  // CullingLOD.cpp:69-72 GetDepthScaleParams
  P.proj_x = R->zfar / (R->zfar - R->znear);
  P.proj_y = (R->zfar * R->znear / (R->znear - R->zfar));
  for (int a = 0; a < 3; ++a)  // GLRenderer.cpp:2807-2808
    P.iso_diffuse[a] = (R->diffuse[a] * R->diffuse[3]) * R->iso_color[a];
  P.max_q = 1.0e6f;
  P.width = rw;
  P.height = rh;
  P.out_w = rw;
  P.out_h = rh;
  P.stride = 1;
  P.off_x = P.off_y = 0;
  const size_t npix = size_t(R->width) * R->height;
  R->d_img.ensure(npix * sizeof(float4));
  R->d_spp.ensure(size_t(rw) * rh * sizeof(uint32_t));
  st.d_counters->ensure(8 * sizeof(unsigned long long));
  const bool upscale = rw != R->width || rh != R->height;
  if (upscale) R->d_lowimg.ensure(size_t(rw) * rh * sizeof(float4));
  P.out = upscale ? R->d_lowimg.as<float4>() : R->d_img.as<float4>();
  P.spp = R->d_spp.as<uint32_t>();
  if (R->depth_out) {
    R->d_depth.ensure(size_t(rw) * rh * sizeof(float));
    P.depth = R->d_depth.as<float>();
  }
  P.counters = st.d_counters->as<unsigned long long>();
  TVK_CUDA(cudaMemsetAsync(st.d_counters->p, 0, 8 * sizeof(unsigned long long), st.stream));
  R->stats.bricks_visible = nvis;
  R->stats.bricks_total = nbl;
  CvComposeParams cv;
  std::memset(&cv, 0, sizeof(cv));
  if (iso_mode && R->cv_on && !color) {  // GLRaycaster::SupportsClearView: scalar data
    // GLRaycaster.cpp:571-575 (GetNormalizedCVIsovalue: isovalue / 2^bits)
    P.cv_on = 1;
    P.cv_iso = float(double(R->cv_iso) / double(1u << cbits));
    P.cv_cell_skip = P.cv_iso >= iso_norm ? 1 : 0;
    R->d_cvhits.ensure(size_t(rw) * rh * 4 * sizeof(float4));
    P.cv_hits = R->d_cvhits.as<float4>();
    // GLRenderer.cpp:2777-2794 ComposeSurfaceImage uniforms
    cv.hits = P.cv_hits;
    cv.out = P.out;
    cv.w = rw;
    cv.h = rh;
    cv.fbo_w = R->width;
    cv.fbo_h = R->height;
    for (int a = 0; a < 3; ++a) {
      cv.light_a[a] = P.light_a[a];
      cv.diffuse_context[a] = P.iso_diffuse[a];
      cv.diffuse_focus[a] = (R->diffuse[a] * R->diffuse[3]) * R->cv_color[a];
      cv.light_s[a] = P.light_s[a];
      cv.light_dir[a] = P.light_dir[a];
      // vCVPickPos = m_vCVPos * modelView
      double e = 0;
      for (int j = 0; j < 4; ++j) e += view.mv[a][j] * double(R->cv_pos[j]);
      cv.pick[a] = float(e);
    }
    cv.size = R->cv_size;
    cv.context_scale = R->cv_context_scale;
    cv.border_scale = R->cv_border_scale;
    std::memcpy(R->cv_last_inv, view.inv, sizeof(R->cv_last_inv));
  }
  return PlannedFrame{P, rw, rh, upscale, launches0, cv};
}

// GLRenderer.cpp:717-747 CopyOverCompletedRegion: the reduced image is
// stretched over the viewport with GL_LINEAR
void launch_upscale_of(tvk_renderer* R, const PlannedFrame& F, cudaStream_t s,
                       uint64_t* launches) {
  if (F.upscale)
    launch_upscale(R->d_lowimg.as<float4>(), F.rw, F.rh, R->d_img.as<float4>(), R->width,
                   R->height, 1.0f / R->screen_dec, s, launches);
}

// After the frame's kernels are ordered on the renderer's stream: the counters'
// read-back and the bookkeeping of a finished paint.
void finish_frame(tvk_renderer* R, const PlannedFrame& F) {
  R->render_w = F.rw;
  R->render_h = F.rh;
  R->h_counters.ensure(8 * sizeof(unsigned long long));
  TVK_CUDA(cudaMemcpyAsync(R->h_counters.p, R->d_counters.p, 8 * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, R->stream));
  R->stats.kernel_launches = R->launches - F.launches0;
  R->painted = true;
}

void paint(tvk_renderer* R, const Subframe& sf) {
  const PlannedFrame F = plan_frame(R, sf);
  TVK_CUDA(cudaEventRecord(R->ev_start, R->stream));
  launch_raycast(F.P, R->stream, &R->launches);
  if (F.P.cv_on) launch_cv_compose(F.cv, R->stream, &R->launches);
  R->cv_painted = F.P.cv_on != 0;
  launch_upscale_of(R, F, R->stream, &R->launches);
  TVK_CUDA(cudaEventRecord(R->ev_stop, R->stream));
  finish_frame(R, F);
}

// CullingLOD::GetLODLevel (CullingLOD.cpp:126-138) with the screen parameters of
// SetScreenParams (:57-67, screen-space error 1) as ComputeMinLODForCurrentView
// (AbstrRenderer.cpp:789-803) calls it: the volume centre at the origin, the
// normalised domain extent and the LOD-0 voxel count, clamped to the LOD limits.
uint64_t min_lod_for_view(const tvk_renderer* R, const tvk_volume* V) {
  const View view = make_view(R->eye, R->at, R->up, R->fovy, R->width, R->height, R->model);
  float ext[3];
  for (int a = 0; a < 3; ++a) ext[a] = float(V->dims[a]);  // times GetScale() = 1
  const float emax = std::max(ext[0], std::max(ext[1], ext[2]));
  float err = 0.0f;
  for (int a = 0; a < 3; ++a) err = std::max(err, (ext[a] / emax) / float(V->dims[a]));
  const float lod_factor = 2.0f * std::tan(R->fovy * ((3.1416f / 180.0f) / 2.0f)) * 1.0f /
                           float(R->height);
  const float z_center = float(view.mv[2][3]);
  const float fz = std::max(R->znear, -z_center);
  const int level = int(std::floor(std::log(lod_factor * fz / err) / std::log(2.0f)));
  const int hi = int(V->lods.size()) - 1;
  return uint64_t(std::min(std::max(level, int(R->lod_limits[1])), hi));
}

// AbstrRenderer::ComputeMaxLODForCurrentView (AbstrRenderer.cpp:681-787).
void compute_start_lod(tvk_renderer* R) {
  if (!R->capture && R->msec_passed[0] >= 0.0f) {
    if (R->msec_passed[0] > R->max_ms_per_frame) {
      if (R->lod_not_ok < 3) {
        R->lod_not_ok++;
      } else {
        R->lod_not_ok = 0;
        const uint64_t skip = std::max<uint64_t>(1, R->perf_lod_skip) - 1;
        if (R->perf_lod_skip != skip) {
          R->msec_passed[0] = R->msec_passed[1];
          R->perf_lod_skip = skip;
        } else if (R->low_res_intermediate) {
          if (!(R->decrease_sampling_rate && R->decrease_screen_res)) {
            if (!R->decrease_screen_res)
              R->decrease_screen_res = true;
            else
              R->decrease_sampling_rate = true;
          }
        }
      }
    } else if (R->msec_passed[1] >= 0.0f && R->msec_passed[1] <= R->max_ms_per_frame) {
      // the last frame finished (our subframes always render every brick)
      R->lod_not_ok = 0;
      if (R->decrease_sampling_rate || R->decrease_screen_res) {
        if (R->decrease_sampling_rate)
          R->decrease_sampling_rate = false;
        else
          R->decrease_screen_res = false;
      } else {
        R->perf_lod_skip =
            std::min<uint64_t>(R->max_lod_index - R->min_lod_view, R->perf_lod_skip + 1);
      }
    }
    // unsigned arithmetic as in the reference (wraps where it does)
    R->start_lod_offset = std::max<uint64_t>(R->min_lod_view, R->max_lod_index - R->perf_lod_skip);
  } else if (R->capture) {
    R->start_lod_offset = R->min_lod_view;
  } else {
    R->start_lod_offset = R->max_lod_index;  // the very first frame
  }
  R->start_lod_offset =
      std::min<uint64_t>(R->start_lod_offset, R->max_lod_index - uint64_t(R->lod_limits[0]));
  R->current_lod_offset = R->start_lod_offset;
  R->msec_passed[0] = R->msec_passed[1] = -1.0f;  // RestartTimers
}

// One subframe of a progressive frame: AbstrRenderer::PlanFrame
// (AbstrRenderer.cpp:1125-1212), the paint, and CompletedASubframe (:651-670).
void paint_progressive(tvk_renderer* R, bool new_frame, tvk_subframe_info* info) {
  const tvk_volume* V = R->vol;
  if (!V) fail(TVK_ERR_STATE, "no volume attached (tvk_renderer_set_volume)");
  if (!new_frame && !R->frame_started) new_frame = true;
  bool build = false;
  if (new_frame) {
    R->min_lod_view = min_lod_for_view(R, V);
    compute_start_lod(R);
    R->decrease_sampling_rate_now = R->decrease_sampling_rate;
    R->decrease_screen_res_now = R->decrease_screen_res;
    build = true;
    if (R->decrease_sampling_rate_now || R->decrease_screen_res_now)
      R->another_redraw_low_res = true;
  } else if (R->decrease_sampling_rate_now || R->decrease_screen_res_now) {
    R->decrease_screen_res_now = false;
    R->decrease_sampling_rate_now = false;
    R->another_redraw_low_res = false;
  } else if (R->current_lod_offset > R->min_lod_view) {
    build = true;
    R->current_lod_offset--;
  } else {
    // the frame is complete: the reference's CheckForRedraw asks for nothing more
    std::memset(info, 0, sizeof(*info));
    info->lod = uint32_t(R->current_lod);
    info->frame_complete = 1;
    return;
  }
  if (build)
    R->current_lod = R->capture ? 0
                                : std::min<uint64_t>(R->current_lod_offset, V->lods.size() - 1);
  // LODs the volume does not hold fall back to the coarsest built one
  const uint64_t built = V->lod_first.size() - 2;
  const uint32_t lod = uint32_t(std::min<uint64_t>(R->current_lod, built));
  R->frame_started = true;
  paint(R, Subframe{lod, R->decrease_screen_res_now, R->decrease_sampling_rate_now});
  TVK_CUDA(cudaEventSynchronize(R->ev_stop));
  float ms = 0.0f;
  TVK_CUDA(cudaEventElapsedTime(&ms, R->ev_start, R->ev_stop));
  R->msec_current_frame += ms;
  // CompletedASubframe
  const bool first_sub = R->current_lod_offset == R->start_lod_offset &&
                         (!R->decrease_screen_res || R->decrease_screen_res_now) &&
                         (!R->decrease_sampling_rate || R->decrease_sampling_rate_now);
  const bool second_sub = !first_sub && (R->current_lod_offset == R->start_lod_offset ||
                                         (R->current_lod_offset + 1 == R->start_lod_offset &&
                                          !(R->decrease_screen_res || R->decrease_sampling_rate)));
  if (first_sub)
    R->msec_passed[0] = R->msec_current_frame;
  else if (second_sub)
    R->msec_passed[1] = R->msec_current_frame;
  R->msec_current_frame = 0.0f;
  info->lod = lod;
  info->decreased_screen_res = R->decrease_screen_res_now ? 1 : 0;
  info->decreased_sampling_rate = R->decrease_sampling_rate_now ? 1 : 0;
  info->render_width = R->render_w;
  info->render_height = R->render_h;
  info->min_lod = uint32_t(R->min_lod_view);
  info->start_lod = uint32_t(R->start_lod_offset);
  info->ms = ms;
  // AbstrRenderer::CheckForRedraw (AbstrRenderer.cpp:440-470)
  info->frame_complete =
      (R->current_lod_offset > R->min_lod_view || R->another_redraw_low_res) ? 0 : 1;
}

// The launches of one batch on the batch stream: the work counters cleared,
// one persistent kernel per launch (frame tables travel as kernel parameters),
// the reduced frames' upscales.
// Work items of the launches for `rpt` rays per thread: tiles of (16 rpt) x 8
// pixels, and the kernel variants that march them.
void set_batch_tiles(tvk_batch* B, uint32_t rpt) {
  B->rpt = rpt;
  for (size_t k = 0; k < B->launch.size(); ++k) {
    BatchLaunch& L = B->launch[k];
    const uint32_t tw = 16 * rpt;
    L.tile_first[0] = 0;
    for (uint32_t f = 0; f < L.n_frames; ++f)
      L.tile_first[f + 1] = L.tile_first[f] + ((L.frames[f].out_w + tw - 1) / tw) *
                                                  ((L.frames[f].out_h + 7) / 8);
    B->variant[k] = (B->variant[k] & 3) + (rpt == 2 ? 4 : 0);
  }
}

void enqueue_batch(tvk_batch* B, tvk_renderer* const* rs, const std::vector<PlannedFrame>& F,
                   uint32_t ctas) {
  const size_t nl = B->launch.size();
  TVK_CUDA(cudaMemsetAsync(B->d_next.p, 0, nl * sizeof(uint32_t), B->stream));
  uint64_t dummy = 0;
  // the launches are independent (each has its own frames and work counter):
  // run them concurrently, so a launch's last CTAs share the GPU with the next
  while (B->aux.size() + 1 < nl) {
    cudaStream_t st = nullptr;
    TVK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    B->aux.push_back(st);
  }
  while (B->fork_join.size() < nl) {
    cudaEvent_t e = nullptr;
    TVK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    B->fork_join.push_back(e);
  }
  if (nl > 1) TVK_CUDA(cudaEventRecord(B->fork_join[0], B->stream));
  for (size_t k = 0; k < nl; ++k) {
    cudaStream_t st = k == 0 ? B->stream : B->aux[k - 1];
    if (k > 0) TVK_CUDA(cudaStreamWaitEvent(st, B->fork_join[0], 0));
    launch_raycast_batch(B->launch[k], B->variant[k], B->d_next.as<uint32_t>() + k, ctas, st,
                         &dummy);
  }
  for (size_t k = 1; k < nl; ++k) {
    TVK_CUDA(cudaEventRecord(B->fork_join[k], B->aux[k - 1]));
    TVK_CUDA(cudaStreamWaitEvent(B->stream, B->fork_join[k], 0));
  }
  for (size_t i = 0; i < F.size(); ++i) launch_upscale_of(rs[i], F[i], B->stream, &dummy);
}

void paint_batch(tvk_batch* B, tvk_renderer* const* rs, uint32_t n) {
  TVK_CUDA(cudaSetDevice(B->device));
  for (uint32_t i = 0; i < n; ++i) {
    if (!rs[i]) fail(TVK_ERR_INVALID_ARG, "null renderer in the batch");
    if (rs[i]->device != B->device)
      fail(TVK_ERR_INVALID_ARG, "every renderer of a batch must be on the batch's device");
    for (uint32_t j = 0; j < i; ++j)
      if (rs[j] == rs[i]) fail(TVK_ERR_INVALID_ARG, "a renderer appears twice in the batch");
    if (rs[i]->cv_on && rs[i]->mode == TVK_RM_ISOSURFACE)
      fail(TVK_ERR_UNSUPPORTED, "ClearView frames are painted one at a time (tvk_paint)");
    if (rs[i]->vol) require_scalar(rs[i]->vol, "batches");
    if (rs[i]->hw_filter)
      fail(TVK_ERR_UNSUPPORTED, "batches use the exact lookups (hardware filtering off)");
  }
  // plan every frame on its renderer's stream, then order the batch stream after them
  std::vector<PlannedFrame> F;
  F.reserve(n);
  for (uint32_t i = 0; i < n; ++i) {
    tvk_renderer* R = rs[i];
    F.push_back(plan_frame(R, Subframe{R->lod, R->dec_screen, R->dec_sampling}));
    TVK_CUDA(cudaEventRecord(R->ev_ready, R->stream));
    TVK_CUDA(cudaStreamWaitEvent(B->stream, R->ev_ready, 0));
  }
  // group the frames by kernel variant, at most kBatchFrames per launch
  B->launch.clear();
  B->variant.clear();
  for (int v = 0; v < 4; ++v) {
    for (uint32_t i = 0; i < n; ++i) {
      const int fv = (F[i].P.bytes == 2 ? 2 : 0) + (F[i].P.mode == TVK_RM_ISOSURFACE ? 1 : 0);
      if (fv != v) continue;
      if (B->launch.empty() || B->variant.back() != v ||
          B->launch.back().n_frames == kBatchFrames) {
        B->launch.emplace_back();
        B->launch.back().n_frames = 0;
        B->launch.back().tile_first[0] = 0;
        B->variant.push_back(v);
      }
      BatchLaunch& L = B->launch.back();
      L.frames[L.n_frames] = F[i].P;
      L.n_frames++;
    }
  }
  const size_t nl = B->launch.size();
  B->d_next.ensure(nl * sizeof(uint32_t));
  // The shape of the launch sequence (what a captured graph bakes in): the
  // launches' variants and frame counts, and per frame the renderer, sizes and
  // upscale buffers.
  std::vector<uint64_t> shape = {nl, uint64_t(uintptr_t(B->d_next.p))};
  for (size_t k = 0; k < nl; ++k) {
    shape.push_back(uint64_t(B->variant[k]));
    shape.push_back(B->launch[k].n_frames);
  }
  for (uint32_t i = 0; i < n; ++i) {
    tvk_renderer* R = rs[i];
    for (uint64_t v : {uint64_t(uintptr_t(R)), uint64_t(F[i].rw), uint64_t(F[i].rh),
                       uint64_t(R->width), uint64_t(R->height), uint64_t(F[i].upscale),
                       uint64_t(uintptr_t(R->d_lowimg.p)), uint64_t(uintptr_t(R->d_img.p))})
      shape.push_back(v);
  }
  int sms = 0;
  TVK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device));
  auto max_per_sm_for = [&](uint32_t rpt) {
    uint32_t m = 1u << 30;
    for (int v : B->variant)
      m = std::min(m, uint32_t(std::max(1, batch_ctas_per_sm_max((v & 3) + (rpt == 2 ? 4 : 0)))));
    return m;
  };
  uint32_t rpt = B->fixed_rays_per_thread ? B->fixed_rays_per_thread : 1;
  uint32_t per_sm = B->fixed_ctas_per_sm ? std::min(B->fixed_ctas_per_sm, max_per_sm_for(rpt))
                                         : max_per_sm_for(rpt);
  bool tuned_now = false;
  const bool tune_grid = !B->fixed_ctas_per_sm, tune_rpt = !B->fixed_rays_per_thread;
  if (tune_grid || tune_rpt) {
    auto it = B->tuned.find(shape);
    if (it != B->tuned.end()) {
      if (tune_grid) per_sm = it->second.first;
      if (tune_rpt) rpt = it->second.second;
    } else if (B->autotune) {
      // time each candidate (rays per thread x persistent-grid size) on this
      // batch; the frames are re-rendered identically, only the counters are
      // cleared in between
      float best = std::numeric_limits<float>::infinity();
      for (uint32_t r : {1u, 2u}) {
        if (!tune_rpt && r != rpt) continue;
        const uint32_t mx = max_per_sm_for(r);
        std::vector<uint32_t> cands;
        if (!tune_grid) {
          cands.push_back(std::min(B->fixed_ctas_per_sm, mx));
        } else {
          for (uint32_t c : {mx, (mx * 3) / 4, mx / 2, 2u, 1u})
            if (c >= 1 && c <= mx && std::find(cands.begin(), cands.end(), c) == cands.end())
              cands.push_back(c);
        }
        set_batch_tiles(B, r);
        for (uint32_t c : cands) {
          TVK_CUDA(cudaEventRecord(B->ev_start, B->stream));
          enqueue_batch(B, rs, F, c * uint32_t(sms));
          TVK_CUDA(cudaEventRecord(B->ev_stop, B->stream));
          for (uint32_t i = 0; i < n; ++i)
            TVK_CUDA(cudaMemsetAsync(rs[i]->d_counters.p, 0, 4 * sizeof(unsigned long long),
                                     B->stream));
          TVK_CUDA(cudaEventSynchronize(B->ev_stop));
          float ms = 0;
          TVK_CUDA(cudaEventElapsedTime(&ms, B->ev_start, B->ev_stop));
          if (ms < best) {
            best = ms;
            per_sm = c;
            rpt = r;
          }
        }
      }
      B->tuned[shape] = {per_sm, rpt};
      tuned_now = true;
    }
  }
  set_batch_tiles(B, rpt);
  const uint32_t ctas = per_sm * uint32_t(sms);
  shape.push_back(ctas);
  shape.push_back(rpt);
  // one CUDA graph per launch shape; replays update the kernel nodes' frame
  // tables (new cameras, TFs, brick lists) in place
  const bool reused = B->exec && shape == B->graph_sig;
  if (!reused) {
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    B->exec = nullptr;
    B->graph = nullptr;
    B->graph_sig.clear();
    B->kernel_nodes.clear();
    TVK_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_batch(B, rs, F, ctas);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(B->stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    TVK_CUDA(cudaStreamEndCapture(B->stream, &B->graph));
    size_t nn = 0;
    TVK_CUDA(cudaGraphGetNodes(B->graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    TVK_CUDA(cudaGraphGetNodes(B->graph, nodes.data(), &nn));
    B->kernel_nodes.assign(nl, nullptr);
    const uint32_t* base = B->d_next.as<uint32_t>();
    for (cudaGraphNode_t node : nodes) {
      cudaGraphNodeType t;
      TVK_CUDA(cudaGraphNodeGetType(node, &t));
      if (t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      TVK_CUDA(cudaGraphKernelNodeGetParams(node, &kp));
      bool batch = false;
      for (int v = 0; v < 8; ++v) batch |= kp.func == batch_kernel_function(v);
      if (!batch) continue;
      // the launch is identified by its work counter, the second argument
      const uint32_t* counter = *static_cast<uint32_t* const*>(kp.kernelParams[1]);
      const size_t k = size_t(counter - base);
      if (k >= nl) fail(TVK_ERR_INTERNAL, "unrecognised batch kernel node");
      B->kernel_nodes[k] = node;
    }
    for (cudaGraphNode_t node : B->kernel_nodes)
      if (!node) fail(TVK_ERR_INTERNAL, "batch kernel node missing from the graph");
    TVK_CUDA(cudaGraphInstantiate(&B->exec, B->graph, 0));
    B->graph_sig = shape;
  } else {
    for (size_t k = 0; k < nl; ++k) {
      uint32_t* counter = B->d_next.as<uint32_t>() + k;
      void* args[2] = {&B->launch[k], &counter};
      cudaKernelNodeParams kp{};
      kp.func = const_cast<void*>(batch_kernel_function(B->variant[k]));
      kp.gridDim = dim3(ctas);
      kp.blockDim = dim3(128);
      kp.sharedMemBytes = 0;
      kp.kernelParams = args;
      TVK_CUDA(cudaGraphExecKernelNodeSetParams(B->exec, B->kernel_nodes[k], &kp));
    }
  }
  for (uint32_t i = 0; i < n; ++i) TVK_CUDA(cudaEventRecord(rs[i]->ev_start, B->stream));
  TVK_CUDA(cudaEventRecord(B->ev_start, B->stream));
  TVK_CUDA(cudaGraphLaunch(B->exec, B->stream));
  TVK_CUDA(cudaEventRecord(B->ev_stop, B->stream));
  for (uint32_t i = 0; i < n; ++i) TVK_CUDA(cudaEventRecord(rs[i]->ev_stop, B->stream));
  TVK_CUDA(cudaEventRecord(B->ev_done, B->stream));
  uint32_t tiles = 0;
  for (const BatchLaunch& L : B->launch) tiles += L.tile_first[L.n_frames];
  for (uint32_t i = 0; i < n; ++i) {
    tvk_renderer* R = rs[i];
    TVK_CUDA(cudaStreamWaitEvent(R->stream, B->ev_done, 0));
    R->launches += 1 + (F[i].upscale ? 1 : 0);  // its batch kernel (+ upscale)
    finish_frame(R, F[i]);
  }
  B->info.frames = n;
  B->info.tiles = tiles;
  B->info.ctas = ctas;
  B->info.ctas_per_sm = per_sm;
  B->info.rays_per_thread = rpt;
  B->info.launches = uint32_t(nl);
  B->info.graph_reused = reused ? 1 : 0;
  B->info.autotuned = tuned_now ? 1 : 0;
}

// The U-Net over the reduced frame's 16-channel input (BF16 [hp][wp][16]); the
// head's residual is added to the full-resolution base image in place.
void run_unet(tvk_learned* N, const void* x16, float* base_out, int out_h, int out_w,
              cudaStream_t s) {
  const int h0 = N->hp, w0 = N->wp;
  const size_t px0 = size_t(h0) * w0, px1 = px0 / 4, px2 = px0 / 16, px3 = px0 / 64;
  // activation buffers (BF16 elements), carved from one allocation
  constexpr int kBufs = 13;
  const size_t sizes[kBufs] = {px0 * 32, px0 * 32, px1 * 32, px1 * 48, px1 * 48, px2 * 48, px2 * 64,
                               px2 * 64, px3 * 64, px3 * 64, px2 * 64, px1 * 48, px0 * 32};
  size_t total = 0;
  for (size_t z : sizes) total += (z + 127) / 128 * 128;
  N->d_act.ensure(total * 2);
  N->d_head.ensure(px0 * 16 * sizeof(float));
  void* buf[kBufs];
  size_t off = 0;
  for (int i = 0; i < kBufs; ++i) {
    buf[i] = static_cast<uint8_t*>(N->d_act.p) + off * 2;
    off += (sizes[i] + 127) / 128 * 128;
  }
  void *a0 = buf[0], *s0 = buf[1], *p0 = buf[2], *a1 = buf[3], *s1 = buf[4], *p1 = buf[5];
  void *a2 = buf[6], *s2 = buf[7], *p2 = buf[8], *bt = buf[9], *d2 = buf[10], *d1 = buf[11];
  void *d0 = buf[12];
  // up_h > 0: x1 is the coarser level's up_h x up_w output, upsampled on the fly
  auto conv = [&](int li, const void* x1, const void* x2, int h, int w, void* ybf, float* yf,
                  int up_h = 0, int up_w = 0) {
    const UNetLayer& L = kUNet[li];
    CnnConv c{};
    c.upsample1 = up_h > 0 ? 1 : 0;
    c.h1 = up_h;
    c.w1 = up_w;
    c.x1 = x1;
    c.x2 = x2;
    c.c1 = L.c1;
    c.c2 = L.c2;
    c.n = 1;
    c.h = h;
    c.w = w;
    c.weights = static_cast<const uint16_t*>(N->d_w.p) + N->w_off[li];
    c.bias = N->d_b.as<float>() + N->b_off[li];
    c.cout = L.cout;
    c.slope = L.slope;
    c.y_bf16 = ybf;
    c.y_f32 = yf;
    c.split = L.cout;
    cnn_conv3x3(c, s);
  };
  conv(0, x16, nullptr, h0, w0, a0, nullptr);
  conv(1, a0, nullptr, h0, w0, s0, nullptr);
  cnn_avgpool2(s0, 1, h0, w0, 32, p0, s);
  conv(2, p0, nullptr, h0 / 2, w0 / 2, a1, nullptr);
  conv(3, a1, nullptr, h0 / 2, w0 / 2, s1, nullptr);
  cnn_avgpool2(s1, 1, h0 / 2, w0 / 2, 48, p1, s);
  conv(4, p1, nullptr, h0 / 4, w0 / 4, a2, nullptr);
  conv(5, a2, nullptr, h0 / 4, w0 / 4, s2, nullptr);
  cnn_avgpool2(s2, 1, h0 / 4, w0 / 4, 64, p2, s);
  conv(6, p2, nullptr, h0 / 8, w0 / 8, bt, nullptr);
  conv(7, bt, s2, h0 / 4, w0 / 4, d2, nullptr, h0 / 8, w0 / 8);
  conv(8, d2, s1, h0 / 2, w0 / 2, d1, nullptr, h0 / 4, w0 / 4);
  conv(9, d1, s0, h0, w0, d0, nullptr, h0 / 2, w0 / 2);
  // the head's residual, pixel-shuffled into the upscaled frame by the epilogue
  const UNetLayer& H = kUNet[10];
  CnnConv c{};
  c.x1 = d0;
  c.c1 = H.c1;
  c.n = 1;
  c.h = h0;
  c.w = w0;
  c.weights = static_cast<const uint16_t*>(N->d_w.p) + N->w_off[10];
  c.bias = N->d_b.as<float>() + N->b_off[10];
  c.cout = H.cout;
  c.slope = H.slope;
  c.y_f32 = N->d_head.as<float>();
  c.split = H.cout;
  cnn_conv3x3_shuffle(c, base_out, out_h, out_w, s);
}

// One learned frame: the reduced frame (half resolution, half sample rate) and
// its bilinear upscale, the network's residual added to it, then 1/64 of the
// pixels marched at full quality as probes; below threshold_db of probe PSNR
// the frame falls back to the plain full-quality render.
void paint_learned(tvk_renderer* R, tvk_learned* N, float threshold_db, tvk_learned_info* info) {
  if (R->device != N->device) fail(TVK_ERR_INVALID_ARG, "renderer and network on other devices");
  if (R->cv_on && R->mode == TVK_RM_ISOSURFACE)
    fail(TVK_ERR_UNSUPPORTED, "the learned reconstruction does not take ClearView frames");
  if (R->vol) require_scalar(R->vol, "the learned reconstruction");
  TVK_CUDA(cudaSetDevice(R->device));
  cudaStream_t s = R->stream;
  TVK_CUDA(cudaEventRecord(N->ev[0], s));
  // Both frames are planned before either launches: the full-rate plan (the
  // probe rays and the fallback) first, so that the viewport-sized buffers
  // are allocated before the reduced frame's parameters point into them.
  const Stage probe_stage{&N->p_bricks, &N->p_hbricks, N->ev_pstaged, &N->p_counters,
                          N->probe_stream};
  const PlannedFrame full = plan_frame(R, Subframe{0, false, false}, &probe_stage);
  const float saved_dec = R->screen_dec, saved_sdec = R->sample_dec;
  const bool saved_depth = R->depth_out;
  R->screen_dec = 2.0f;
  R->sample_dec = 2.0f;
  R->depth_out = true;  // the network reads the reduced frame's first-hit depth
  PlannedFrame low;
  try {
    low = plan_frame(R, Subframe{0, true, true});
  } catch (...) {
    R->screen_dec = saved_dec;
    R->sample_dec = saved_sdec;
    R->depth_out = saved_depth;
    throw;
  }
  R->screen_dec = saved_dec;
  R->sample_dec = saved_sdec;
  R->depth_out = saved_depth;
  // TF tables and empty-cell bits of both plans were written on the
  // renderer's stream: the probe stream starts after them
  TVK_CUDA(cudaEventRecord(N->ev_planned, s));
  TVK_CUDA(cudaStreamWaitEvent(N->probe_stream, N->ev_planned, 0));

  // probes: one pixel of every 8x8 block at full quality, offset per frame,
  // marched on the probe stream while the reduced frame and the network run
  const int stride = 8, ox = int((N->frame * 5u + 3u) % 8u), oy = int((N->frame * 3u + 1u) % 8u);
  ++N->frame;
  RenderParams P = full.P;
  P.stride = stride;
  P.off_x = ox;
  P.off_y = oy;
  P.out_w = (R->width - ox + stride - 1) / stride;
  P.out_h = (R->height - oy + stride - 1) / stride;
  P.spp = nullptr;
  N->d_sum.ensure(4 * P.out_w * P.out_h * sizeof(float) + 256);
  float4* probe = reinterpret_cast<float4*>(static_cast<uint8_t*>(N->d_sum.p) + 256);
  float* sum = N->d_sum.as<float>();
  P.out = probe;
  TVK_CUDA(cudaEventRecord(N->ev_pstart, N->probe_stream));
  launch_raycast(P, N->probe_stream, &R->launches);
  TVK_CUDA(cudaEventRecord(N->ev_pdone, N->probe_stream));

  // the reduced frame, upscaled into the viewport image, and the network
  launch_raycast(low.P, s, &R->launches);
  launch_upscale_of(R, low, s, &R->launches);
  TVK_CUDA(cudaEventRecord(N->ev[1], s));
  const float* lowimg = low.upscale ? R->d_lowimg.as<float>() : R->d_img.as<float>();
  N->hp = int((low.rh + 7) / 8 * 8);
  N->wp = int((low.rw + 7) / 8 * 8);
  if (2 * N->hp < int(R->height) || 2 * N->wp < int(R->width))
    fail(TVK_ERR_INTERNAL, "reduced frame smaller than half the viewport");
  DevBuf& x16 = N->d_input;
  x16.ensure(size_t(N->hp) * N->wp * 16 * 2);
  cnn_prepare_input(lowimg, R->d_depth.as<float>(), int(low.rh), int(low.rw), N->hp, N->wp,
                    x16.p, s);
  run_unet(N, x16.p, R->d_img.as<float>(), int(R->height), int(R->width), s);
  R->launches += kUNetLayers + 8;
  TVK_CUDA(cudaEventRecord(N->ev[2], s));

  // the judge: probe error against the network's frame
  TVK_CUDA(cudaStreamWaitEvent(s, N->ev_pdone, 0));
  TVK_CUDA(cudaMemsetAsync(sum, 0, sizeof(float), s));
  cnn_probe_mse(R->d_img.as<float>(), int(R->width), reinterpret_cast<const float*>(probe),
                int(P.out_w), int(P.out_h), stride, ox, oy, sum, s);
  N->h_sum.ensure(sizeof(float));
  TVK_CUDA(cudaMemcpyAsync(N->h_sum.p, sum, sizeof(float), cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaEventRecord(N->ev[3], s));
  TVK_CUDA(cudaEventSynchronize(N->ev[3]));
  if (cnn_tc_timeouts(true))
    fail(TVK_ERR_INTERNAL, "a tensor-core convolution gave up waiting for its MMAs");
  const double mse = double(*N->h_sum.as<float>()) / (4.0 * P.out_w * P.out_h);
  const float psnr = mse > 0 ? float(10.0 * std::log10(1.0 / mse)) : 1000.0f;
  const bool fall_back = psnr < threshold_db;
  if (fall_back) {
    TVK_CUDA(cudaMemsetAsync(N->p_counters.p, 0, 4 * sizeof(unsigned long long), s));
    launch_raycast(full.P, s, &R->launches);
    // the frame's stats are the plain frame's
    TVK_CUDA(cudaMemcpyAsync(R->d_counters.p, N->p_counters.p, 4 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToDevice, s));
  }
  TVK_CUDA(cudaEventRecord(N->ev[4], s));
  finish_frame(R, fall_back ? full : low);
  TVK_CUDA(cudaEventSynchronize(N->ev[4]));
  float t[4], tp = 0.0f;
  for (int i = 0; i < 4; ++i) TVK_CUDA(cudaEventElapsedTime(&t[i], N->ev[i], N->ev[i + 1]));
  TVK_CUDA(cudaEventElapsedTime(&tp, N->ev_pstart, N->ev_pdone));
  info->probe_psnr_db = psnr;
  info->fell_back = fall_back ? 1 : 0;
  info->ms_reduced = t[0];
  info->ms_network = t[1];
  info->ms_probe = tp;
  info->ms_fallback = t[3];
  info->ms_judge = t[2];
  TVK_CUDA(cudaEventElapsedTime(&info->ms_frame, N->ev[0], N->ev[4]));
  info->reduced_width = low.rw;
  info->reduced_height = low.rh;
}

// GLGridLeaper.cpp:266-273: hash table size from the brick volume
uint32_t reference_hash_size(const tvk_volume* v) {
  const double rmax = double(v->brick_size[0]) * v->brick_size[1] * v->brick_size[2] / 32768.0;
  return std::max<uint32_t>(15, uint32_t(509 / rmax));
}

// GLVolumePool.cpp:89-107 GetFloatBrickLayout
void float_brick_layout(const tvk_volume* V, uint32_t lod, float out[3]) {
  for (int a = 0; a < 3; ++a) {
    const uint32_t inner = V->brick_size[a] - 2 * V->overlap;
    float c = float(V->dims[a]) / float(inner);
    c /= float(uint64_t(1) << lod);
    if (float(uint32_t(c)) == c) c -= c * std::numeric_limits<float>::epsilon();
    out[a] = c;
  }
}

// GLVolumePool::RecomputeVisibility (GLVolumePool.cpp:1580-1700) with the
// ContainsData tests of :962-989 (the 2D mode's gradient test always passes:
// bricks of an ExtendedOctree carry the gradient range [-DBL_MAX, DBL_MAX],
// MaxMinDataBlock.cpp:175-195).  Every entry is reset to MISSING; cached
// bricks keep their slot when visible, else become EMPTY and their slot is
// flagged for early eviction (RecomputeVisibilityForBrickPool, :991-1018);
// then every brick not cached-and-visible that holds nothing visible becomes
// CHILD_EMPTY when all its children are CHILD_EMPTY (finest bricks by
// definition), else EMPTY (RecomputeVisibilityForOctree, :1020-1359).
void pool_visibility(tvk_pool* pool, int mode, double lo, double hi, float iso) {
  const tvk_volume* V = pool->vol;
  auto contains = [&](uint64_t id) {
    const double mn = V->bmin[id], mx = V->bmax[id];
    return mode == TVK_RM_ISOSURFACE ? (double(iso) >= mn && double(iso) <= mx)
                                     : (hi >= mn && lo <= mx);
  };
  std::fill(pool->page.begin(), pool->page.end(), kBiMissing);
  for (uint32_t i = 0; i < pool->n_slots; ++i) {
    tvk_pool::Slot& S = pool->slots[i];
    if (S.brick < 0) continue;
    const bool now = contains(uint64_t(S.brick)), before = S.time > 1;
    if (now) {
      if (!before) S.time = S.orig_time;  // Restore
      pool->page[uint64_t(S.brick)] = i + kBiFlagCount;
    } else {
      if (before) {  // FlagEmpty
        S.orig_time = S.time;
        S.time = 1;
      }
      pool->page[uint64_t(S.brick)] = kBiEmpty;
    }
  }
  const size_t n_lods = V->lod_first.size() - 1;
  for (size_t l = 0; l < n_lods; ++l) {
    const LodInfo& li = V->lods[l];
    for (uint64_t k = 0; k < V->lod_first[l + 1] - V->lod_first[l]; ++k) {
      const uint64_t id = V->lod_first[l] + k;
      if (pool->page[id] >= kBiFlagCount || contains(id)) continue;
      bool child_empty = true;
      if (l > 0) {
        const LodInfo& lc = V->lods[l - 1];
        const uint64_t x = k % li.bricks[0], y = (k / li.bricks[0]) % li.bricks[1],
                       z = k / (li.bricks[0] * li.bricks[1]);
        for (int c = 0; c < 8 && child_empty; ++c) {
          const uint64_t cx = 2 * x + (c & 1), cy = 2 * y + ((c >> 1) & 1), cz = 2 * z + (c >> 2);
          if (cx >= lc.bricks[0] || cy >= lc.bricks[1] || cz >= lc.bricks[2]) continue;
          const uint64_t cid = V->lod_first[l - 1] + cx + cy * lc.bricks[0] +
                               cz * lc.bricks[0] * lc.bricks[1];
          child_empty = pool->page[cid] == kBiChildEmpty;
        }
      }
      pool->page[id] = child_empty ? kBiChildEmpty : kBiEmpty;
    }
  }
}

// Copies brick `id` into slot `slot` on the paging stream (UploadBrick,
// GLVolumePool.cpp:673-717): a visible brick evicted from the slot becomes
// MISSING (one flagged empty keeps its EMPTY / CHILD_EMPTY entry).
uint64_t pool_upload(tvk_pool* pool, uint32_t slot, uint64_t id, uint64_t time) {
  const tvk_volume* V = pool->vol;
  tvk_pool::Slot& S = pool->slots[slot];
  if (S.brick >= 0 && S.time > 1) pool->page[uint64_t(S.brick)] = kBiMissing;
  S.brick = int64_t(id);
  S.time = time;
  pool->page[id] = slot + kBiFlagCount;
  const size_t bytes = size_t(V->sizes[3 * id]) * V->sizes[3 * id + 1] * V->sizes[3 * id + 2] *
                       V->bytes;
  void* dst = static_cast<uint8_t*>(pool->d_slots.p) + size_t(slot) * pool->slot_voxels * V->bytes;
  const void* src = pool->host_source
                        ? static_cast<const void*>(pool->h_bricks.as<uint8_t>() +
                                                   V->offsets[id] * V->bytes)
                        : static_cast<const void*>(static_cast<const uint8_t*>(device_bricks(V)) +
                                                   V->offsets[id] * V->bytes);
  TVK_CUDA(cudaMemcpyAsync(dst, src, bytes,
                           pool->host_source ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                           pool->page_stream));
  return bytes;
}

void pool_upload_page_table(tvk_pool* pool) {
  const size_t n = pool->page.size();
  // the staging copy of the previous upload may still be in flight
  TVK_CUDA(cudaEventSynchronize(pool->ev_paged));
  std::memcpy(pool->h_page.p, pool->page.data(), n * sizeof(uint32_t));
  TVK_CUDA(cudaMemcpyAsync(pool->d_page.p, pool->h_page.p, n * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, pool->page_stream));
  TVK_CUDA(cudaEventRecord(pool->ev_paged, pool->page_stream));
}

// One GridLeaper frame (GLGridLeaper::Render3DRegion, GLGridLeaper.cpp:914-1154):
// passes of the traversal, each followed by paging in the bricks its rays
// reported missing, until a pass reports none or max_passes is reached.
void leaper_paint(tvk_renderer* R, tvk_pool* pool, uint32_t max_passes, tvk_leaper_info* info) {
  const tvk_volume* V = R->vol;
  if (!V || V != pool->vol) fail(TVK_ERR_STATE, "the renderer's volume is not the pool's volume");
  const bool iso_mode = R->mode == TVK_RM_ISOSURFACE;
  if (!iso_mode && R->tf.empty()) fail(TVK_ERR_STATE, "no transfer function set");
  if (R->width == 0 || R->height == 0) fail(TVK_ERR_STATE, "no viewport (tvk_resize)");
  if (R->mode == TVK_RM_2DTRANS && !R->tf_2d) fail(TVK_ERR_STATE, "2D mode needs a 2D TF");
  if (R->mode == TVK_RM_1DTRANS && R->tf_2d) fail(TVK_ERR_STATE, "1D mode needs a 1D TF");
  if (R->clip_on) fail(TVK_ERR_UNSUPPORTED, "the GridLeaper does not clip (disable the clip plane)");
  TVK_CUDA(cudaSetDevice(R->device));
  const uint64_t launches0 = R->launches;
  const float srm = R->srm;
  // GLGridLeaper-blend.glsl OpacityCorrectColor with ocFactor = 1 / srm
  // (a colour pool's alpha is the TF's alpha, so the same corrected table)
  if (!R->tf.empty()) upload_tf(R, 1.0f / srm);
  // CalculateScaling and GetNormalizedIsovalue with the bit width per
  // channel (8 for RGBA8 colour volumes)
  const bool color = V->dtype == TVK_RGBA8;
  const uint32_t cbits = color ? 8 : 8 * V->bytes;
  const uint32_t imax = (1u << cbits) - 1;
  const float trans_scale = float(double(imax) / V->range_max);
  const float iso_norm = float(double(R->isovalue) / double(1u << cbits));
  // the visible range of the TF (AbstrRenderer::ContainsData's limits)
  uint64_t nz_lo = R->tf_w, nz_hi = 0;
  for (uint32_t y = 0; y < R->tf_h; ++y)
    for (uint32_t x = 0; x < R->tf_w; ++x)
      if (R->tf[4 * (size_t(y) * R->tf_w + x) + 3] != 0) {
        nz_lo = std::min<uint64_t>(nz_lo, x);
        nz_hi = std::max<uint64_t>(nz_hi, x);
      }
  const double rescale = V->range_max / double(std::max<uint32_t>(R->tf_w, 2) - 1);
  const double lo = double(nz_lo) * rescale, hi = double(nz_hi) * rescale;
  if (!pool->vis_valid || pool->vis_mode != R->mode || pool->vis_lo != lo ||
      pool->vis_hi != hi || pool->vis_iso != R->isovalue) {
    pool_visibility(pool, R->mode, lo, hi, R->isovalue);
    if (pool->page[pool->coarsest] == kBiMissing) {
      // The coarsest brick was evicted while it held nothing visible and now
      // does: a ray whose every coarser fallback is MISSING would never find
      // a brick (GLVolumePool.cpp:553-590 loops until one is found), so the
      // single brick of the coarsest LOD is brought back first.
      uint32_t oldest = 0;
      for (uint32_t i = 1; i < pool->n_slots; ++i)
        if (pool->slots[i].time < pool->slots[oldest].time) oldest = i;
      pool_upload(pool, oldest, pool->coarsest, ~uint64_t(0));
    }
    pool->vis_valid = true;
    pool->vis_mode = R->mode;
    pool->vis_lo = lo;
    pool->vis_hi = hi;
    pool->vis_iso = R->isovalue;
    pool_upload_page_table(pool);
  }

  // empty-cell distances of every brick for this TF / isovalue (colour
  // bricks have no macro cells)
  if (R->cell_skip && !color) update_empty_cells(R, V, trans_scale, iso_mode, iso_norm);
  const View view = make_view(R->eye, R->at, R->up, R->fovy, R->width, R->height, R->model);
  LeaperParams L;
  std::memset(&L, 0, sizeof(L));
  RenderParams& P = L.R;
  P.bytes = V->bytes;
  P.tf = R->slots[R->slot].d_tf.as<float4>();
  P.tf_col_nonzero = R->slots[R->slot].d_tfcol.as<uint8_t>();
  P.tf_w = R->tf_w;
  P.tf_h = R->tf_h;
  P.mode = R->mode;
  P.lighting = R->lighting ? 1 : 0;
  P.light_model = R->light_model;
  P.trans_scale = trans_scale;
  const float mg = float(V->max_grad);
  P.grad_scale = (mg == 0) ? 1.0f : 1.0f / mg;
  P.inv_max_raw = V->bytes == 2 ? 1.0f / 65535.0f : 1.0f / 255.0f;
  for (int a = 0; a < 3; ++a) {
    P.light_a[a] = R->ambient[a] * R->ambient[3];
    P.light_d[a] = R->diffuse[a] * R->diffuse[3];
    P.light_s[a] = R->specular[a] * R->specular[3];
    P.light_dir[a] = R->light_dir[a];
    P.domain_scale[a] = 1.0f;
    P.iso_diffuse[a] = (R->diffuse[a] * R->diffuse[3]) * R->iso_color[a];
  }
  P.kx = view.kx;
  P.ky = view.ky;
  P.inv_w2 = view.inv_w2;
  P.inv_h2 = view.inv_h2;
  P.znear = R->znear;
  P.zfar = R->zfar;
  P.iso_norm = iso_norm;
  P.width = P.out_w = R->width;
  P.height = P.out_h = R->height;
  P.stride = 1;
  const size_t npix = size_t(R->width) * R->height;
  R->d_img.ensure(npix * sizeof(float4));
  R->d_spp.ensure(npix * sizeof(uint32_t));
  R->d_counters.ensure(4 * sizeof(unsigned long long));
  P.out = R->d_img.as<float4>();
  P.spp = R->d_spp.as<uint32_t>();
  P.counters = R->d_counters.as<unsigned long long>();
  // pool geometry
  L.slots = pool->d_slots.p;
  L.slot_voxels = pool->slot_voxels;
  L.page = pool->d_page.as<uint32_t>();
  L.brick_dims = pool->d_dims.as<uint32_t>();
  const uint32_t n_lods = uint32_t(V->lod_first.size() - 1);
  L.max_lod = n_lods - 1;
  for (uint32_t l = 0; l < n_lods; ++l) {
    float_brick_layout(V, l, L.layout[l]);
    const LodInfo& li = V->lods[l];
    for (int a = 0; a < 3; ++a)
      if (uint64_t(L.layout[l][a]) >= li.bricks[a])
        fail(TVK_ERR_UNSUPPORTED, "the pool's float brick layout exceeds the LOD's bricks");
    L.lod_offset[l] = uint32_t(V->lod_first[l]);
    L.lod_lx[l] = uint32_t(li.bricks[0]);
    L.lod_lxy[l] = uint32_t(li.bricks[0] * li.bricks[1]);
  }
  float ext[3];
  const float dmax = float(std::max(V->dims[0], std::max(V->dims[1], V->dims[2])));
  for (int a = 0; a < 3; ++a) {
    L.vol_size[a] = float(V->dims[a]);
    L.max_inner[a] = float(V->brick_size[a] - 2 * V->overlap);
    ext[a] = float(V->dims[a]) / dmax;  // GetVolumeAABB extent (scale 1)
  }
  L.ghost = float(V->overlap);
  // CullingLOD::SetScreenParams (CullingLOD.cpp:57-67), GLVolumePool::Enable (:790-803)
  L.lod_factor = 2.0f * std::tan(R->fovy * ((3.1416f / 180.0f) / 2.0f)) * 1.0f / float(R->height);
  L.lod0_err = std::max(ext[0] / L.vol_size[0], std::max(ext[1] / L.vol_size[1], ext[2] / L.vol_size[2]));
  // ComputeEyeToModelMatrix (GLGridLeaper.cpp:558-571): eye -> model -> [0, 1]^3
  double e2n[3][4];
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) e2n[r][c] = view.inv[r][c] / double(ext[r]);
    e2n[r][3] += 0.5;
  }
  for (int r = 0; r < 3; ++r) {
    double acc = view.mv[r][3];
    for (int c = 0; c < 4; ++c) L.eye2norm[r][c] = float(e2n[r][c]);
    for (int c = 0; c < 3; ++c) {
      L.norm2eye[r][c] = float(view.mv[r][c] * double(ext[c]));
      acc -= view.mv[r][c] * double(ext[c]) * 0.5;
      L.norm_to_eye_n[r][c] = float(view.mv[r][c]);
    }
    L.norm2eye[r][3] = float(acc);
  }
  // GLGridLeaper.cpp:739-742: the light direction through the eye -> norm
  // matrix (normalised), and the camera's eye point taken through the same
  // matrix as if it were an eye-space point
  double ld[3], em[3];
  for (int r = 0; r < 3; ++r) {
    ld[r] = e2n[r][0] * R->light_dir[0] + e2n[r][1] * R->light_dir[1] + e2n[r][2] * R->light_dir[2];
    em[r] = e2n[r][0] * R->eye[0] + e2n[r][1] * R->eye[1] + e2n[r][2] * R->eye[2] + e2n[r][3];
  }
  const double ll = std::sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2]);
  for (int a = 0; a < 3; ++a) {
    L.light_dir_model[a] = float(ld[a] / ll);
    L.eye_model[a] = float(em[a]);
  }
  L.srm = srm;
  L.hash = pool->d_hash.as<uint32_t>();
  L.hash_size = pool->hash_size;
  L.rehash = pool->rehash;
  const LodInfo& l0 = V->lods[0];
  L.ser_x = uint32_t(l0.bricks[0]);
  L.ser_xy = uint32_t(l0.bricks[0] * l0.bricks[1]);
  L.ser_xyz = uint32_t(l0.bricks[0] * l0.bricks[1] * l0.bricks[2]);
  pool->d_resume_pos.ensure(npix * sizeof(float4));
  pool->d_resume_col.ensure(npix * sizeof(float4));
  L.resume_pos = pool->d_resume_pos.as<float4>();
  L.resume_col = pool->d_resume_col.as<float4>();
  L.cell_dist = (R->cell_skip && !color) ? R->slots[R->slot].d_dist.as<uint8_t>() : nullptr;
  L.cell_off = static_cast<const uint64_t*>(V->d_cell_meta);

  std::memset(info, 0, sizeof(*info));
  const uint64_t l0n = L.ser_xyz;
  TVK_CUDA(cudaEventRecord(R->ev_start, R->stream));
  for (uint32_t pass = 0; pass < std::max(1u, max_passes); ++pass) {
    L.first_pass = pass == 0 ? 1u : 0u;
    TVK_CUDA(cudaStreamWaitEvent(R->stream, pool->ev_paged, 0));
    TVK_CUDA(cudaMemsetAsync(pool->d_hash.p, 0, pool->hash_size * sizeof(uint32_t), R->stream));
    TVK_CUDA(cudaMemsetAsync(R->d_counters.p, 0, 4 * sizeof(unsigned long long), R->stream));
    TVK_CUDA(cudaEventRecord(pool->ev_pass[0], R->stream));
    launch_leaper(L, R->stream, &R->launches);
    TVK_CUDA(cudaEventRecord(pool->ev_pass[1], R->stream));
    TVK_CUDA(cudaMemcpyAsync(pool->h_hash.p, pool->d_hash.p, pool->hash_size * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, R->stream));
    R->h_counters.ensure(4 * sizeof(unsigned long long));
    TVK_CUDA(cudaMemcpyAsync(R->h_counters.p, R->d_counters.p, 4 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, R->stream));
    TVK_CUDA(cudaStreamSynchronize(R->stream));
    float pass_ms = 0.0f;
    TVK_CUDA(cudaEventElapsedTime(&pass_ms, pool->ev_pass[0], pool->ev_pass[1]));
    info->ms_traversal += pass_ms;
    info->samples += R->h_counters.as<unsigned long long>()[0];
    ++info->passes;
    // the missing bricks this pass reported (GLHashTable::GetData)
    std::vector<uint64_t> want;
    const uint32_t* h = pool->h_hash.as<uint32_t>();
    for (uint32_t i = 0; i < pool->hash_size; ++i) {
      if (!h[i]) continue;
      const uint64_t key = h[i] - 1u;
      const uint64_t lod = key / l0n, rem = key % l0n;
      const uint64_t x = rem % L.ser_x, y = (rem / L.ser_x) % (L.ser_xy / L.ser_x),
                     z = rem / L.ser_xy;
      if (lod >= n_lods) continue;
      const LodInfo& li = V->lods[lod];
      if (x >= li.bricks[0] || y >= li.bricks[1] || z >= li.bricks[2]) continue;
      want.push_back(V->lod_first[lod] + x + y * li.bricks[0] + z * li.bricks[0] * li.bricks[1]);
    }
    info->missing_last = uint32_t(want.size());
    pool->requests = want;
    std::sort(pool->requests.begin(), pool->requests.end());
    if (want.empty()) {
      info->converged = 1;
      break;
    }
    if (pass + 1 >= std::max(1u, max_passes)) break;
    // PrepareForPaging (:955-959): slots by creation time (never used 0,
    // flagged empty 1, the coarsest brick the maximum); the bricks go into the
    // first n - 1 of that order (UploadBrick, :768-778).  Only as many slots
    // as there are requests are needed, so only those are ordered (ties by
    // slot index, as a stable sort would leave them).
    const auto t_host0 = std::chrono::steady_clock::now();
    std::vector<std::pair<uint64_t, uint32_t>> order(pool->n_slots);
    for (uint32_t i = 0; i < pool->n_slots; ++i) order[i] = {pool->slots[i].time, i};
    const size_t need = std::min<size_t>(want.size(), order.size());
    std::partial_sort(order.begin(), order.begin() + need, order.end());
    uint32_t ins = 0;
    for (uint64_t id : want) {
      if (ins + 1 >= pool->n_slots || ins >= need) break;  // every slot replaced this round
      if (pool->page[id] >= kBiFlagCount) continue;
      info->bytes_paged += pool_upload(pool, order[ins++].second, id, pool->clock++);
      ++info->paged;
      ++pool->paged_total;
    }
    pool_upload_page_table(pool);
    info->ms_host += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() -
                                                              t_host0).count();
  }
  TVK_CUDA(cudaEventRecord(R->ev_stop, R->stream));
  TVK_CUDA(cudaEventSynchronize(R->ev_stop));
  TVK_CUDA(cudaEventElapsedTime(&info->ms, R->ev_start, R->ev_stop));
  uint32_t resident = 0;
  for (const tvk_pool::Slot& sl : pool->slots) resident += sl.brick >= 0 ? 1u : 0u;
  info->resident = resident;
  R->render_w = R->width;
  R->render_h = R->height;
  R->stats.bricks_visible = resident;
  R->stats.bricks_total = V->total_bricks;
  R->stats.kernel_launches = R->launches - launches0;
  R->painted = true;
}

}  // namespace
}  // namespace tvk

// ------------------------------------------------------------------ C ABI

using tvk::guarded;

extern "C" {

const char* tvk_status_string(tvk_status s) {
  switch (s) {
    case TVK_OK: return "ok";
    case TVK_ERR_INVALID_ARG: return "invalid argument";
    case TVK_ERR_CUDA: return "CUDA error";
    case TVK_ERR_OUT_OF_MEMORY: return "out of memory";
    case TVK_ERR_UNSUPPORTED: return "unsupported";
    case TVK_ERR_STATE: return "invalid state";
    case TVK_ERR_INTERNAL: return "internal error";
  }
  return "unknown status";
}

const char* tvk_last_error(void) { return tvk::g_last_error.c_str(); }

int tvk_abi_version(void) { return TVK_ABI_VERSION; }

tvk_status tvk_volume_create(const void* voxels, tvk_dtype dtype, const uint64_t dims[3],
                             const uint32_t brick_size[3], uint32_t overlap, int clamp_to_edge,
                             tvk_volume** out) {
  return guarded([&] {
    REQUIRE(out, "null output handle");
    *out = tvk::create_volume(voxels, false, dtype, dims, brick_size, overlap, clamp_to_edge);
  });
}

tvk_status tvk_volume_create_device(const void* device_voxels, tvk_dtype dtype,
                                    const uint64_t dims[3], const uint32_t brick_size[3],
                                    uint32_t overlap, int clamp_to_edge, tvk_volume** out) {
  return guarded([&] {
    REQUIRE(out, "null output handle");
    *out = tvk::create_volume(device_voxels, true, dtype, dims, brick_size, overlap,
                              clamp_to_edge);
  });
}

tvk_status tvk_volume_create_ex(const void* voxels, tvk_dtype dtype, const uint64_t dims[3],
                                const uint32_t brick_size[3], uint32_t overlap, uint32_t flags,
                                tvk_volume** out) {
  return guarded([&] {
    REQUIRE(out, "null output handle");
    REQUIRE((flags & ~uint32_t(TVK_VOLUME_CLAMP_TO_EDGE | TVK_VOLUME_DEVICE_INPUT |
                               TVK_VOLUME_MEDIAN | TVK_VOLUME_LOD0_ONLY)) == 0,
            "unknown volume flag");
    *out = tvk::create_volume(voxels, (flags & TVK_VOLUME_DEVICE_INPUT) != 0, dtype, dims,
                              brick_size, overlap, (flags & TVK_VOLUME_CLAMP_TO_EDGE) ? 1 : 0,
                              (flags & TVK_VOLUME_MEDIAN) != 0,
                              (flags & TVK_VOLUME_LOD0_ONLY) == 0);
  });
}

tvk_status tvk_eo_read_brick(const char* path, uint64_t offset, uint32_t uvf_version,
                             uint64_t index, void* out, size_t capacity, size_t* n_bytes) {
  return guarded([&] {
    REQUIRE(path && n_bytes, "null argument");
    tvk::EoFile e;
    tvk::eo_open(path, offset, uvf_version, e);
    REQUIRE(index < e.toc.size(), "brick index beyond the table of contents");
    const uint32_t bs[3] = {uint32_t(e.brick_size[0]), uint32_t(e.brick_size[1]),
                            uint32_t(e.brick_size[2])};
    const std::vector<tvk::LodInfo> lods = tvk::lod_table(e.dims, bs, e.overlap);
    // the brick's LOD and coordinates from its TOC index
    uint64_t k = index;
    size_t l = 0;
    while (l < lods.size()) {
      const uint64_t nl = lods[l].bricks[0] * lods[l].bricks[1] * lods[l].bricks[2];
      if (k < nl) break;
      k -= nl;
      ++l;
    }
    REQUIRE(l < lods.size(), "brick index beyond the LOD table");
    const uint64_t c[3] = {k % lods[l].bricks[0], (k / lods[l].bricks[0]) % lods[l].bricks[1],
                           k / (lods[l].bricks[0] * lods[l].bricks[1])};
    uint32_t n[3];
    tvk::brick_size(lods[l], bs, e.overlap, c, n);
    const size_t vb = size_t(e.component_type == 1 ? 2 : (e.component_type == 0 ? 1 : 0)) *
                      size_t(e.components);
    if (vb == 0)
      tvk::fail(TVK_ERR_UNSUPPORTED, "ExtendedOctree: component types other than uint8/uint16");
    const size_t nb = size_t(n[0]) * n[1] * n[2] * vb;
    *n_bytes = nb;
    if (!out) return;
    REQUIRE(capacity >= nb, "output smaller than the brick");
    std::vector<uint8_t> brick;
    tvk::eo_read_brick(e, index, nb, brick);
    std::memcpy(out, brick.data(), nb);
  });
}

namespace {

// The volume of the ExtendedOctree at byte `offset` of `path`; throws tvk::Error.
void open_eo_volume(const char* path, uint64_t offset, uint32_t uvf_version, uint32_t flags,
                    tvk_volume** out) {
  REQUIRE(path && out, "null argument");
  *out = nullptr;
  tvk::EoFile e;
  tvk::eo_open(path, offset, uvf_version, e);
  tvk_dtype dt;
  if (e.component_type == 0 && e.components == 1) dt = TVK_U8;
  else if (e.component_type == 1 && e.components == 1) dt = TVK_U16;
  else if (e.component_type == 0 && e.components == 4) dt = TVK_RGBA8;
  else
    tvk::fail(TVK_ERR_UNSUPPORTED,
              "ExtendedOctree: 1-component uint8 / uint16 and 4-component uint8 volumes only");
  if (e.normals) tvk::fail(TVK_ERR_UNSUPPORTED, "ExtendedOctree: precomputed normals");
  if (e.aspect[0] != 1.0 || e.aspect[1] != 1.0 || e.aspect[2] != 1.0)
    tvk::fail(TVK_ERR_UNSUPPORTED, "ExtendedOctree: volume aspect other than 1:1:1");
  const uint32_t bs[3] = {uint32_t(e.brick_size[0]), uint32_t(e.brick_size[1]),
                          uint32_t(e.brick_size[2])};
  const uint32_t ov = e.overlap;
  const size_t vb = size_t(dt == TVK_U16 ? 2 : 1) * e.components;  // bytes per voxel
  // the flat volume from the LOD-0 bricks' inner voxels
  const std::vector<tvk::LodInfo> lods = tvk::lod_table(e.dims, bs, ov);
  std::vector<tvk_brick_md> md0;
  tvk::brick_metadata(lods[0], bs, ov, md0);
  std::vector<uint8_t> raw(size_t(e.dims[0] * e.dims[1] * e.dims[2]) * vb), brick;
  const uint64_t core[3] = {bs[0] - 2ull * ov, bs[1] - 2ull * ov, bs[2] - 2ull * ov};
  for (uint64_t k = 0; k < md0.size(); ++k) {
    const uint32_t* n = md0[k].n_voxels;
    tvk::eo_read_brick(e, k, size_t(n[0]) * n[1] * n[2] * vb, brick);
    const uint64_t c[3] = {k % lods[0].bricks[0], (k / lods[0].bricks[0]) % lods[0].bricks[1],
                           k / (lods[0].bricks[0] * lods[0].bricks[1])};
    for (uint32_t z = ov; z + ov < n[2]; ++z)
      for (uint32_t y = ov; y + ov < n[1]; ++y) {
        const uint64_t gx = c[0] * core[0], gy = c[1] * core[1] + (y - ov),
                       gz = c[2] * core[2] + (z - ov);
        std::memcpy(raw.data() + ((gz * e.dims[1] + gy) * e.dims[0] + gx) * vb,
                    brick.data() + ((size_t(z) * n[1] + y) * n[0] + ov) * vb,
                    size_t(n[0] - 2 * ov) * vb);
      }
  }
  // Rebuild from the LOD-0 data: the border setting (not recorded in the
  // header) is the one whose LOD-0 bricks equal the file's, trying `flags`
  // first; then the filter whose coarser bricks equal the file's.  Where no
  // filter reproduces a coarser brick the file's bytes are kept: the
  // converter's coarser bricks can carry stale buffer contents in some ghost
  // corners (DownsampleBrick skips its memset under clamp, ExtendedOctree
  // Converter.inc:261-262, and FillOverlap copies corners from neighbours
  // not yet filled), which no rebuild reproduces.
  const bool lod0_only = (flags & TVK_VOLUME_LOD0_ONLY) != 0;
  const bool clamp0 = (flags & TVK_VOLUME_CLAMP_TO_EDGE) != 0,
             median0 = (flags & TVK_VOLUME_MEDIAN) != 0 && !lod0_only;
  std::vector<uint8_t> dev;
  struct Drop {
    void operator()(tvk_volume* v) const {
      tvk::free_volume_device(v);
      delete v;
    }
  };
  using VolPtr = std::unique_ptr<tvk_volume, Drop>;
  auto brick_bytes = [&](const tvk_volume* V, uint64_t k) {
    return size_t(V->sizes[3 * k]) * V->sizes[3 * k + 1] * V->sizes[3 * k + 2] * vb;
  };
  auto same_as_file = [&](const tvk_volume* V, uint64_t k) {
    const size_t nb = brick_bytes(V, k);
    tvk::eo_read_brick(e, k, nb, brick);
    dev.resize(nb);
    TVK_CUDA(cudaMemcpy(dev.data(), static_cast<const uint8_t*>(V->d_pool) + V->offsets[k] * vb,
                        nb, cudaMemcpyDeviceToHost));
    return std::memcmp(dev.data(), brick.data(), nb) == 0;
  };
  for (int ci = 0; ci < 2; ++ci) {
    const bool clamp = clamp0 ^ (ci == 1);
    VolPtr best;
    std::vector<uint64_t> best_bad;
    for (int mi = 0; mi < (lod0_only ? 1 : 2); ++mi) {
      const bool median = median0 ^ (mi == 1);
      VolPtr V(tvk::create_volume(raw.data(), false, dt, e.dims, bs, ov, clamp ? 1 : 0, median,
                                  !lod0_only));
      bool lod0 = true;
      for (uint64_t k = 0; k < V->n_bricks && lod0; ++k) lod0 = same_as_file(V.get(), k);
      if (!lod0) break;  // LOD 0 does not depend on the filter
      std::vector<uint64_t> bad;
      for (uint64_t k = V->n_bricks; k < V->total_bricks; ++k)
        if (!same_as_file(V.get(), k)) bad.push_back(k);
      if (bad.empty()) {
        *out = V.release();
        return;
      }
      if (!best || bad.size() < best_bad.size()) {
        best = std::move(V);
        best_bad = std::move(bad);
      }
    }
    if (!best) continue;
    // keep the file's coarser bricks that no filter reproduced, with their
    // statistics (min/max over the whole brick, ComputeBrickStats) and macro cells
    tvk_volume* V = best.get();
    for (uint64_t k : best_bad) {
      const size_t nb = brick_bytes(V, k);
      tvk::eo_read_brick(e, k, nb, brick);
      TVK_CUDA(cudaMemcpy(static_cast<uint8_t*>(V->d_pool) + V->offsets[k] * vb, brick.data(), nb,
                          cudaMemcpyHostToDevice));
      if (dt == TVK_RGBA8) continue;  // colour bricks carry no statistics
      double lo = 1e300, hi = -1e300;
      for (size_t i = 0; i < nb / vb; ++i) {
        const double x = vb == 1 ? double(brick[i])
                                 : double(reinterpret_cast<const uint16_t*>(brick.data())[i]);
        lo = std::min(lo, x);
        hi = std::max(hi, x);
      }
      V->bmin[k] = lo;
      V->bmax[k] = hi;
    }
    if (dt == TVK_RGBA8) {  // no macro cells to refresh
      *out = best.release();
      return;
    }
    tvk::DevBuf d_off, d_sizes;
    d_off.ensure(V->total_bricks * sizeof(uint64_t));
    d_sizes.ensure(V->total_bricks * 3 * sizeof(uint32_t));
    TVK_CUDA(cudaMemcpy(d_off.p, V->offsets.data(), V->total_bricks * sizeof(uint64_t),
                        cudaMemcpyHostToDevice));
    TVK_CUDA(cudaMemcpy(d_sizes.p, V->sizes.data(), V->total_bricks * 3 * sizeof(uint32_t),
                        cudaMemcpyHostToDevice));
    uint32_t max_rows = 0;
    for (uint32_t d : V->cell_dims)
      max_rows = std::max(max_rows, (d >> 10) & 1023u);
    uint64_t launches = 0;
    tvk::launch_cell_minmax(V->d_pool, V->bytes, d_off.as<uint64_t>(), d_sizes.as<uint32_t>(),
                            static_cast<const uint64_t*>(V->d_cell_meta), V->total_bricks,
                            max_rows, static_cast<uint32_t*>(V->d_cells), nullptr, &launches);
    TVK_CUDA(cudaDeviceSynchronize());
    *out = best.release();
    return;
  }
  tvk::fail(TVK_ERR_INVALID_ARG,
            "ExtendedOctree: the file's LOD-0 bricks differ from a rebricking of their own "
            "inner voxels with zero or clamped borders");
}

}  // namespace

tvk_status tvk_volume_open_extended_octree(const char* path, uint64_t offset,
                                           uint32_t uvf_version, uint32_t flags,
                                           tvk_volume** out) {
  return guarded([&] { open_eo_volume(path, offset, uvf_version, flags, out); });
}

tvk_status tvk_uvf_read_blocks(const char* path, uint32_t flags, tvk_uvf_info* info,
                               tvk_uvf_block* blocks, uint32_t capacity) {
  return guarded([&] {
    REQUIRE(path && info, "null argument");
    REQUIRE(blocks || capacity == 0, "null block array with a non-zero capacity");
    REQUIRE((flags & ~uint32_t(TVK_UVF_VERIFY_CHECKSUM)) == 0, "unknown flag");
    tvk::UvfFile u;
    tvk::uvf_open(path, (flags & TVK_UVF_VERIFY_CHECKSUM) != 0, u);
    *info = tvk_uvf_info{};
    info->file_version = u.version;
    info->checksum_semantics = u.checksum_semantics;
    info->checksum_bytes = u.checksum_bytes;
    info->data_offset = u.data_offset;
    info->file_bytes = u.file_bytes;
    info->big_endian = u.big_endian ? 1 : 0;
    info->block_count = uint32_t(u.blocks.size());
    info->timestep_count = uint32_t(u.timesteps.size());
    info->checksum_verified = u.checksum_verified ? 1 : 0;
    for (size_t i = 0; i < u.blocks.size() && i < capacity; ++i) blocks[i] = u.blocks[i];
  });
}

tvk_status tvk_volume_open_uvf(const char* path, uint32_t timestep, uint32_t flags,
                               tvk_volume** out) {
  return guarded([&] {
    REQUIRE(path && out, "null argument");
    *out = nullptr;
    tvk::UvfFile u;
    tvk::uvf_open(path, (flags & TVK_UVF_VERIFY_CHECKSUM) != 0, u);
    if (u.timesteps.empty()) {
      if (u.has_raster)
        tvk::fail(TVK_ERR_UNSUPPORTED,
                  "UVF: volumes stored as RasterDataBlocks (files without TOC blocks) are not read");
      tvk::fail(TVK_ERR_INVALID_ARG,
                "UVF: no TOC block of a 1- or 4-component volume in the file");
    }
    REQUIRE(timestep < u.timesteps.size(), "timestep out of range");
    if (u.version > 0xffffffffull) tvk::fail(TVK_ERR_INVALID_ARG, "UVF: file version out of range");
    const tvk_uvf_block& b = u.blocks[u.timesteps[timestep]];
    open_eo_volume(path, b.offset + b.header_bytes, uint32_t(u.version),
                   flags & ~uint32_t(TVK_UVF_VERIFY_CHECKSUM), out);
  });
}

tvk_status tvk_volume_destroy(tvk_volume* v) {
  return guarded([&] {
    if (!v) return;
    tvk::free_volume_device(v);
    delete v;
  });
}

tvk_status tvk_volume_get_info(const tvk_volume* v, tvk_volume_info* out) {
  return guarded([&] {
    REQUIRE(v && out, "null argument");
    std::memset(out, 0, sizeof(*out));
    for (int a = 0; a < 3; ++a) {
      out->dims[a] = v->dims[a];
      out->brick_size[a] = v->brick_size[a];
    }
    out->dtype = v->dtype;
    out->bit_width = v->dtype == TVK_RGBA8 ? 8u : 8u * v->bytes;  // per channel
    out->overlap = v->overlap;
    out->lod_count = uint32_t(v->lods.size());
    out->lod0_bricks = v->n_bricks;
    out->range_min = v->range_min;
    out->range_max = v->range_max;
    out->max_gradient = double(float(v->max_grad));
    out->device_bytes = v->pool_bytes;
  });
}

tvk_status tvk_volume_get_lod(const tvk_volume* v, uint32_t lod, uint64_t size[3],
                              uint64_t brick_count[3]) {
  return guarded([&] {
    REQUIRE(v && size && brick_count, "null argument");
    REQUIRE(lod < v->lods.size(), "LOD out of range");
    for (int a = 0; a < 3; ++a) {
      size[a] = v->lods[lod].size[a];
      brick_count[a] = v->lods[lod].bricks[a];
    }
  });
}

tvk_status tvk_volume_get_brick_md(const tvk_volume* v, uint64_t ts, uint64_t lod, uint64_t index,
                                   tvk_brick_md* out) {
  return guarded([&] {
    REQUIRE(out, "null argument");
    *out = v->md[tvk::key_check(v, ts, lod, index)];
  });
}

tvk_status tvk_volume_get_brick(const tvk_volume* v, uint64_t ts, uint64_t lod, uint64_t index,
                                void* host_out, size_t bytes) {
  return guarded([&] {
    const uint64_t k = tvk::key_check(v, ts, lod, index);
    REQUIRE(host_out, "null argument");
    const size_t n = size_t(v->sizes[3 * k]) * v->sizes[3 * k + 1] * v->sizes[3 * k + 2] * v->bytes;
    REQUIRE(bytes >= n, "output buffer smaller than the brick");
    TVK_CUDA(cudaSetDevice(v->device));
    TVK_CUDA(cudaMemcpy(host_out,
                        static_cast<const uint8_t*>(tvk::device_bricks(v)) + v->offsets[k] * v->bytes,
                        n, cudaMemcpyDeviceToHost));
  });
}

tvk_status tvk_volume_release_bricks(tvk_volume* v) {
  return guarded([&] {
    REQUIRE(v, "null argument");
    TVK_CUDA(cudaSetDevice(v->device));
    TVK_CUDA(cudaDeviceSynchronize());  // no launch may still read the pool
    if (v->d_pool) TVK_CUDA(cudaFree(v->d_pool));
    v->d_pool = nullptr;
    tvk::free_brick_textures(v);  // the bricks' texture copies go with them
  });
}

tvk_status tvk_volume_get_minmax(const tvk_volume* v, uint64_t ts, uint64_t lod, uint64_t index,
                                 tvk_minmax* out) {
  return guarded([&] {
    const uint64_t k = tvk::key_check(v, ts, lod, index);
    REQUIRE(out, "null argument");
    // MaxMinDataBlock::SetDataFromFlatVector (IO/UVF/MaxMinDataBlock.cpp:175-195)
    out->min_scalar = v->bmin[k];
    out->max_scalar = v->bmax[k];
    out->min_gradient = -std::numeric_limits<double>::max();
    out->max_gradient = std::numeric_limits<double>::max();
  });
}

tvk_status tvk_volume_get_histogram(const tvk_volume* v, uint64_t* host_out, size_t bins,
                                    uint64_t* trimmed_len) {
  return guarded([&] {
    REQUIRE(v && host_out, "null argument");
    tvk::require_scalar(v, "histograms");
    std::memset(host_out, 0, bins * sizeof(uint64_t));
    const size_t n = std::min(bins, v->hist.size());
    for (size_t i = 0; i < n; ++i) host_out[i] = v->hist[i];
    if (trimmed_len) *trimmed_len = v->hist_trimmed;
  });
}

tvk_status tvk_volume_get_histogram2d(const tvk_volume* v, uint64_t* host_out, size_t value_bins,
                                      size_t entries, uint64_t* value_bins_used,
                                      float* max_gradient) {
  return guarded([&] {
    REQUIRE(v && host_out, "null argument");
    tvk::require_scalar(v, "histograms");
    if (v->rebricked)
      tvk::fail(TVK_ERR_UNSUPPORTED,
                "a rebricked volume forwards its histograms to the source volume; query that");
    const uint64_t bins = value_bins ? value_bins : v->hist_trimmed;
    REQUIRE(bins >= 1 && bins <= 65536, "value_bins must be 1 .. 65536");
    REQUIRE(entries >= bins * 256, "output holds fewer than value_bins * 256 entries");
    if (v->overlap == 0)
      tvk::fail(TVK_ERR_UNSUPPORTED, "central differences need an overlap of at least 1");
    TVK_CUDA(cudaSetDevice(v->device));
    tvk::compute_histogram2d(v, bins, host_out);
    if (value_bins_used) *value_bins_used = bins;
    // Histogram2DDataBlock::m_fMaxGradMagnitude is a float
    if (max_gradient) *max_gradient = float(v->max_grad);
  });
}

tvk_status tvk_volume_get_brick_histograms(const tvk_volume* v, uint32_t* host_out,
                                           size_t n_bricks, uint32_t* shift) {
  return guarded([&] {
    REQUIRE(v && host_out, "null argument");
    tvk::require_scalar(v, "histograms");
    if (v->rebricked)
      tvk::fail(TVK_ERR_UNSUPPORTED, "per-brick histograms exist for bricked source volumes only");
    REQUIRE(n_bricks >= v->n_bricks, "output holds fewer bricks than the volume");
    std::memcpy(host_out, v->bhist.data(), v->bhist.size() * sizeof(uint32_t));
    if (shift) *shift = v->hist_shift;
  });
}

tvk_status tvk_volume_rebrick(const tvk_volume* src, const uint32_t brick_size[3], int minmax_mode,
                              tvk_volume** out) {
  return guarded([&] {
    REQUIRE(src && brick_size && out, "null argument");
    *out = nullptr;
    tvk::require_scalar(src, "rebricking");
    *out = tvk::rebrick_volume(src, brick_size, minmax_mode);
  });
}

tvk_status tvk_volume_get_max_used_brick_size(const tvk_volume* v, uint32_t out[3]) {
  return guarded([&] {
    REQUIRE(v && out, "null argument");
    // BrickedDataset::GetMaxUsedBrickSizes (IO/BrickedDataset.cpp:139-145)
    out[0] = out[1] = out[2] = 0;
    for (uint64_t k = 0; k < v->total_bricks; ++k)
      for (int a = 0; a < 3; ++a) out[a] = std::max(out[a], v->md[k].n_voxels[a]);
  });
}

tvk_status tvk_volume_index_from_4d(const tvk_volume* v, const uint64_t xyzl[4], uint64_t* index) {
  return guarded([&] {
    REQUIRE(v && xyzl && index, "null argument");
    REQUIRE(xyzl[3] < v->lods.size(), "LOD out of range");
    const tvk::LodInfo& l = v->lods[xyzl[3]];
    REQUIRE(xyzl[0] < l.bricks[0] && xyzl[1] < l.bricks[1] && xyzl[2] < l.bricks[2],
            "brick coordinate out of range");
    *index = xyzl[0] + xyzl[1] * l.bricks[0] + xyzl[2] * l.bricks[0] * l.bricks[1];
  });
}

tvk_status tvk_volume_index_to_4d(const tvk_volume* v, uint64_t lod, uint64_t index,
                                  uint64_t xyzl[4]) {
  return guarded([&] {
    REQUIRE(v && xyzl, "null argument");
    REQUIRE(lod < v->lods.size(), "LOD out of range");
    const tvk::LodInfo& l = v->lods[lod];
    REQUIRE(index < l.bricks[0] * l.bricks[1] * l.bricks[2], "brick index out of range");
    xyzl[0] = index % l.bricks[0];
    xyzl[1] = (index / l.bricks[0]) % l.bricks[1];
    xyzl[2] = index / (l.bricks[0] * l.bricks[1]);
    xyzl[3] = lod;
  });
}

tvk_status tvk_renderer_create(tvk_renderer** out) {
  return guarded([&] {
    REQUIRE(out, "null output handle");
    std::unique_ptr<tvk_renderer> R(new tvk_renderer());
    TVK_CUDA(cudaGetDevice(&R->device));
    TVK_CUDA(cudaStreamCreateWithFlags(&R->stream, cudaStreamNonBlocking));
    TVK_CUDA(cudaEventCreate(&R->ev_start));
    TVK_CUDA(cudaEventCreate(&R->ev_stop));
    TVK_CUDA(cudaEventCreateWithFlags(&R->ev_staged, cudaEventDisableTiming));
    TVK_CUDA(cudaEventCreateWithFlags(&R->ev_ready, cudaEventDisableTiming));
    TVK_CUDA(cudaEventRecord(R->ev_staged, R->stream));
    *out = R.release();
  });
}

tvk_status tvk_renderer_destroy(tvk_renderer* r) {
  return guarded([&] {
    if (!r) return;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->copy_stream) {
      cudaStreamSynchronize(r->copy_stream);
      cudaStreamDestroy(r->copy_stream);
    }
    if (r->ev_img_ready) cudaEventDestroy(r->ev_img_ready);
    if (r->ev_img_copied) cudaEventDestroy(r->ev_img_copied);
    if (r->ev_start) cudaEventDestroy(r->ev_start);
    if (r->ev_stop) cudaEventDestroy(r->ev_stop);
    if (r->ev_staged) cudaEventDestroy(r->ev_staged);
    if (r->ev_ready) cudaEventDestroy(r->ev_ready);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
  });
}

tvk_status tvk_renderer_set_volume(tvk_renderer* r, const tvk_volume* v) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    if (v && v->rebricked)
      tvk::fail(TVK_ERR_UNSUPPORTED, "rendering runs on bricked source volumes, not rebricked ones");
    r->vol = v;
    for (auto& sl : r->slots) sl.empty_valid = false;
    r->frame_started = false;
    // AbstrRenderer.cpp:247: m_iMaxLODIndex = GetLargestSingleBrickLOD(0)
    r->max_lod_index = 0;
    if (v) {
      for (size_t l = 0; l < v->lods.size(); ++l)
        if (v->lods[l].bricks[0] * v->lods[l].bricks[1] * v->lods[l].bricks[2] == 1) {
          r->max_lod_index = l;
          break;
        }
    }
    // AbstrRenderer.cpp:252-261: the isovalue starts at half the data range,
    // the ClearView isovalue half as much again above it
    if (v) {
      r->isovalue = float(v->range_max - v->range_min) / 2.0f;
      r->cv_iso = r->isovalue + (r->isovalue / 2.0f);
    }
  });
}

tvk_status tvk_set_tf1d_rgba8(tvk_renderer* r, const uint8_t* rgba, uint32_t n) {
  return guarded([&] {
    REQUIRE(r && rgba && n >= 2, "need a renderer and at least two TF entries");
    // TransferFunction1D::Set (TransferFunction1D.cpp:146-177); a constant
    // channel divides by zero, and the NaN it yields becomes 0 in the RGBA8
    // upload below, as in the reference
    std::vector<float> f(size_t(4) * n);
    tvk::tf1d_from_bytes(rgba, n, f.data());
    tvk::set_tf(r, f.data(), n, 1, true);
  });
}

tvk_status tvk_set_tf1d_float(tvk_renderer* r, const float* rgba, uint32_t n, int rgba8_upload) {
  return guarded([&] {
    REQUIRE(r && rgba && n >= 2, "need a renderer and at least two TF entries");
    tvk::set_tf(r, rgba, n, 1, rgba8_upload != 0);
  });
}

tvk_status tvk_set_tf2d_float(tvk_renderer* r, const float* rgba, uint32_t w, uint32_t h,
                              int rgba8_upload) {
  return guarded([&] {
    REQUIRE(r && rgba && w >= 2 && h >= 2, "need a renderer and a TF of at least 2x2");
    tvk::set_tf(r, rgba, w, h, rgba8_upload != 0);
  });
}

tvk_status tvk_set_render_mode(tvk_renderer* r, tvk_render_mode mode) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(mode == TVK_RM_1DTRANS || mode == TVK_RM_2DTRANS || mode == TVK_RM_ISOSURFACE,
            "unknown render mode");
    r->mode = mode;
  });
}

tvk_status tvk_set_lighting(tvk_renderer* r, int enable) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->lighting = enable != 0;
  });
}

tvk_status tvk_set_sample_rate_modifier(tvk_renderer* r, float srm) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(srm > 0.0f && srm < 1e4f, "sample rate modifier must be in (0, 1e4)");
    r->srm = srm;
  });
}

tvk_status tvk_set_isovalue(tvk_renderer* r, float isovalue) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->isovalue = isovalue;
  });
}

tvk_status tvk_set_iso_color(tvk_renderer* r, const float rgb[3]) {
  return guarded([&] {
    REQUIRE(r && rgb, "null argument");
    for (int a = 0; a < 3; ++a) r->iso_color[a] = rgb[a];
  });
}

tvk_status tvk_set_colors(tvk_renderer* r, const float ambient[4], const float diffuse[4],
                          const float specular[4], const float light_dir[3]) {
  return guarded([&] {
    REQUIRE(r && ambient && diffuse && specular && light_dir, "null argument");
    for (int a = 0; a < 4; ++a) {
      r->ambient[a] = ambient[a];
      r->diffuse[a] = diffuse[a];
      r->specular[a] = specular[a];
    }
    for (int a = 0; a < 3; ++a) r->light_dir[a] = light_dir[a];
  });
}

tvk_status tvk_set_scaling_method(tvk_renderer* r, tvk_scaling_method method) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    REQUIRE(method == TVK_SCALE_BIT_WIDTH || method == TVK_SCALE_BIAS_AND_SCALE,
            "unknown scaling method");
    r->tf_scaling = method;
  });
}

tvk_status tvk_set_light_model(tvk_renderer* r, tvk_light_model model, float ka, float kd,
                               float ks, float shininess) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(model == TVK_LIGHT_REFERENCE || model == TVK_LIGHT_BLINN_PHONG, "unknown model");
    REQUIRE(shininess >= 0.0f, "shininess must be >= 0");
    r->light_model = model;
    r->bp[0] = ka;
    r->bp[1] = kd;
    r->bp[2] = ks;
    r->bp[3] = shininess;
  });
}

tvk_status tvk_set_view(tvk_renderer* r, const float eye[3], const float at[3], const float up[3],
                        float fovy_deg, float znear, float zfar) {
  return guarded([&] {
    REQUIRE(r && eye && at && up, "null argument");
    REQUIRE(fovy_deg > 0.0f && fovy_deg < 180.0f, "field of view must be in (0, 180)");
    REQUIRE(znear > 0.0f && zfar > znear, "need 0 < znear < zfar");
    for (int a = 0; a < 3; ++a) {
      r->eye[a] = eye[a];
      r->at[a] = at[a];
      r->up[a] = up[a];
    }
    r->fovy = fovy_deg;
    r->znear = znear;
    r->zfar = zfar;
  });
}

tvk_status tvk_set_model_transform(tvk_renderer* r, const float rotation[16],
                                   const float translation[16]) {
  return guarded([&] {
    REQUIRE(r && rotation && translation, "null argument");
    // row-vector matrices (Basics/Vectors.h): p' = p * Rot * Trans; as a
    // column-vector affine map: M[row][col] = Trans^T * Rot^T
    double Rm[3][4], Tm[3][4];
    for (int row = 0; row < 3; ++row)
      for (int col = 0; col < 4; ++col) {
        Rm[row][col] = rotation[col * 4 + row];
        Tm[row][col] = translation[col * 4 + row];
      }
    for (int row = 0; row < 3; ++row)
      for (int col = 0; col < 4; ++col) {
        double acc = (col == 3) ? Tm[row][3] : 0.0;
        for (int k = 0; k < 3; ++k) acc += Tm[row][k] * Rm[k][col];
        r->model[row][col] = acc;
      }
    // rigidity check: the upper 3x3 must be orthonormal
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double d = 0;
        for (int k = 0; k < 3; ++k) d += r->model[k][i] * r->model[k][j];
        if (std::fabs(d - (i == j ? 1.0 : 0.0)) > 1e-4)
          tvk::fail(TVK_ERR_INVALID_ARG, "model transform must be rigid");
      }
  });
}

tvk_status tvk_resize(tvk_renderer* r, uint32_t width, uint32_t height) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(width >= 1 && height >= 1 && width <= 16384 && height <= 16384,
            "viewport must be 1..16384 pixels per side");
    r->width = width;
    r->height = height;
  });
}

tvk_status tvk_set_frame_termination(tvk_renderer* r, float threshold) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(threshold > 0.0f && threshold <= 1.0f, "threshold must be in (0, 1]");
    r->frame_ert = threshold;
  });
}

tvk_status tvk_paint(tvk_renderer* r) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    tvk::paint(r, tvk::Subframe{r->lod, r->dec_screen, r->dec_sampling});
  });
}

tvk_status tvk_set_lod(tvk_renderer* r, uint32_t lod) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->lod = lod;
  });
}

tvk_status tvk_set_reduced_quality(tvk_renderer* r, int decrease_screen_res,
                                   int decrease_sampling_rate) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->dec_screen = decrease_screen_res != 0;
    r->dec_sampling = decrease_sampling_rate != 0;
  });
}

tvk_status tvk_set_perf_measures(tvk_renderer* r, uint32_t min_framerate,
                                 int low_res_intermediate, float screen_res_dec_factor,
                                 float sample_dec_factor) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    REQUIRE(screen_res_dec_factor >= 1.0f && screen_res_dec_factor <= 64.0f,
            "screen resolution decrease factor must be in [1, 64]");
    REQUIRE(sample_dec_factor > 0.0f, "sample rate decrease factor must be > 0");
    // AbstrRenderer::SetPerfMeasures (AbstrRenderer.cpp:1435-1454)
    r->max_ms_per_frame = (min_framerate == 0) ? 10000.0f : 1000.0f / float(min_framerate);
    r->screen_dec = screen_res_dec_factor;
    r->sample_dec = sample_dec_factor;
    r->low_res_intermediate = low_res_intermediate != 0;
    if (!r->low_res_intermediate) {
      r->decrease_screen_res = r->decrease_screen_res_now = false;
      r->decrease_sampling_rate = r->decrease_sampling_rate_now = false;
      r->another_redraw_low_res = false;
    }
    r->frame_started = false;
  });
}

tvk_status tvk_set_lod_limits(tvk_renderer* r, uint32_t coarsest_skip, uint32_t finest) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->lod_limits[0] = coarsest_skip;
    r->lod_limits[1] = finest;
    r->frame_started = false;
  });
}

tvk_status tvk_set_capture_mode(tvk_renderer* r, int capture) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->capture = capture != 0;
    r->frame_started = false;
  });
}

tvk_status tvk_compute_min_lod(tvk_renderer* r, uint32_t* lod) {
  return guarded([&] {
    REQUIRE(r && lod, "null argument");
    if (!r->vol) tvk::fail(TVK_ERR_STATE, "no volume attached (tvk_renderer_set_volume)");
    if (r->width == 0 || r->height == 0) tvk::fail(TVK_ERR_STATE, "no viewport (tvk_resize)");
    *lod = uint32_t(tvk::min_lod_for_view(r, r->vol));
  });
}

tvk_status tvk_paint_progressive(tvk_renderer* r, int new_frame, tvk_subframe_info* info) {
  return guarded([&] {
    REQUIRE(r && info, "null argument");
    tvk::paint_progressive(r, new_frame != 0, info);
  });
}

tvk_status tvk_batch_create(tvk_batch** out) {
  return guarded([&] {
    REQUIRE(out, "null output handle");
    std::unique_ptr<tvk_batch> B(new tvk_batch());
    TVK_CUDA(cudaGetDevice(&B->device));
    TVK_CUDA(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    TVK_CUDA(cudaEventCreate(&B->ev_start));
    TVK_CUDA(cudaEventCreate(&B->ev_stop));
    TVK_CUDA(cudaEventCreateWithFlags(&B->ev_done, cudaEventDisableTiming));
    *out = B.release();
  });
}

tvk_status tvk_batch_destroy(tvk_batch* b) {
  return guarded([&] {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : {b->ev_start, b->ev_stop, b->ev_done})
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b->fork_join) cudaEventDestroy(e);
    for (cudaStream_t st : b->aux) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
  });
}

tvk_status tvk_batch_set_autotune(tvk_batch* b, int autotune, uint32_t ctas_per_sm) {
  return guarded([&] {
    REQUIRE(b, "null batch");
    b->autotune = autotune != 0;
    b->fixed_ctas_per_sm = ctas_per_sm;
    b->tuned.clear();
  });
}

tvk_status tvk_paint_batch(tvk_batch* b, tvk_renderer* const* renderers, uint32_t n) {
  return guarded([&] {
    REQUIRE(b && renderers && n >= 1, "need a batch and at least one renderer");
    tvk::paint_batch(b, renderers, n);
  });
}

tvk_status tvk_batch_set_rays_per_thread(tvk_batch* b, uint32_t rays_per_thread) {
  return guarded([&] {
    REQUIRE(b, "null argument");
    REQUIRE(rays_per_thread <= 2, "rays per thread must be 0 (tuned), 1 or 2");
    b->fixed_rays_per_thread = rays_per_thread;
  });
}

tvk_status tvk_batch_get_info(tvk_batch* b, tvk_batch_info* out) {
  return guarded([&] {
    REQUIRE(b && out, "null argument");
    if (b->info.frames == 0) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    TVK_CUDA(cudaEventSynchronize(b->ev_stop));
    TVK_CUDA(cudaEventElapsedTime(&b->info.ms, b->ev_start, b->ev_stop));
    *out = b->info;
  });
}

// ---- learned reconstruction

static cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

tvk_status tvk_learned_param_count(size_t* n) {
  return guarded([&] {
    REQUIRE(n, "null argument");
    *n = tvk::unet_param_count();
  });
}

tvk_status tvk_learned_create(const float* host_params, size_t n, tvk_learned** out) {
  return guarded([&] {
    REQUIRE(host_params && out, "null argument");
    REQUIRE(n == tvk::unet_param_count(), "parameter count does not match the network");
    std::unique_ptr<tvk_learned> N(new tvk_learned());
    TVK_CUDA(cudaGetDevice(&N->device));
    size_t nw = 0, nb = 0;
    for (int i = 0; i < tvk::kUNetLayers; ++i) {
      const tvk::UNetLayer& L = tvk::kUNet[i];
      N->w_off[i] = nw;
      N->b_off[i] = nb;
      nw += size_t(9) * L.cout * (L.c1 + L.c2);
      nb += L.cout;
    }
    // host layout: per layer the FP32 weights [9][cout][cin] then the bias
    std::vector<float> w(nw), b(nb);
    size_t src = 0;
    for (int i = 0; i < tvk::kUNetLayers; ++i) {
      const tvk::UNetLayer& L = tvk::kUNet[i];
      const size_t lw = size_t(9) * L.cout * (L.c1 + L.c2);
      std::copy(host_params + src, host_params + src + lw, w.begin() + N->w_off[i]);
      src += lw;
      std::copy(host_params + src, host_params + src + L.cout, b.begin() + N->b_off[i]);
      src += L.cout;
    }
    tvk::DevBuf d_w32;
    d_w32.ensure(nw * sizeof(float));
    N->d_w.ensure(nw * 2);
    N->d_b.ensure(nb * sizeof(float));
    TVK_CUDA(cudaMemcpy(d_w32.p, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
    TVK_CUDA(cudaMemcpy(N->d_b.p, b.data(), nb * sizeof(float), cudaMemcpyHostToDevice));
    tvk::cnn_to_bf16(d_w32.as<float>(), nw, N->d_w.p, nullptr);
    TVK_CUDA(cudaDeviceSynchronize());
    for (cudaEvent_t& e : N->ev) TVK_CUDA(cudaEventCreate(&e));
    TVK_CUDA(cudaStreamCreateWithFlags(&N->probe_stream, cudaStreamNonBlocking));
    TVK_CUDA(cudaEventCreateWithFlags(&N->ev_pstaged, cudaEventDisableTiming));
    TVK_CUDA(cudaEventRecord(N->ev_pstaged, N->probe_stream));
    TVK_CUDA(cudaEventCreateWithFlags(&N->ev_planned, cudaEventDisableTiming));
    TVK_CUDA(cudaEventCreate(&N->ev_pstart));
    TVK_CUDA(cudaEventCreate(&N->ev_pdone));
    *out = N.release();
  });
}

tvk_status tvk_learned_destroy(tvk_learned* n) {
  return guarded([&] {
    if (!n) return;
    if (n->probe_stream) cudaStreamSynchronize(n->probe_stream);
    for (cudaEvent_t e : n->ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {n->ev_pstaged, n->ev_planned, n->ev_pstart, n->ev_pdone})
      if (e) cudaEventDestroy(e);
    if (n->probe_stream) cudaStreamDestroy(n->probe_stream);
    delete n;
  });
}

tvk_status tvk_paint_learned(tvk_renderer* r, tvk_learned* net, float threshold_db,
                             tvk_learned_info* info) {
  return guarded([&] {
    REQUIRE(r && net && info, "null argument");
    tvk::paint_learned(r, net, threshold_db, info);
  });
}

tvk_status tvk_cnn_prepare_input(const float* image_rgba, const float* depth, int h, int w, int hp,
                                 int wp, void* out, void* stream) {
  return guarded([&] {
    REQUIRE(image_rgba && out && hp >= h && wp >= w, "null argument or padding too small");
    tvk::cnn_prepare_input(image_rgba, depth, h, w, hp, wp, out, as_stream(stream));
  });
}

tvk_status tvk_set_clip_plane(tvk_renderer* r, const float plane[4]) {
  return guarded([&] {
    REQUIRE(r && plane, "null argument");
    REQUIRE(std::isfinite(plane[0]) && std::isfinite(plane[1]) && std::isfinite(plane[2]) &&
                std::isfinite(plane[3]),
            "clip plane must be finite");
    REQUIRE(plane[0] != 0.0f || plane[1] != 0.0f || plane[2] != 0.0f,
            "clip plane normal must not be zero");
    for (int a = 0; a < 4; ++a) r->clip_plane[a] = plane[a];
  });
}

tvk_status tvk_enable_clip_plane(tvk_renderer* r, int on) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    r->clip_on = on != 0;
  });
}

tvk_status tvk_set_clearview(tvk_renderer* r, int on) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    r->cv_on = on != 0;
  });
}

tvk_status tvk_set_cv_isovalue(tvk_renderer* r, float isovalue) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    REQUIRE(std::isfinite(isovalue), "isovalue must be finite");
    r->cv_iso = isovalue;
  });
}

tvk_status tvk_set_cv_color(tvk_renderer* r, const float rgb[3]) {
  return guarded([&] {
    REQUIRE(r && rgb, "null argument");
    for (int a = 0; a < 3; ++a) r->cv_color[a] = rgb[a];
  });
}

tvk_status tvk_set_cv_params(tvk_renderer* r, float size, float context_scale,
                             float border_scale) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    REQUIRE(std::isfinite(size) && std::isfinite(context_scale) && std::isfinite(border_scale),
            "ClearView parameters must be finite");
    r->cv_size = size;
    r->cv_context_scale = context_scale;
    r->cv_border_scale = border_scale;
  });
}

tvk_status tvk_set_cv_focus_pos(tvk_renderer* r, const float pos[4]) {
  return guarded([&] {
    REQUIRE(r && pos, "null argument");
    for (int a = 0; a < 4; ++a) r->cv_pos[a] = pos[a];
  });
}

tvk_status tvk_get_cv_focus_pos(const tvk_renderer* r, float pos[4]) {
  return guarded([&] {
    REQUIRE(r && pos, "null argument");
    for (int a = 0; a < 4; ++a) pos[a] = r->cv_pos[a];
  });
}

// GLRenderer::CVFocusHasChanged (GLRenderer.cpp:2833-2854): the context hit
// of the last ClearView frame at pixel (x, y) (row 0 at the bottom), moved to
// model space; a pixel without a hit moves the focus far away (w = 0).
tvk_status tvk_set_cv_focus_pixel(tvk_renderer* r, uint32_t x, uint32_t y) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    if (!r->cv_painted) tvk::fail(TVK_ERR_STATE, "no ClearView frame painted yet");
    TVK_CUDA(cudaSetDevice(r->device));
    float hit[4] = {0, 0, 0, 0};
    if (x < r->render_w && y < r->render_h) {
      TVK_CUDA(cudaStreamSynchronize(r->stream));
      const size_t pix = size_t(y) * r->render_w + x;
      TVK_CUDA(cudaMemcpy(hit, r->d_cvhits.as<float4>() + 4 * pix, sizeof(hit),
                          cudaMemcpyDeviceToHost));
    }
    if (hit[3] != 0.0f) {
      for (int a = 0; a < 3; ++a) {
        double m = r->cv_last_inv[a][3];
        for (int j = 0; j < 3; ++j) m += r->cv_last_inv[a][j] * double(hit[j]);
        r->cv_pos[a] = float(m);
      }
      r->cv_pos[3] = 1.0f;
    } else {
      r->cv_pos[0] = r->cv_pos[1] = r->cv_pos[2] = 10000000.0f;
      r->cv_pos[3] = 0.0f;
    }
  });
}

tvk_status tvk_set_depth_output(tvk_renderer* r, int on) {
  return guarded([&] {
    REQUIRE(r, "null argument");
    r->depth_out = on != 0;
  });
}

tvk_status tvk_copy_depth_device(tvk_renderer* r, void* dst, size_t bytes) {
  return guarded([&] {
    REQUIRE(r && dst, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    if (!r->depth_out || !r->d_depth.p) tvk::fail(TVK_ERR_STATE, "depth output is off");
    const size_t n = size_t(r->render_w) * r->render_h * sizeof(float);
    REQUIRE(bytes >= n, "destination smaller than the depth image");
    TVK_CUDA(cudaMemcpyAsync(dst, r->d_depth.p, n, cudaMemcpyDeviceToDevice, r->stream));
  });
}

tvk_status tvk_copy_image_device(tvk_renderer* r, int reduced, void* dst, size_t bytes) {
  return guarded([&] {
    REQUIRE(r && dst, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    const size_t n = reduced ? size_t(r->render_w) * r->render_h * 16
                             : size_t(r->width) * r->height * 16;
    REQUIRE(bytes >= n, "destination smaller than the image");
    const void* src = (reduced && (r->render_w != r->width || r->render_h != r->height))
                          ? r->d_lowimg.p : r->d_img.p;
    TVK_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, r->stream));
  });
}

// ---- learned reconstruction primitives

tvk_status tvk_cnn_conv3x3(const tvk_cnn_conv* a, void* stream) {
  return guarded([&] {
    REQUIRE(a && a->x1 && a->weights, "null argument");
    REQUIRE(a->c2 == 0 || a->x2, "second input missing");
    REQUIRE((a->c1 + a->c2) % 16 == 0 && a->c1 % 2 == 0 && a->c1 + a->c2 <= 128,
            "input channels must be a multiple of 16, at most 128");
    REQUIRE(a->cout % 8 == 0 && a->cout >= 8 && a->cout <= 128, "cout must be 8 .. 128");
    REQUIRE(a->n >= 1 && a->h >= 1 && a->w >= 1, "empty tensor");
    REQUIRE(a->y_bf16 || a->y_f32, "no output");
    REQUIRE(!a->y2_f32 || (a->split > 0 && a->split < a->cout && a->y_f32), "bad split");
    REQUIRE(!a->upsample1 || (a->h1 >= 1 && a->w1 >= 1 && a->h1 >= a->h / 2 &&
                              a->w1 >= a->w / 2 && a->h1 <= (a->h + 1) / 2 &&
                              a->w1 <= (a->w + 1) / 2),
            "an upsampled input must be half the output size");
    tvk::cnn_conv3x3(*a, as_stream(stream));
  });
}

tvk_status tvk_cnn_check(void* stream) {
  return guarded([&] {
    TVK_CUDA(cudaStreamSynchronize(as_stream(stream)));
    if (tvk::cnn_tc_timeouts(true))
      tvk::fail(TVK_ERR_INTERNAL,
                "a tensor-core convolution gave up waiting for its MMAs; its output is undefined");
  });
}

tvk_status tvk_cnn_conv3x3_wgrad(const tvk_cnn_wgrad* a, void* stream) {
  return guarded([&] {
    REQUIRE(a && a->x1 && a->gy && a->dw, "null argument");
    REQUIRE(a->c2 == 0 || a->x2, "second input missing");
    REQUIRE((a->c1 + a->c2) % 16 == 0 && a->c1 + a->c2 <= 128,
            "input channels must be a multiple of 16, at most 128");
    REQUIRE(a->cout % 8 == 0 && a->cout >= 8 && a->cout <= 64, "cout must be 8 .. 64");
    tvk::cnn_conv3x3_wgrad(*a, as_stream(stream));
  });
}

tvk_status tvk_cnn_act_grad(const float* dy, const void* y, float slope, void* g, size_t n,
                            void* stream) {
  return guarded([&] {
    REQUIRE(dy && g, "null argument");
    tvk::cnn_act_grad(dy, y, slope, g, n, as_stream(stream));
  });
}

tvk_status tvk_cnn_avgpool2(const void* x, int n, int h, int w, int c, void* y, void* stream) {
  return guarded([&] {
    REQUIRE(x && y && h % 2 == 0 && w % 2 == 0, "even sizes and buffers needed");
    tvk::cnn_avgpool2(x, n, h, w, c, y, as_stream(stream));
  });
}

tvk_status tvk_cnn_avgpool2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                                     int accumulate, void* stream) {
  return guarded([&] {
    REQUIRE(dy && dx && h % 2 == 0 && w % 2 == 0, "even sizes and buffers needed");
    tvk::cnn_avgpool2_backward(dy, n, h, w, c, dx, accumulate, as_stream(stream));
  });
}

tvk_status tvk_cnn_upsample2(const void* x, int n, int h, int w, int c, void* y, void* stream) {
  return guarded([&] {
    REQUIRE(x && y, "null argument");
    tvk::cnn_upsample2(x, n, h, w, c, y, as_stream(stream));
  });
}

tvk_status tvk_cnn_upsample2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                                      void* stream) {
  return guarded([&] {
    REQUIRE(dy && dx, "null argument");
    tvk::cnn_upsample2_backward(dy, n, h, w, c, dx, as_stream(stream));
  });
}

tvk_status tvk_cnn_head(const float* head, const float* base, int n, int h, int w, float* out,
                        void* stream) {
  return guarded([&] {
    REQUIRE(head && base && out, "null argument");
    tvk::cnn_head(head, base, n, h, w, 2 * h, 2 * w, out, as_stream(stream));
  });
}

tvk_status tvk_cnn_head_backward(const float* dout, int n, int h, int w, float* dhead,
                                 void* stream) {
  return guarded([&] {
    REQUIRE(dout && dhead, "null argument");
    tvk::cnn_head_backward(dout, n, h, w, dhead, as_stream(stream));
  });
}

tvk_status tvk_cnn_mse(const float* out, const float* target, size_t n, float* dout, float* loss,
                       void* stream) {
  return guarded([&] {
    REQUIRE(out && target && loss && n > 0, "null argument");
    tvk::cnn_mse(out, target, n, dout, loss, as_stream(stream));
  });
}

tvk_status tvk_cnn_adam(float* w, const float* g, float* m, float* v, size_t n, float lr,
                        float b1, float b2, float eps, int step, void* stream) {
  return guarded([&] {
    REQUIRE(w && g && m && v && step >= 1, "null argument or step < 1");
    tvk::cnn_adam(w, g, m, v, n, lr, b1, b2, eps, step, as_stream(stream));
  });
}

tvk_status tvk_cnn_weights_bf16(const float* w, int cout, int cin, void* fwd, void* bwd,
                                void* stream) {
  return guarded([&] {
    REQUIRE(w && fwd, "null argument");
    tvk::cnn_weights_bf16(w, cout, cin, fwd, bwd, as_stream(stream));
  });
}

tvk_status tvk_cnn_to_bf16(const float* x, size_t n, void* y, void* stream) {
  return guarded([&] {
    REQUIRE(x && y, "null argument");
    tvk::cnn_to_bf16(x, n, y, as_stream(stream));
  });
}

// ---- GridLeaper brick cache

tvk_status tvk_pool_create(const tvk_volume* v, uint64_t budget_bytes, int host_source,
                           tvk_pool** out) {
  return guarded([&] {
    REQUIRE(v && out, "null argument");
    if (v->rebricked) tvk::fail(TVK_ERR_UNSUPPORTED, "pools are built over bricked volumes");
    const size_t n_lods = v->lod_first.size() - 1;
    if (n_lods != v->lods.size())
      tvk::fail(TVK_ERR_UNSUPPORTED, "the GridLeaper needs every LOD (volume built with LODs)");
    REQUIRE(n_lods <= tvk::kLeaperMaxLods, "too many LODs");
    for (int a = 0; a < 3; ++a)
      REQUIRE(v->brick_size[a] <= 1023, "pool bricks are at most 1023 voxels per axis");
    std::unique_ptr<tvk_pool> P(new tvk_pool());
    P->vol = v;
    P->device = v->device;
    TVK_CUDA(cudaSetDevice(v->device));
    for (uint64_t k = 0; k < v->total_bricks; ++k)
      P->slot_voxels = std::max<uint64_t>(P->slot_voxels, uint64_t(v->sizes[3 * k]) *
                                                              v->sizes[3 * k + 1] * v->sizes[3 * k + 2]);
    const uint64_t slot_bytes = P->slot_voxels * v->bytes;
    P->n_slots = uint32_t(std::min<uint64_t>(v->total_bricks, budget_bytes / slot_bytes));
    REQUIRE(P->n_slots >= 2, "the budget holds fewer than two bricks");
    P->d_slots.ensure(size_t(P->n_slots) * slot_bytes);
    P->host_source = host_source != 0;
    tvk::device_bricks(v);  // the bricks are copied or paged from the device pool
    if (P->host_source) {
      P->h_bricks.ensure(v->pool_bytes);
      TVK_CUDA(cudaMemcpy(P->h_bricks.p, tvk::device_bricks(v), v->pool_bytes,
                          cudaMemcpyDeviceToHost));
    }
    P->page.assign(v->total_bricks, tvk::kBiMissing);
    P->h_page.ensure(v->total_bricks * sizeof(uint32_t));
    P->d_page.ensure(v->total_bricks * sizeof(uint32_t));
    std::vector<uint32_t> dims(v->total_bricks);
    for (uint64_t k = 0; k < v->total_bricks; ++k)
      dims[k] = v->sizes[3 * k] | (v->sizes[3 * k + 1] << 10) | (v->sizes[3 * k + 2] << 20);
    P->d_dims.ensure(v->total_bricks * sizeof(uint32_t));
    TVK_CUDA(cudaMemcpy(P->d_dims.p, dims.data(), dims.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice));
    P->hash_size = tvk::reference_hash_size(v);
    P->d_hash.ensure(P->hash_size * sizeof(uint32_t));
    P->h_hash.ensure(P->hash_size * sizeof(uint32_t));
    TVK_CUDA(cudaStreamCreateWithFlags(&P->page_stream, cudaStreamNonBlocking));
    TVK_CUDA(cudaEventCreateWithFlags(&P->ev_paged, cudaEventDisableTiming));
    TVK_CUDA(cudaEventCreate(&P->ev_pass[0]));
    TVK_CUDA(cudaEventCreate(&P->ev_pass[1]));
    P->slots.assign(P->n_slots, tvk_pool::Slot{});
    // the single brick of the coarsest LOD stays in the last slot
    P->coarsest = uint32_t(v->total_bricks - 1);
    tvk::pool_upload(P.get(), P->n_slots - 1, P->coarsest, ~uint64_t(0));
    tvk::pool_upload_page_table(P.get());
    TVK_CUDA(cudaStreamSynchronize(P->page_stream));
    *out = P.release();
  });
}

tvk_status tvk_pool_destroy(tvk_pool* p) {
  return guarded([&] {
    if (!p) return;
    if (p->page_stream) cudaStreamSynchronize(p->page_stream);
    if (p->ev_paged) cudaEventDestroy(p->ev_paged);
    for (cudaEvent_t e : p->ev_pass)
      if (e) cudaEventDestroy(e);
    if (p->page_stream) cudaStreamDestroy(p->page_stream);
    delete p;
  });
}

tvk_status tvk_pool_get_page_table(const tvk_pool* p, uint32_t* out, size_t n) {
  return guarded([&] {
    REQUIRE(p && out, "null argument");
    REQUIRE(n >= p->page.size(), "output smaller than the page table");
    std::memcpy(out, p->page.data(), p->page.size() * sizeof(uint32_t));
  });
}

tvk_status tvk_pool_get_requests(const tvk_pool* p, uint64_t* out, size_t n, size_t* count) {
  return guarded([&] {
    REQUIRE(p && count, "null argument");
    REQUIRE(out || n == 0, "null output");
    const size_t k = std::min(n, p->requests.size());
    std::copy(p->requests.begin(), p->requests.begin() + k, out);
    *count = p->requests.size();
  });
}

tvk_status tvk_pool_reset(tvk_pool* p) {
  return guarded([&] {
    REQUIRE(p, "null argument");
    TVK_CUDA(cudaSetDevice(p->device));
    TVK_CUDA(cudaStreamSynchronize(p->page_stream));
    // GLVolumePool::PH_Reset (GLVolumePool.cpp:261-282): every slot but the
    // one holding the coarsest brick is emptied, every entry but that brick's
    // becomes MISSING, and visibility is recomputed before the next pass
    const uint32_t keep = p->page[p->coarsest];
    for (tvk_pool::Slot& sl : p->slots)
      if (sl.brick != int64_t(p->coarsest)) sl = tvk_pool::Slot{};
    std::fill(p->page.begin(), p->page.end(), tvk::kBiMissing);
    p->page[p->coarsest] = keep;
    p->vis_valid = false;
    tvk::pool_upload_page_table(p);
    TVK_CUDA(cudaStreamSynchronize(p->page_stream));
  });
}

tvk_status tvk_pool_set_request_table(tvk_pool* p, uint32_t size, uint32_t rehash) {
  return guarded([&] {
    REQUIRE(p, "null argument");
    REQUIRE(size <= (1u << 24), "request table above 2^24 entries");
    REQUIRE(rehash >= 1 || size == 0, "rehash must be at least 1");
    TVK_CUDA(cudaSetDevice(p->device));
    TVK_CUDA(cudaStreamSynchronize(p->page_stream));
    const uint32_t n = size ? size : tvk::reference_hash_size(p->vol);
    p->d_hash.ensure(size_t(n) * sizeof(uint32_t));
    p->h_hash.ensure(size_t(n) * sizeof(uint32_t));
    p->hash_size = n;
    p->rehash = size ? rehash : 10u;
  });
}

tvk_status tvk_pool_get_info(const tvk_pool* p, tvk_pool_info* out) {
  return guarded([&] {
    REQUIRE(p && out, "null argument");
    out->slots = p->n_slots;
    out->slot_bytes = p->slot_voxels * p->vol->bytes;
    out->bricks = p->vol->total_bricks;
    out->hash_size = p->hash_size;
    out->host_source = p->host_source ? 1 : 0;
    out->paged_total = p->paged_total;
  });
}

tvk_status tvk_leaper_paint(tvk_renderer* r, tvk_pool* pool, uint32_t max_passes,
                            tvk_leaper_info* info) {
  return guarded([&] {
    REQUIRE(r && pool && info, "null argument");
    tvk::leaper_paint(r, pool, max_passes, info);
  });
}

tvk_status tvk_get_render_size(tvk_renderer* r, uint32_t* width, uint32_t* height) {
  return guarded([&] {
    REQUIRE(r && width && height, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    *width = r->render_w;
    *height = r->render_h;
  });
}

tvk_status tvk_get_image_device(tvk_renderer* r, const float** device_rgba, uint32_t* width,
                                uint32_t* height) {
  return guarded([&] {
    REQUIRE(r && device_rgba, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    *device_rgba = r->d_img.as<const float>();
    if (width) *width = r->width;
    if (height) *height = r->height;
  });
}

tvk_status tvk_read_image(tvk_renderer* r, float* host_rgba, size_t n_floats) {
  return guarded([&] {
    REQUIRE(r && host_rgba, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    const size_t n = size_t(r->width) * r->height * 4;
    REQUIRE(n_floats >= n, "output buffer smaller than the image");
    TVK_CUDA(cudaMemcpyAsync(host_rgba, r->d_img.p, n * sizeof(float), cudaMemcpyDeviceToHost,
                             r->stream));
    TVK_CUDA(cudaStreamSynchronize(r->stream));
  });
}

tvk_status tvk_read_image_async(tvk_renderer* r, float* host_rgba, size_t n_floats) {
  return guarded([&] {
    REQUIRE(r && host_rgba, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    const size_t n = size_t(r->width) * r->height * 4;
    REQUIRE(n_floats >= n, "output buffer smaller than the image");
    TVK_CUDA(cudaSetDevice(r->device));
    if (!r->copy_stream) {
      TVK_CUDA(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
      TVK_CUDA(cudaEventCreateWithFlags(&r->ev_img_ready, cudaEventDisableTiming));
      TVK_CUDA(cudaEventCreateWithFlags(&r->ev_img_copied, cudaEventDisableTiming));
    }
    // the previous readback may still read d_img_ro
    if (r->img_pending) TVK_CUDA(cudaStreamWaitEvent(r->stream, r->ev_img_copied, 0));
    r->d_img_ro.ensure(n * sizeof(float));
    TVK_CUDA(cudaMemcpyAsync(r->d_img_ro.p, r->d_img.p, n * sizeof(float),
                             cudaMemcpyDeviceToDevice, r->stream));
    TVK_CUDA(cudaEventRecord(r->ev_img_ready, r->stream));
    TVK_CUDA(cudaStreamWaitEvent(r->copy_stream, r->ev_img_ready, 0));
    TVK_CUDA(cudaMemcpyAsync(host_rgba, r->d_img_ro.p, n * sizeof(float),
                             cudaMemcpyDeviceToHost, r->copy_stream));
    TVK_CUDA(cudaEventRecord(r->ev_img_copied, r->copy_stream));
    r->img_pending = true;
  });
}

tvk_status tvk_wait_image(tvk_renderer* r) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    if (r->img_pending) TVK_CUDA(cudaEventSynchronize(r->ev_img_copied));
    r->img_pending = false;
  });
}

tvk_status tvk_read_sample_counts(tvk_renderer* r, uint32_t* host_counts, size_t n) {
  return guarded([&] {
    REQUIRE(r && host_counts, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    // counts of the ray-marched image (render size; smaller than the viewport
    // while the screen resolution is decreased)
    const size_t np = size_t(r->render_w) * r->render_h;
    REQUIRE(n >= np, "output buffer smaller than the image");
    TVK_CUDA(cudaMemcpyAsync(host_counts, r->d_spp.p, np * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, r->stream));
    TVK_CUDA(cudaStreamSynchronize(r->stream));
  });
}

tvk_status tvk_renderer_get_stream(tvk_renderer* r, void** stream) {
  return guarded([&] {
    REQUIRE(r && stream, "null argument");
    *stream = r->stream;
  });
}

tvk_status tvk_get_stats(tvk_renderer* r, tvk_stats* out) {
  return guarded([&] {
    REQUIRE(r && out, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    TVK_CUDA(cudaStreamSynchronize(r->stream));
    const unsigned long long* c = r->h_counters.as<unsigned long long>();
    r->stats.samples = c[0];
    r->stats.shaded_samples = c[1];
    r->stats.gradient_samples = c[3];
    float ms = 0;
    TVK_CUDA(cudaEventElapsedTime(&ms, r->ev_start, r->ev_stop));
    r->stats.last_paint_ms = ms;
    if (c[2] != 0)
      tvk::fail(TVK_ERR_INTERNAL, "ray march guard tripped on " + std::to_string(c[2]) + " rays");
    *out = r->stats;
  });
}

tvk_status tvk_set_hardware_filtering(tvk_renderer* r, int on) {
  return guarded([&] {
    REQUIRE(r, "null renderer");
    r->hw_filter = on != 0;
  });
}

tvk_status tvk_volume_cell_minmax(const tvk_volume* v, uint64_t index, uint32_t* out,
                                  uint64_t capacity, uint32_t dims[3]) {
  return guarded([&] {
    REQUIRE(v && dims, "null argument");
    if (v->dtype == TVK_RGBA8) tvk::fail(TVK_ERR_UNSUPPORTED, "colour volumes have no macro cells");
    REQUIRE(index < v->total_bricks && index < v->cell_dims.size(), "brick index out of range");
    const uint32_t d = v->cell_dims[index];
    dims[0] = d & 1023u;
    dims[1] = (d >> 10) & 1023u;
    dims[2] = d >> 20;
    if (!out) return;
    const uint64_t n = v->cell_counts[index];
    REQUIRE(capacity >= n, "capacity below the brick's cell count");
    TVK_CUDA(cudaSetDevice(v->device));
    TVK_CUDA(cudaMemcpy(out, static_cast<const uint32_t*>(v->d_cells) + v->cell_offsets[index],
                        n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  });
}

tvk_status tvk_get_counters(tvk_renderer* r, uint64_t out[8]) {
  return guarded([&] {
    REQUIRE(r && out, "null argument");
    if (!r->painted) tvk::fail(TVK_ERR_STATE, "nothing painted yet");
    TVK_CUDA(cudaStreamSynchronize(r->stream));
    if (r->h_counters.bytes < 8 * sizeof(unsigned long long)) {
      for (int i = 0; i < 8; ++i) out[i] = 0;
      const unsigned long long* c = r->h_counters.as<unsigned long long>();
      for (int i = 0; i < 4 && r->h_counters.bytes >= (i + 1) * sizeof(*c); ++i) out[i] = c[i];
      return;
    }
    const unsigned long long* c = r->h_counters.as<unsigned long long>();
    for (int i = 0; i < 8; ++i) out[i] = c[i];
  });
}

tvk_status tvk_generate_volume(void* device_out, tvk_dtype dtype, const uint64_t dims[3],
                               const float* host_blobs, uint32_t n_blobs, float noise_amp,
                               uint32_t noise_octaves, float noise_cell, uint64_t seed,
                               int int_noise, float vmax) {
  return guarded([&] {
    REQUIRE(device_out && dims, "null argument");
    REQUIRE(n_blobs == 0 || host_blobs, "null blob table");
    REQUIRE(dtype == TVK_U8 || dtype == TVK_U16, "bad dtype");
    REQUIRE(noise_octaves == 0 || noise_cell > 0, "noise cell must be > 0");
    REQUIRE(dims[0] >= 1 && dims[1] >= 1 && dims[2] >= 1, "volume dimensions must be >= 1");
    tvk::launch_generate(device_out, dtype == TVK_U8 ? 1 : 2, dims, host_blobs, n_blobs,
                         noise_amp, noise_octaves, noise_cell, seed, int_noise, vmax, 0);
    TVK_CUDA(cudaDeviceSynchronize());
  });
}

}  // extern "C"
