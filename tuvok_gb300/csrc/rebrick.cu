// rebrick.cu -- DynamicBrickingDS on the GPU: re-cut a bricked volume into
// smaller bricks that divide the source bricks (IO/DynamicBrickingDS.cpp).
//
// The reference builds the brick table up front (Rebrick, :1090-1180) and then,
// per GetBrick call, reads the whole source brick (through a cache) and copies a
// window of it (Brick/CopyBrick, :495-538, :566-620).  Here the table is planned
// on the host with the reference's arithmetic and every target brick of every
// LOD is gathered from the source pool in a single launch, which also reduces the
// brick's min/max (minmax_brick, IO/BMinMax.cpp:8-47) for MM_PRECOMPUTE and
// MM_DYNAMIC.  The copy is HBM-bound: rows are contiguous along x on both sides.
//
// Reference arithmetic kept as is:
//   * integer_multiple (:963-971): the source's inner brick size must be i times
//     the target's (i < 128), else the reference throws;
//   * the loop over target bricks uses the real ghost width
//     (dbinfo::BrickSansGhost :218-223), while ComputedTargetBrickSize (:414-434),
//     SourceBrickIndex (:272-303), OffsetIntoSource (:305-335) and BrickMetadata
//     (:1034-1088) use the static BrickSansGhost (:208-217) that subtracts 4;
//   * layout() divides in float (:113-121); the world-space lerps follow
//     MathTools::lerp (Basics/MathTools.h:79-92);
//   * the copy indexes the source brick linearly, so a window row that runs past
//     the source's x extent continues on the next row.  A window that would read
//     past the end of the source brick (the reference reads outside its buffer)
//     is refused with TVK_ERR_UNSUPPORTED.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>

#include "tvk_internal.h"

namespace tvk {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kZChunk = 8;

struct RebrickEntry {
  uint64_t src_off, dst_off;  // voxels into the source / target pools
  uint32_t sx, sy;            // source brick row and slice widths
  uint32_t ox, oy, oz;        // window origin in the source brick
  uint32_t tx, ty, tz;        // target brick size (ghost included)
};

template <class T>
__global__ void __launch_bounds__(kThreads)
rebrick_kernel(const T* __restrict__ src, T* __restrict__ dst,
               const RebrickEntry* __restrict__ table, uint32_t* __restrict__ bmin,
               uint32_t* __restrict__ bmax) {
  const RebrickEntry e = table[blockIdx.x];
  const uint32_t z0 = blockIdx.y * kZChunk;
  uint32_t lo = 0xffffffffu, hi = 0;
  if (z0 < e.tz) {
    const uint32_t z1 = min(e.tz, z0 + kZChunk);
    const uint32_t row = e.tx, slice = e.tx * e.ty;
    const uint32_t n = (z1 - z0) * slice;
    const uint64_t sxy = uint64_t(e.sx) * e.sy;
    for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) {
      const uint32_t z = z0 + t / slice;
      const uint32_t r = t - (z - z0) * slice;
      const uint32_t y = r / row;
      const uint32_t x = r - y * row;
      const T v = src[e.src_off + uint64_t(e.oz + z) * sxy + uint64_t(e.oy + y) * e.sx + e.ox + x];
      dst[e.dst_off + uint64_t(z) * slice + r] = v;
      lo = min(lo, uint32_t(v));
      hi = max(hi, uint32_t(v));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0 && lo <= hi) {
    atomicMin(&bmin[blockIdx.x], lo);
    atomicMax(&bmax[blockIdx.x], hi);
  }
}

using U3 = std::array<uint64_t, 3>;

U3 layout_f(const U3& v, const U3& b) {
  U3 r;
  for (int a = 0; a < 3; ++a) r[a] = uint64_t(std::ceil(static_cast<float>(v[a]) / float(b[a])));
  return r;
}

U3 sans4(U3 b) {
  for (int a = 0; a < 3; ++a) b[a] = b[a] > 4 ? b[a] - 4 : b[a];
  return b;
}

template <class In>
float lerp_ref(In value, In imin, In imax, float omin, float omax) {
  return float(omin + (value - imin) * (static_cast<double>(omax - omin) / (imax - imin)));
}

struct DevMem {
  void* p = nullptr;
  ~DevMem() { if (p) cudaFree(p); }
};

}  // namespace

tvk_volume* rebrick_volume(const tvk_volume* S, const uint32_t Bt[3], int mm_mode) {
  if (S->rebricked) fail(TVK_ERR_UNSUPPORTED, "the source is itself a rebricked volume");
  if (mm_mode < 0 || mm_mode > 2) fail(TVK_ERR_INVALID_ARG, "unknown min/max mode");
  const uint64_t ghost = 2ull * S->overlap;
  const U3 B = {Bt[0], Bt[1], Bt[2]};
  // SourceMaxBrickSize: the converter's brick size minus the ghost width
  const U3 src_bs = {S->brick_size[0] - ghost, S->brick_size[1] - ghost,
                     S->brick_size[2] - ghost};
  static const char* kAxis[3] = {"x", "y", "z"};
  for (int a = 0; a < 3; ++a) {
    bool ok = B[a] > ghost;
    if (ok) {
      ok = false;
      for (uint64_t i = 0; i < 128 && !ok; ++i) ok = (B[a] - ghost) * i == src_bs[a];
    }
    if (!ok)
      fail(TVK_ERR_INVALID_ARG, std::string(kAxis[a]) +
                                    " dimension is not an integer multiple of original brick size.");
  }
  const size_t n_src_lods = S->lods.size();
  const size_t n_built = S->lod_first.size() - 1;

  // DatasetExtents (:993-1014): brick 0 of the first LOD that is a single brick
  size_t single = 0;
  for (size_t l = 0; l < n_src_lods; ++l) {
    const LodInfo& li = S->lods[l];
    if (li.bricks[0] * li.bricks[1] * li.bricks[2] == 1) {
      single = l;
      break;
    }
  }
  std::vector<tvk_brick_md> smd;
  brick_metadata(S->lods[single], S->brick_size, S->overlap, smd);
  float elow[3], ehigh[3];
  for (int a = 0; a < 3; ++a) {
    elow[a] = -(smd[0].extents[a] / 2.0f);
    ehigh[a] = smd[0].extents[a] / 2.0f;
  }

  std::unique_ptr<tvk_volume> V(new tvk_volume());
  V->device = S->device;
  V->dtype = S->dtype;
  V->bytes = S->bytes;
  for (int a = 0; a < 3; ++a) {
    V->dims[a] = S->dims[a];
    V->brick_size[a] = Bt[a];  // DynamicBrickingDS::GetMaxBrickSize
  }
  V->overlap = S->overlap;    // GetBrickOverlapSize forwards to the source
  V->clamp = S->clamp;
  V->median = S->median;
  V->build_lods = S->build_lods;
  V->rebricked = true;
  V->mm_mode = mm_mode;
  V->hist = S->hist;
  V->hist_shift = S->hist_shift;
  V->hist_trimmed = S->hist_trimmed;
  V->range_min = S->range_min;
  V->range_max = S->range_max;
  V->max_grad = S->max_grad;  // MaxGradientMagnitude forwards too

  const U3 real_sans = {B[0] - ghost, B[1] - ghost, B[2] - ghost};
  const U3 ssans = sans4(B);
  std::vector<RebrickEntry> table;
  V->lod_first.assign(1, 0);
  const uint64_t align = 256 / V->bytes;
  uint64_t dst = 0;
  for (size_t l = 0; l < n_src_lods; ++l) {
    const LodInfo& sl = S->lods[l];
    const U3 vox = {sl.size[0], sl.size[1], sl.size[2]};
    const U3 bl = layout_f(vox, real_sans);  // GenericBrickLayout
    LodInfo tl = sl;
    for (int a = 0; a < 3; ++a) tl.bricks[a] = bl[a];
    V->lods.push_back(tl);
    if (l >= n_built) continue;  // no source bricks to read at this LOD
    const U3 bls = layout_f(vox, ssans);
    const U3 src_lay = layout_f(vox, src_bs);
    const uint64_t nb = bl[0] * bl[1] * bl[2];
    for (uint64_t idx = 0; idx < nb; ++idx) {
      const U3 bi = {idx % bl[0], (idx / bl[0]) % bl[1], idx / (bl[0] * bl[1])};
      U3 cur;  // ComputedTargetBrickSize
      for (int a = 0; a < 3; ++a) {
        const uint64_t extra = vox[a] % ssans[a];
        cur[a] = (bi[a] == bls[a] - 1 && extra) ? 4 + extra : B[a];
      }
      // SourceBrickIndex / OffsetIntoSource / SourceKey
      if (idx >= bls[0] * bls[1] * bls[2])
        fail(TVK_ERR_UNSUPPORTED, "target brick index outside the reference's source layout");
      const U3 i3 = {idx % bls[0], (idx / bls[0]) % bls[1], idx / (bls[0] * bls[1])};
      uint64_t sidx[3], off[3];
      for (int a = 0; a < 3; ++a) {
        const uint64_t bps = src_bs[a] / ssans[a];
        if (bps == 0) fail(TVK_ERR_UNSUPPORTED, "target bricks larger than the source bricks");
        sidx[a] = i3[a] / bps;
        off[a] = (i3[a] % bps) * ssans[a];
        if (sidx[a] >= src_lay[a] || sidx[a] >= sl.bricks[a])
          fail(TVK_ERR_UNSUPPORTED, "target brick maps outside the source bricks");
      }
      const uint64_t sk = sidx[0] + sidx[1] * src_lay[0] + sidx[2] * src_lay[0] * src_lay[1];
      uint32_t sbs[3];
      brick_size(sl, S->brick_size, S->overlap, sidx, sbs);
      const uint64_t last = (off[2] + cur[2] - 1) * sbs[0] * sbs[1] +
                            (off[1] + cur[1] - 1) * sbs[0] + off[0] + cur[0] - 1;
      if (last >= uint64_t(sbs[0]) * sbs[1] * sbs[2])
        fail(TVK_ERR_UNSUPPORTED, "a target brick would read past the end of its source brick");

      // BrickMetadata with size = BrickSansGhost(cur), bsize = BrickSansGhost(B)
      tvk_brick_md m;
      const U3 size = sans4(cur);
      for (int a = 0; a < 3; ++a) {
        const uint64_t lo = bi[a] * ssans[a];
        const uint64_t hi = lo + size[a];
        const float vc = ((hi - lo) / 2.0f) + lo;
        m.center[a] = lerp_ref<float>(vc, 0.0f, static_cast<float>(vox[a]), elow[a], ehigh[a]);
        const float wl = lerp_ref<uint64_t>(lo, 0ull, vox[a], elow[a], ehigh[a]);
        const float wh = lerp_ref<uint64_t>(hi, 0ull, vox[a], elow[a], ehigh[a]);
        m.extents[a] = wh - wl;
        m.n_voxels[a] = uint32_t(cur[a]);
      }
      V->md.push_back(m);
      const uint64_t s_toc = S->lod_first[l] + sk;
      V->src_index.push_back(s_toc);
      for (int a = 0; a < 3; ++a) V->sizes.push_back(uint32_t(cur[a]));
      V->offsets.push_back(dst);
      RebrickEntry e;
      e.src_off = S->offsets[s_toc];
      e.dst_off = dst;
      e.sx = sbs[0];
      e.sy = sbs[1];
      e.ox = uint32_t(off[0]);
      e.oy = uint32_t(off[1]);
      e.oz = uint32_t(off[2]);
      e.tx = uint32_t(cur[0]);
      e.ty = uint32_t(cur[1]);
      e.tz = uint32_t(cur[2]);
      table.push_back(e);
      const uint64_t nv = cur[0] * cur[1] * cur[2];
      dst += (nv + align - 1) / align * align;
    }
    V->lod_first.push_back(V->md.size());
  }
  V->total_bricks = V->md.size();
  V->n_bricks = V->lod_first.size() > 1 ? V->lod_first[1] : 0;
  V->pool_bytes = dst * V->bytes;
  if (V->total_bricks == 0) fail(TVK_ERR_INTERNAL, "no target bricks");

  TVK_CUDA(cudaSetDevice(V->device));
  TVK_CUDA(cudaMalloc(&V->d_pool, V->pool_bytes));
  struct PoolGuard {
    tvk_volume* v;
    ~PoolGuard() {
      if (v && v->d_pool) cudaFree(v->d_pool);
    }
  } pg{V.get()};
  const uint64_t n = V->total_bricks;
  DevMem d_table, d_mm;
  TVK_CUDA(cudaMalloc(&d_table.p, n * sizeof(RebrickEntry)));
  TVK_CUDA(cudaMalloc(&d_mm.p, 2 * n * sizeof(uint32_t)));
  uint32_t* bmin = static_cast<uint32_t*>(d_mm.p);
  uint32_t* bmax = bmin + n;
  cudaStream_t s;
  TVK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  TVK_CUDA(cudaMemcpyAsync(d_table.p, table.data(), n * sizeof(RebrickEntry),
                           cudaMemcpyHostToDevice, s));
  TVK_CUDA(cudaMemsetAsync(bmin, 0xff, n * sizeof(uint32_t), s));
  TVK_CUDA(cudaMemsetAsync(bmax, 0, n * sizeof(uint32_t), s));
  uint32_t max_tz = 0;
  for (const RebrickEntry& e : table) max_tz = std::max(max_tz, e.tz);
  const dim3 grid(uint32_t(n), (max_tz + kZChunk - 1) / kZChunk);
  if (V->bytes == 1)
    rebrick_kernel<uint8_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint8_t*>(device_bricks(S)), static_cast<uint8_t*>(V->d_pool),
        static_cast<const RebrickEntry*>(d_table.p), bmin, bmax);
  else
    rebrick_kernel<uint16_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint16_t*>(device_bricks(S)), static_cast<uint16_t*>(V->d_pool),
        static_cast<const RebrickEntry*>(d_table.p), bmin, bmax);
  TVK_CUDA(cudaGetLastError());
  std::vector<uint32_t> mn(n), mx(n);
  TVK_CUDA(cudaMemcpyAsync(mn.data(), bmin, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaMemcpyAsync(mx.data(), bmax, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  TVK_CUDA(cudaStreamSynchronize(s));
  V->bmin.resize(n);
  V->bmax.resize(n);
  for (uint64_t t = 0; t < n; ++t) {
    if (mm_mode == 0) {  // MM_SOURCE: the source brick's statistics
      V->bmin[t] = S->bmin[V->src_index[t]];
      V->bmax[t] = S->bmax[V->src_index[t]];
    } else {             // MM_PRECOMPUTE / MM_DYNAMIC: minmax_brick of the copy
      V->bmin[t] = mn[t];
      V->bmax[t] = mx[t];
    }
  }
  pg.v = nullptr;
  return V.release();
}

}  // namespace tvk
