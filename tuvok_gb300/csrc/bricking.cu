// bricking.cu -- LOD-0 bricking, per-brick statistics and histograms on sm_103a.
//
// One pass over the flat volume writes every brick of LOD 0 (ghost voxels
// included) into the brick pool, and on the way accumulates
//   * per-brick min/max over the whole brick (ExtendedOctreeConverter::
//     ComputeBrickStats, IO/UVF/ExtendedOctree/ExtendedOctreeConverter.inc:408-444),
//   * the global histogram of inner voxels (Histogram1DDataBlock::ComputeTemplate,
//     IO/UVF/Histogram1DDataBlock.cpp:120-161),
//   * a 256-bin histogram of each brick's inner voxels.
// A second kernel finds the maximum gradient magnitude over inner voxels
// (Histogram2DDataBlock::ComputeGradient/ComputeTemplate, Histogram2DDataBlock.cpp:327-397);
// a third, run on request, fills the value x |gradient| histogram (:399-435).
//
// The voxel a brick position reads follows GetInputBrick
// (ExtendedOctreeConverter.cpp:288-373) exactly: the reference copies x-scanlines
// at linear file offsets, so a ghost read past the end of an x-line continues on
// the next line, and a read past the end of the file yields zero.  Clamping
// (ClampToEdge, :376-462) replicates the outermost inner plane on volume borders.
//
// All of this is integer work and HBM-bound: reads are contiguous along x, the
// pool is written in the same order, histograms live in shared memory and are
// merged with one atomic per non-zero bin and CTA.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "tvk_internal.h"

namespace tvk {
namespace {

constexpr int kThreads = 256;
// row segments of 32 voxels whose loads a warp of brick_copy_kernel issues together
constexpr uint32_t kUnroll = 4;
// global-histogram bins kept in a CTA's shared memory (16 KB: 12-bit data
// entirely; larger values go to the global bins directly)
constexpr uint32_t kSmemGlobalBins = 4096;

// Source voxel of brick-local position (i, j, k) of brick (cx, cy, cz).
template <class T>
__device__ __forceinline__ T source_voxel(const T* __restrict__ raw, const BrickGrid& g,
                                          const uint32_t c[3], const uint32_t bs[3],
                                          uint32_t i, uint32_t j, uint32_t k) {
  const uint32_t loc[3] = {i, j, k};
  uint64_t gc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    uint32_t l = loc[a];
    const bool first = c[a] == 0, last = c[a] == g.cnt[a] - 1;
    if (g.clamp) {
      if (first && l < g.ov) l = g.ov;
      if (last && l > bs[a] - 1 - g.ov) l = bs[a] - 1 - g.ov;
    }
    const uint32_t s = first ? g.ov : 0;
    const uint32_t e = bs[a] - (last ? g.ov : 0);
    if (l < s || l >= e) return T(0);
    gc[a] = uint64_t(c[a]) * (g.B[a] - 2u * g.ov) + l - g.ov;
  }
  const uint64_t L = gc[0] + gc[1] * g.dims[0] + gc[2] * g.dims[0] * g.dims[1];
  return L < g.total ? raw[L] : T(0);
}

// One histogram increment per lane with `in` set: a plain atomic per voxel.
// Keys below n_shared go to the CTA's shared bins, others to the global
// 64-bit bins.  Measured on the 1024^3 u16 volume's whole build (12.3 ms with
// warp merging, 11.2 ms without): merging a warp's increments when all its
// keys agree, merging every group of equal keys (__match_any_sync) or every
// run of equal keys in consecutive lanes all cost more than the same-address
// serialisation they save.
__device__ __forceinline__ void hist_add_warp(uint32_t* __restrict__ sh,
                                              unsigned long long* __restrict__ gl,
                                              uint32_t n_shared, bool in, uint32_t key,
                                              uint32_t lane) {
  (void)lane;
  if (!in) return;
  if (key < n_shared) atomicAdd(&sh[key], 1u);
  else atomicAdd(&gl[key], 1ull);
}

// Source line of brick-local row (j, k): GetInputBrick's y and z terms
// (ExtendedOctreeConverter.cpp:288-373, clamping :376-462), or a zero row.
__device__ __forceinline__ bool source_row(const BrickGrid& g, const uint32_t c[3],
                                           const uint32_t bs[3], uint32_t j, uint32_t k,
                                           uint64_t& rowbase) {
  const uint32_t loc[2] = {j, k};
  uint64_t gc[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int a = q + 1;
    uint32_t l = loc[q];
    const bool first = c[a] == 0, last = c[a] == g.cnt[a] - 1;
    if (g.clamp) {
      if (first && l < g.ov) l = g.ov;
      if (last && l > bs[a] - 1 - g.ov) l = bs[a] - 1 - g.ov;
    }
    const uint32_t s = first ? g.ov : 0;
    const uint32_t e = bs[a] - (last ? g.ov : 0);
    if (l < s || l >= e) return false;
    gc[q] = uint64_t(c[a]) * (g.B[a] - 2u * g.ov) + l - g.ov;
  }
  rowbase = gc[0] * g.dims[0] + gc[1] * g.dims[0] * g.dims[1];
  return true;
}

// LOD-0 bricking as a tile copy: one warp per brick row (x-scanline of the
// brick), the row's source line found once, lanes copying consecutive voxels
// (coalesced reads of the raw volume and writes of the pool).  On the way:
// per-brick min/max over every voxel written (ComputeBrickStats, ghost
// included) and the global histogram of inner voxels (Histogram1DDataBlock),
// which counts every voxel of the volume exactly once, so its first and last
// non-zero bins are the data range.  The per-brick 256-bin histograms need that
// range (their bin shift) and are taken by brick_sweep_kernel.  Persistent:
// each CTA takes (brick, z-chunk) items in turn and merges its shared
// histogram into the global one once, at the end.
template <class T>
__global__ void __launch_bounds__(kThreads, 5)
brick_copy_kernel(const T* __restrict__ raw, BrickGrid g, const uint64_t* __restrict__ offsets,
                  const uint32_t* __restrict__ sizes, T* __restrict__ pool, BrickScratch sc,
                  uint32_t smem_bins, uint32_t z_chunk, uint32_t chunks_per_brick,
                  uint32_t n_items) {
  extern __shared__ uint32_t gh[];  // global bins [0, smem_bins)
  for (uint32_t i = threadIdx.x; i < smem_bins; i += blockDim.x) gh[i] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (uint32_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const uint32_t b = item / chunks_per_brick;
    const uint32_t bs[3] = {sizes[3 * b + 0], sizes[3 * b + 1], sizes[3 * b + 2]};
    const uint32_t c[3] = {b % g.cnt[0], (b / g.cnt[0]) % g.cnt[1], b / (g.cnt[0] * g.cnt[1])};
    const uint32_t z0 = (item - b * chunks_per_brick) * z_chunk;
    const uint32_t z1 = min(bs[2], z0 + z_chunk);
    const uint32_t ov = g.ov;
    const bool fx = c[0] == 0, lx = c[0] == g.cnt[0] - 1;
    const uint32_t sx = fx ? ov : 0, ex = bs[0] - (lx ? ov : 0);
    const uint64_t xbase = uint64_t(c[0]) * (g.B[0] - 2u * ov);
    T* const brick = pool + offsets[b];
    uint32_t lo = 0xffffffffu, hi = 0;
    const uint32_t rows = z1 > z0 ? (z1 - z0) * bs[1] : 0;
    for (uint32_t r = warp; r < rows; r += nwarps) {
      const uint32_t k = z0 + r / bs[1];
      const uint32_t j = r - (k - z0) * bs[1];
      uint64_t rowbase = 0;
      const bool live = source_row(g, c, bs, j, k, rowbase);
      const bool inner_row = j >= ov && j < bs[1] - ov && k >= ov && k < bs[2] - ov;
      T* const out = brick + (uint64_t(k) * bs[1] + j) * bs[0];
      // an interior brick column reads its whole row from one source line
      // segment that ends inside the volume: no per-voxel clamping or limits
      const uint64_t src0 = xbase + rowbase - ov;
      const bool fast = live && !fx && !lx && src0 + bs[0] <= g.total;
      // kUnroll row segments of 32 voxels per pass: their loads are all in
      // flight before the first store
      for (uint32_t base = 0; base < bs[0]; base += 32 * kUnroll) {
        T v[kUnroll];
#pragma unroll
        for (uint32_t u = 0; u < kUnroll; ++u) {
          const uint32_t i = base + 32 * u + lane;
          v[u] = T(0);
          if (fast) {
            if (i < bs[0]) v[u] = __ldg(raw + src0 + i);
          } else if (i < bs[0] && live) {
            uint32_t l = i;
            if (g.clamp) {
              if (fx && l < ov) l = ov;
              if (lx && l > bs[0] - 1 - ov) l = bs[0] - 1 - ov;
            }
            if (l >= sx && l < ex) {
              const uint64_t L = (xbase + l - ov) + rowbase;
              if (L < g.total) v[u] = __ldg(raw + L);
            }
          }
        }
#pragma unroll
        for (uint32_t u = 0; u < kUnroll; ++u) {
          const uint32_t i = base + 32 * u + lane;
          if (base + 32 * u >= bs[0]) break;  // warp-uniform
          const bool act = i < bs[0];
          if (act) {
            out[i] = v[u];
            lo = min(lo, uint32_t(v[u]));
            hi = max(hi, uint32_t(v[u]));
          }
          hist_add_warp(gh, sc.hist, smem_bins,
                        act && inner_row && i >= ov && i < bs[0] - ov, uint32_t(v[u]), lane);
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0 && lo <= hi) {
      atomicMin(&sc.bmin[b], lo);
      atomicMax(&sc.bmax[b], hi);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < smem_bins; i += blockDim.x)
    if (gh[i]) atomicAdd(&sc.hist[i], (unsigned long long)gh[i]);
}

// Second pass over the LOD-0 bricks in the pool: each brick's 256-bin
// histogram of inner voxels (bin = value >> shift) and the largest squared
// central-difference sum Q = dx^2 + dy^2 + dz^2 over inner voxels
// (Histogram2DDataBlock::ComputeGradient, Histogram2DDataBlock.cpp:327-345, in
// integers).  One warp per inner row of a brick z-chunk, each lane loading its
// voxel's six neighbours (L1 serves the overlap).  (A z-walk that keeps the z
// neighbours in registers and takes x from the adjacent lanes loads half as
// much but measured slower: 3.5 against 3.1 ms on a 1024^3 u16 volume.)
template <class T>
__global__ void __launch_bounds__(kThreads)
brick_sweep_kernel(const T* __restrict__ pool, const uint64_t* __restrict__ offsets,
                   const uint32_t* __restrict__ sizes, uint32_t ov, uint32_t shift,
                   uint32_t z_chunk, uint32_t* __restrict__ bhist,
                   unsigned long long* __restrict__ brick_qmax) {
  __shared__ uint32_t bh[256];
  __shared__ unsigned long long qs[kThreads / 32];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) bh[i] = 0;
  __syncthreads();
  const uint32_t b = blockIdx.x;
  const uint32_t bs[3] = {sizes[3 * b + 0], sizes[3 * b + 1], sizes[3 * b + 2]};
  const T* const p = pool + offsets[b];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t iy = bs[1] > 2 * ov ? bs[1] - 2 * ov : 0;
  const uint32_t z0 = ov + blockIdx.y * z_chunk;
  const uint32_t z1 = bs[2] > ov ? min(bs[2] - ov, z0 + z_chunk) : 0;
  const uint32_t sx = bs[0], sxy = bs[0] * bs[1];
  const bool grad = ov > 0;  // central differences need a ghost layer on every side
  long long qmax = -1;
  const uint32_t rows = z1 > z0 ? (z1 - z0) * iy : 0;
  for (uint32_t r = warp; r < rows; r += nwarps) {
    const uint32_t k = z0 + r / iy;
    const uint32_t j = ov + (r - (k - z0) * iy);
    const T* const line = p + uint64_t(k) * sxy + uint64_t(j) * sx;
    for (uint32_t base = ov; base < bs[0] - ov; base += 32) {
      const uint32_t i = base + lane;
      const bool act = i < bs[0] - ov;
      uint32_t v = 0;
      if (act) {
        const T* const c = line + i;
        v = c[0];
        if (grad) {
          const int dx = int(c[-1]) - int(c[1]);
          const int dy = int(c[-int64_t(sx)]) - int(c[sx]);
          const int dz = int(c[-int64_t(sxy)]) - int(c[sxy]);
          const long long q =
              (long long)dx * dx + (long long)dy * dy + (long long)dz * dz;
          qmax = q > qmax ? q : qmax;
        }
      }
      hist_add_warp(bh, nullptr, 256u, act, min(v >> shift, 255u), lane);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const long long other = __shfl_xor_sync(0xffffffffu, qmax, o);
    qmax = other > qmax ? other : qmax;
  }
  if (lane == 0) qs[warp] = qmax < 0 ? 0ull : (unsigned long long)qmax + 1ull;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    for (uint32_t w = 0; w < nwarps; ++w) m = qs[w] > m ? qs[w] : m;
    if (m) atomicMax(&brick_qmax[b], m);  // Q + 1; 0 = no inner voxel
  }
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x)
    if (bh[i]) atomicAdd(&bhist[256u * b + i], bh[i]);
}

// The reference's double |gradient| (Histogram2DDataBlock.cpp:327-345)
// evaluated at the voxels whose integer Q equals the volume's largest Q, in
// the bricks listed: distinct Q values give |gradient| values whose gap far
// exceeds double rounding, so the maximum |gradient| is the largest of these.
template <class T>
__global__ void __launch_bounds__(kThreads)
max_gradient_at_kernel(const T* __restrict__ pool, const uint64_t* __restrict__ offsets,
                       const uint32_t* __restrict__ sizes, const uint32_t* __restrict__ bricks,
                       uint32_t ov, long long q_target, uint32_t z_chunk,
                       unsigned long long* out_bits) {
  const uint32_t b = bricks[blockIdx.x];
  const uint32_t bs[3] = {sizes[3 * b + 0], sizes[3 * b + 1], sizes[3 * b + 2]};
  const T* const p = pool + offsets[b];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t iy = bs[1] - 2 * ov;
  const uint32_t z0 = ov + blockIdx.y * z_chunk;
  const uint32_t z1 = min(bs[2] - ov, z0 + z_chunk);
  const uint32_t sx = bs[0], sxy = bs[0] * bs[1];
  const double nf2 = double(T(~T(0))) * 2.0;
  unsigned long long best = 0;
  const uint32_t rows = z1 > z0 ? (z1 - z0) * iy : 0;
  for (uint32_t r = warp; r < rows; r += nwarps) {
    const uint32_t k = z0 + r / iy;
    const uint32_t j = ov + (r - (k - z0) * iy);
    const T* const line = p + uint64_t(k) * sxy + uint64_t(j) * sx;
    for (uint32_t i = ov + lane; i < bs[0] - ov; i += 32) {
      const T* const c = line + i;
      const int dx = int(c[-1]) - int(c[1]);
      const int dy = int(c[-int64_t(sx)]) - int(c[sx]);
      const int dz = int(c[-int64_t(sxy)]) - int(c[sxy]);
      const long long q = (long long)dx * dx + (long long)dy * dy + (long long)dz * dz;
      if (q != q_target) continue;
      const double gx = __ddiv_rn(double(dx), nf2);
      const double gy = __ddiv_rn(double(dy), nf2);
      const double gz = __ddiv_rn(double(dz), nf2);
      const double f = __dsqrt_rn(
          __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz)));
      const unsigned long long bits = (unsigned long long)__double_as_longlong(f);
      best = bits > best ? bits : best;  // positive doubles order like their bits
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    best = ob > best ? ob : best;
  }
  if (lane == 0 && best) atomicMax(out_bits, best);
}

// Colour (RGBA8) volumes: the LOD-0 bricks with their ghost voxels (zero or
// clamp-to-edge), one 4-byte RGBA voxel per texel, no statistics.
__global__ void __launch_bounds__(kThreads)
brick_copy4_kernel(const uint32_t* __restrict__ raw, BrickGrid g,
                   const uint64_t* __restrict__ offsets, const uint32_t* __restrict__ sizes,
                   uint32_t* __restrict__ pool, uint32_t z_chunk) {
  const uint32_t b = blockIdx.x;
  const uint32_t bs[3] = {sizes[3 * b + 0], sizes[3 * b + 1], sizes[3 * b + 2]};
  const uint32_t c[3] = {b % g.cnt[0], (b / g.cnt[0]) % g.cnt[1], b / (g.cnt[0] * g.cnt[1])};
  const uint32_t z0 = blockIdx.y * z_chunk;
  const uint32_t z1 = min(bs[2], z0 + z_chunk);
  if (z0 >= z1) return;
  uint32_t* out = pool + offsets[b];
  const uint32_t sxy = bs[0] * bs[1];
  const uint32_t n = (z1 - z0) * sxy;
  for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) {
    const uint32_t k = z0 + t / sxy;
    const uint32_t r = t - (k - z0) * sxy;
    const uint32_t j = r / bs[0];
    const uint32_t i = r - j * bs[0];
    out[uint64_t(k) * sxy + r] = source_voxel<uint32_t>(raw, g, c, bs, i, j, k);
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
histogram2d_kernel(const T* __restrict__ pool, const uint64_t* __restrict__ offsets,
                   const uint32_t* __restrict__ sizes, Hist2DParams hp,
                   unsigned long long* __restrict__ hist) {
  // Value x |grad| counts over the inner voxels (Histogram2DDataBlock.cpp:399-435).
  // The gradient bin is floor(|g| / max|g| * 255) evaluated in double by the
  // reference.  Mathematically |g| / max|g| = sqrt(Q / Qmax) for the integer
  // squared difference sums Q, so a float estimate decides the bin unless it
  // lies within 1e-3 of a bin boundary (the estimate's error is below 1e-4);
  // only those voxels evaluate the reference's double expression.
  const uint32_t b = blockIdx.x;
  const uint32_t bs[3] = {sizes[3 * b + 0], sizes[3 * b + 1], sizes[3 * b + 2]};
  const T* p = pool + offsets[b];
  const uint32_t ix = bs[0] - 2 * hp.ov, iy = bs[1] - 2 * hp.ov;
  const uint32_t z0 = hp.ov + blockIdx.y * hp.z_chunk;
  const uint32_t z1 = min(bs[2] - hp.ov, z0 + hp.z_chunk);
  const uint32_t sx = bs[0], sxy = bs[0] * bs[1];
  const double nf2 = double(T(~T(0))) * 2.0;
  const uint32_t n = (z1 > z0) ? (z1 - z0) * ix * iy : 0;
  const uint32_t n_pad = (n + 31u) & ~31u;
  for (uint32_t t = threadIdx.x; t < n_pad; t += blockDim.x) {
    uint32_t key = 0xffffffffu;
    if (t < n) {
      const uint32_t k = z0 + t / (ix * iy);
      const uint32_t r = t % (ix * iy);
      const uint32_t j = hp.ov + r / ix;
      const uint32_t i = hp.ov + r % ix;
      const uint64_t c = uint64_t(i) + uint64_t(j) * sx + uint64_t(k) * sxy;
      const int dx = int(p[c - 1]) - int(p[c + 1]);
      const int dy = int(p[c - sx]) - int(p[c + sx]);
      const int dz = int(p[c - sxy]) - int(p[c + sxy]);
      const long long q = (long long)dx * dx + (long long)dy * dy + (long long)dz * dz;
      uint32_t g = 0;
      if (q > 0 && hp.qmax > 0) {
        const float est = sqrtf(float(q) * hp.inv_qmax) * 255.0f;
        const float fl = floorf(est);
        if (est - fl > 1e-3f && fl + 1.0f - est > 1e-3f) {
          g = min(255u, uint32_t(fl));
        } else {
          const double gx = __ddiv_rn(double(dx), nf2);
          const double gy = __ddiv_rn(double(dy), nf2);
          const double gz = __ddiv_rn(double(dz), nf2);
          const double len = __dsqrt_rn(
              __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz)));
          const double rel = __dmul_rn(__ddiv_rn(len, hp.gmax), 255.0);
          g = rel >= 255.0 ? 255u : uint32_t(rel);
        }
      }
      const uint32_t v = p[c];
      uint32_t vb = hp.scale_values
                        ? uint32_t(__ddiv_rn(__dmul_rn(double(v), double(hp.value_bins - 1)),
                                             hp.max_nonzero))
                        : v;
      vb = min(vb, hp.value_bins - 1);
      key = vb * 256u + g;
    }
    // one atomic per distinct bin in the warp
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && (threadIdx.x & 31u) == uint32_t(__ffs(peers) - 1))
      atomicAdd(&hist[key], (unsigned long long)__popc(peers));
  }
}

uint32_t blocks_for(uint64_t n) {
  const uint64_t b = (n + kThreads - 1) / kThreads;
  return uint32_t(b < 152ull * 16 ? (b ? b : 1) : 152ull * 16);
}

}  // namespace



void launch_brick_copy4(const void* raw, const BrickGrid& g, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, void* pool, cudaStream_t s,
                        uint64_t* launches) {
  const uint32_t z_chunk = 8;
  const dim3 grid(uint32_t(n_bricks), (g.B[2] + z_chunk - 1) / z_chunk);
  brick_copy4_kernel<<<grid, kThreads, 0, s>>>(static_cast<const uint32_t*>(raw), g, d_offsets,
                                               d_sizes, static_cast<uint32_t*>(pool), z_chunk);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}


void launch_histogram2d(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, uint32_t max_bz,
                        Hist2DParams hp, unsigned long long* hist, cudaStream_t s,
                        uint64_t* launches) {
  // central differences need a ghost layer on every side of the inner voxels
  if (hp.ov == 0 || max_bz <= 2 * hp.ov) return;
  hp.z_chunk = 4;
  const dim3 grid(uint32_t(n_bricks), (max_bz - 2 * hp.ov + hp.z_chunk - 1) / hp.z_chunk);
  if (bytes == 1)
    histogram2d_kernel<uint8_t><<<grid, kThreads, 0, s>>>(static_cast<const uint8_t*>(pool),
                                                          d_offsets, d_sizes, hp, hist);
  else
    histogram2d_kernel<uint16_t><<<grid, kThreads, 0, s>>>(static_cast<const uint16_t*>(pool),
                                                           d_offsets, d_sizes, hp, hist);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

namespace {

// Macro-cell min/max (cell c covers voxels c*kCell .. c*kCell + kCell on each
// axis, clamped to the brick).  One warp per cell row ry of a brick, walking
// the brick's z planes: per plane and voxel column the min/max over the
// kCell + 1 voxel rows the row spans (coalesced reads), folded into the
// running cell of the current z range; a cell is complete at its last plane,
// which also opens the next cell.  Each plane is read once per cell row.
// Lane l owns cells base + l + 32 t (t < kCellT): their kCell own columns,
// the shared column from the next cell's owner by a shuffle.
constexpr int kCellT = 3;

// Two consecutive voxels from a 2-voxel-aligned address, as one load.
__device__ __forceinline__ void load_pair(const uint8_t* p, uint32_t& a, uint32_t& b) {
  const uint32_t w = __ldg(reinterpret_cast<const unsigned short*>(p));
  a = w & 0xffu;
  b = w >> 8;
}
__device__ __forceinline__ void load_pair(const uint16_t* p, uint32_t& a, uint32_t& b) {
  const uint32_t w = __ldg(reinterpret_cast<const unsigned int*>(p));
  a = w & 0xffffu;
  b = w >> 16;
}

template <class T>
__global__ void __launch_bounds__(kThreads)
cell_minmax_kernel(const T* __restrict__ pool, const uint64_t* __restrict__ offsets,
                   const uint32_t* __restrict__ sizes, const uint64_t* __restrict__ cell_off,
                   uint32_t* __restrict__ cells) {
  const uint32_t b = blockIdx.y;
  const uint32_t n0 = sizes[3 * b], n1 = sizes[3 * b + 1], n2 = sizes[3 * b + 2];
  const uint32_t cx = cells_per_axis(n0), cy = cells_per_axis(n1);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ry = blockIdx.x * (kThreads / 32) + warp;  // cell row
  if (ry >= cy) return;  // whole warp
  const T* const p = pool + offsets[b];
  const uint32_t y0 = ry << kCellShift, y1 = min(y0 + kCell, n1 - 1);
  uint32_t* const out = cells + cell_off[b] + uint64_t(ry) * cx;
  const uint64_t cell_plane = uint64_t(cy) * cx;  // cells per z layer of cells
  const bool pairs = (n0 & 1u) == 0 && (offsets[b] & 1u) == 0;
  for (uint32_t cb = 0; cb < cx; cb += 32u * kCellT) {
    // accumulators of the open cell (per owned column, and lane 31's column
    // after its last cell)
    uint32_t lo[kCellT][kCell], hi[kCellT][kCell];
    uint32_t elo = 0xffffffffu, ehi = 0u;
#pragma unroll
    for (int t = 0; t < kCellT; ++t)
#pragma unroll
      for (int q = 0; q < kCell; ++q) { lo[t][q] = 0xffffffffu; hi[t][q] = 0u; }
    const uint32_t x_extra = (cb + 32u * kCellT) << kCellShift;
    // writes cell layer rz of this row from the open cell's accumulators
    auto emit = [&](uint32_t rz) {
#pragma unroll
      for (int t = 0; t < kCellT; ++t) {
        // the column shared with the next cell is its owner's first column:
        // the next lane's, for lane 31 lane 0's next cell (or its own extra)
        const int tn = t + 1 < kCellT ? t + 1 : t;
        uint32_t nlo = __shfl_down_sync(0xffffffffu, lo[t][0], 1);
        uint32_t nhi = __shfl_down_sync(0xffffffffu, hi[t][0], 1);
        const uint32_t wlo = __shfl_sync(0xffffffffu, lo[tn][0], 0);
        const uint32_t whi = __shfl_sync(0xffffffffu, hi[tn][0], 0);
        if (lane == 31) {
          nlo = t + 1 < kCellT ? wlo : elo;
          nhi = t + 1 < kCellT ? whi : ehi;
        }
        const uint32_t c = cb + lane + 32u * t;
        if (c < cx) {
          uint32_t a = nlo, h = nhi;
#pragma unroll
          for (int q = 0; q < kCell; ++q) { a = min(a, lo[t][q]); h = max(h, hi[t][q]); }
          out[uint64_t(rz) * cell_plane + c] = a | (h << 16);
        }
      }
    };
    // one plane's column min/max over rows y0..y1 (every row's loads issued
    // together)
    auto plane = [&](uint32_t z, uint32_t (&plo)[kCellT][kCell], uint32_t (&phi)[kCellT][kCell],
                     uint32_t& pelo, uint32_t& pehi) {
      pelo = 0xffffffffu;
      pehi = 0u;
#pragma unroll
      for (int t = 0; t < kCellT; ++t)
#pragma unroll
        for (int q = 0; q < kCell; ++q) { plo[t][q] = 0xffffffffu; phi[t][q] = 0u; }
#pragma unroll
      for (uint32_t r = 0; r <= uint32_t(kCell); ++r) {
        const uint32_t y = y0 + r;
        if (y > y1) break;  // warp-uniform
        const T* const line = p + (uint64_t(z) * n1 + y) * n0;
        if (kCell == 2 && pairs) {
          // both own columns in one aligned load (even row length: every row
          // and every even column start on a 2-voxel boundary)
#pragma unroll
          for (int t = 0; t < kCellT; ++t) {
            const uint32_t x = (cb + lane + 32u * t) << kCellShift;
            if (x < n0) {
              uint32_t v0, v1;
              load_pair(line + x, v0, v1);
              plo[t][0] = min(plo[t][0], v0);
              phi[t][0] = max(phi[t][0], v0);
              plo[t][1 % kCell] = min(plo[t][1 % kCell], v1);
              phi[t][1 % kCell] = max(phi[t][1 % kCell], v1);
            }
          }
        } else {
#pragma unroll
          for (int t = 0; t < kCellT; ++t)
#pragma unroll
            for (int q = 0; q < kCell; ++q) {
              const uint32_t x = ((cb + lane + 32u * t) << kCellShift) + q;
              if (x < n0) {
                const uint32_t v = __ldg(line + x);
                plo[t][q] = min(plo[t][q], v);
                phi[t][q] = max(phi[t][q], v);
              }
            }
        }
        if (lane == 31 && x_extra < n0) {
          const uint32_t v = __ldg(line + x_extra);
          pelo = min(pelo, v);
          pehi = max(pehi, v);
        }
      }
    };
    // folds plane z into the open cell; plane z closes cell layer z / kCell - 1
    // when it is a multiple of kCell (and then opens layer z / kCell with its
    // own values); the last plane closes the layer it lies in
    auto fold = [&](uint32_t z, const uint32_t (&plo)[kCellT][kCell],
                    const uint32_t (&phi)[kCellT][kCell], uint32_t pelo, uint32_t pehi) {
#pragma unroll
      for (int t = 0; t < kCellT; ++t)
#pragma unroll
        for (int q = 0; q < kCell; ++q) {
          lo[t][q] = min(lo[t][q], plo[t][q]);
          hi[t][q] = max(hi[t][q], phi[t][q]);
        }
      elo = min(elo, pelo);
      ehi = max(ehi, pehi);
      if (z > 0 && (z & (kCell - 1)) == 0) {
        emit((z >> kCellShift) - 1);
#pragma unroll
        for (int t = 0; t < kCellT; ++t)
#pragma unroll
          for (int q = 0; q < kCell; ++q) { lo[t][q] = plo[t][q]; hi[t][q] = phi[t][q]; }
        elo = pelo;
        ehi = pehi;
      }
      if (z == n2 - 1) emit(z >> kCellShift);
    };
    // (two planes per step, the second plane's loads in flight with the
    // first's, measured slower: 2.10 against 1.87 ms on the 1024^3 u16 volume)
    for (uint32_t z = 0; z < n2; ++z) {
      uint32_t plo[kCellT][kCell], phi[kCellT][kCell];
      uint32_t pelo, pehi;
      plane(z, plo, phi, pelo, pehi);
      fold(z, plo, phi, pelo, pehi);
    }
  }
}

}  // namespace

void launch_cell_minmax(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, const uint64_t* d_cell_offsets,
                        uint64_t n_bricks, uint32_t max_cell_rows, uint32_t* cells,
                        cudaStream_t s, uint64_t* launches) {
  const uint32_t per_cta = kThreads / 32;
  const dim3 grid((max_cell_rows + per_cta - 1) / per_cta, uint32_t(n_bricks));
  if (bytes == 1)
    cell_minmax_kernel<uint8_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint8_t*>(pool), d_offsets, d_sizes, d_cell_offsets, cells);
  else
    cell_minmax_kernel<uint16_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint16_t*>(pool), d_offsets, d_sizes, d_cell_offsets, cells);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_brick_copy(const void* raw, int bytes, const BrickGrid& g, const uint64_t* d_offsets,
                       const uint32_t* d_sizes, uint64_t n_bricks, void* pool,
                       const BrickScratch& sc, uint32_t global_bins, cudaStream_t s,
                       uint64_t* launches) {
  const uint32_t z_chunk = 4;
  const uint32_t chunks = (g.B[2] + z_chunk - 1) / z_chunk;
  const uint64_t items = n_bricks * chunks;
  if (items >= (1ull << 32)) fail(TVK_ERR_UNSUPPORTED, "too many bricks for one bricking pass");
  const uint32_t smem_bins = global_bins <= kSmemGlobalBins ? global_bins : kSmemGlobalBins;
  const size_t smem = size_t(smem_bins) * sizeof(uint32_t);
  // persistent: one wave of as many CTAs as fit on every SM at once (items
  // are dealt out round-robin, so a second partial wave would idle most SMs)
  int dev = 0, sms = 0, per_sm = 0;
  TVK_CUDA(cudaGetDevice(&dev));
  TVK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (bytes == 1)
    TVK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brick_copy_kernel<uint8_t>,
                                                           kThreads, smem));
  else
    TVK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brick_copy_kernel<uint16_t>,
                                                           kThreads, smem));
  const uint32_t grid =
      uint32_t(std::min<uint64_t>(items, uint64_t(std::max(1, sms)) * std::max(1, per_sm)));
  if (bytes == 1)
    brick_copy_kernel<uint8_t><<<grid, kThreads, smem, s>>>(
        static_cast<const uint8_t*>(raw), g, d_offsets, d_sizes, static_cast<uint8_t*>(pool), sc,
        smem_bins, z_chunk, chunks, uint32_t(items));
  else
    brick_copy_kernel<uint16_t><<<grid, kThreads, smem, s>>>(
        static_cast<const uint16_t*>(raw), g, d_offsets, d_sizes, static_cast<uint16_t*>(pool),
        sc, smem_bins, z_chunk, chunks, uint32_t(items));
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_brick_sweep(const void* pool, int bytes, const uint64_t* d_offsets,
                        const uint32_t* d_sizes, uint64_t n_bricks, uint32_t ov, uint32_t max_bz,
                        uint32_t shift, uint32_t* bhist, unsigned long long* brick_qmax,
                        cudaStream_t s, uint64_t* launches) {
  if (max_bz <= 2 * ov) return;  // no inner voxels
  const uint32_t z_chunk = 4;
  const dim3 grid(uint32_t(n_bricks), (max_bz - 2 * ov + z_chunk - 1) / z_chunk);
  if (bytes == 1)
    brick_sweep_kernel<uint8_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint8_t*>(pool), d_offsets, d_sizes, ov, shift, z_chunk, bhist,
        brick_qmax);
  else
    brick_sweep_kernel<uint16_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint16_t*>(pool), d_offsets, d_sizes, ov, shift, z_chunk, bhist,
        brick_qmax);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_max_gradient_at(const void* pool, int bytes, const uint64_t* d_offsets,
                            const uint32_t* d_sizes, const uint32_t* d_bricks, uint32_t n_list,
                            uint32_t ov, uint32_t max_bz, long long q_target,
                            unsigned long long* out_bits, cudaStream_t s, uint64_t* launches) {
  if (n_list == 0 || ov == 0 || max_bz <= 2 * ov) return;
  const uint32_t z_chunk = 4;
  const dim3 grid(n_list, (max_bz - 2 * ov + z_chunk - 1) / z_chunk);
  if (bytes == 1)
    max_gradient_at_kernel<uint8_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint8_t*>(pool), d_offsets, d_sizes, d_bricks, ov, q_target, z_chunk,
        out_bits);
  else
    max_gradient_at_kernel<uint16_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint16_t*>(pool), d_offsets, d_sizes, d_bricks, ov, q_target, z_chunk,
        out_bits);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}


// ---------------------------------------------------------------------------
// Allocation-free LOD-0 bricking (tvk_brick_lod0_noalloc).
//
// Callers that cannot allocate device memory at call time -- a host that hands
// the library a fixed memory budget up front, or code running under a stream
// capture or inside a pre-sized memory pool -- still need the per-brick
// statistics, which the regular path accumulates in device scratch it
// allocates per volume.  This variant keeps that scratch in a file-scope
// __device__ array instead: every GPU that loads the library holds
// kNoAllocScratchWords 32-bit words (about 66 KB) of it until the process exits,
// enough for kNoAllocMaxBricks bricks per call.  The array is shared by all
// calls: each call clears the part it uses before accumulating, and calls
// whose work overlaps on the GPU (on different streams, or from several host
// threads) race on it.  Host code cannot use the array's name as a device
// address, so its address is looked up once per device, with that device
// current, on the first call made on that device; make that first call before
// any stream capture begins.
// ---------------------------------------------------------------------------

namespace {

constexpr uint32_t kNoAllocMaxBricks = TVK_NOALLOC_MAX_BRICKS;
constexpr uint32_t kNoAllocWordsPerBrick = 2 + 256;  // min, max, 256 bins
constexpr uint32_t kNoAllocScratchWords = kNoAllocMaxBricks * kNoAllocWordsPerBrick;

__device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

struct NoAllocBatch {
  uint32_t coords[kNoAllocMaxBricks][3];
  uint32_t sizes[kNoAllocMaxBricks][3];
  unsigned long long out_offset[kNoAllocMaxBricks];  // voxels into the output
  uint32_t count;
};

__global__ void noalloc_clear_kernel(uint32_t* scratch, uint32_t count) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count * kNoAllocWordsPerBrick;
       i += gridDim.x * blockDim.x)
    scratch[i] = (i % kNoAllocWordsPerBrick == 0) ? 0xffffffffu : 0u;
}

template <class T>
__global__ void __launch_bounds__(kThreads)
noalloc_brick_kernel(const T* __restrict__ raw, BrickGrid g, NoAllocBatch batch,
                     T* __restrict__ out, uint32_t* scratch, uint32_t shift, uint32_t z_chunk) {
  __shared__ uint32_t bh[256];
  const uint32_t b = blockIdx.x;
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) bh[i] = 0;
  __syncthreads();
  const uint32_t bs[3] = {batch.sizes[b][0], batch.sizes[b][1], batch.sizes[b][2]};
  const uint32_t c[3] = {batch.coords[b][0], batch.coords[b][1], batch.coords[b][2]};
  const uint32_t z0 = blockIdx.y * z_chunk;
  const uint32_t z1 = min(bs[2], z0 + z_chunk);
  T* dst = out + batch.out_offset[b];
  const uint32_t sxy = bs[0] * bs[1];
  uint32_t lo = 0xffffffffu, hi = 0;
  if (z0 < z1) {
    const uint32_t n = (z1 - z0) * sxy;
    for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) {
      const uint32_t k = z0 + t / sxy;
      const uint32_t r = t - (k - z0) * sxy;
      const uint32_t j = r / bs[0];
      const uint32_t i = r - j * bs[0];
      const T v = source_voxel<T>(raw, g, c, bs, i, j, k);
      dst[uint64_t(k) * sxy + r] = v;
      const uint32_t u = v;
      lo = min(lo, u);
      hi = max(hi, u);
      if (i >= g.ov && i < bs[0] - g.ov && j >= g.ov && j < bs[1] - g.ov && k >= g.ov &&
          k < bs[2] - g.ov)
        atomicAdd(&bh[min(u >> shift, 255u)], 1u);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  uint32_t* mine = scratch + b * kNoAllocWordsPerBrick;
  if ((threadIdx.x & 31) == 0 && lo <= hi) {
    atomicMin(&mine[0], lo);
    atomicMax(&mine[1], hi);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x)
    if (bh[i]) atomicAdd(&mine[2 + i], bh[i]);
}

__global__ void noalloc_finish_kernel(const uint32_t* scratch, uint32_t count,
                                      tvk_minmax* minmax_out, uint32_t* hist_out) {
  const uint32_t b = blockIdx.x;
  if (b >= count) return;
  const uint32_t* mine = scratch + b * kNoAllocWordsPerBrick;
  if (threadIdx.x == 0) {
    // MaxMinDataBlock::SetDataFromFlatVector (IO/UVF/MaxMinDataBlock.cpp:175-195)
    tvk_minmax m;
    m.min_scalar = double(mine[0]);
    m.max_scalar = double(mine[1]);
    m.min_gradient = -1.7976931348623157e308;
    m.max_gradient = 1.7976931348623157e308;
    minmax_out[b] = m;
  }
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist_out[256u * b + i] = mine[2 + i];
}

// Device address of g_noalloc_scratch, looked up once per device and kept for
// the life of the process (a cudaDeviceReset ends the context it belongs to:
// the entry point is not for use after one).
uint32_t* noalloc_scratch_for_current_device() {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  TVK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) fail(TVK_ERR_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      fail(TVK_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                             cudaGetErrorString(e));
    addr[dev] = p;
  }
  return static_cast<uint32_t*>(addr[dev]);
}

void brick_lod0_noalloc(const void* raw, tvk_dtype dtype, const uint64_t dims[3],
                        const uint32_t bsz[3], uint32_t ov, int clamp, const uint64_t* coords,
                        uint32_t count, uint32_t shift, void* bricks_out, size_t out_bytes,
                        tvk_minmax* minmax_out, uint32_t* hist_out, cudaStream_t s) {
  if (!raw || !dims || !bsz || !coords || !bricks_out || !minmax_out || !hist_out)
    fail(TVK_ERR_INVALID_ARG, "null argument");
  if (dtype != TVK_U8 && dtype != TVK_U16) fail(TVK_ERR_INVALID_ARG, "dtype must be u8 or u16");
  if (count == 0 || count > kNoAllocMaxBricks)
    fail(TVK_ERR_INVALID_ARG, "count must be 1.." + std::to_string(kNoAllocMaxBricks) +
                                  " bricks per call (the fixed scratch holds that many)");
  if (shift > 16) fail(TVK_ERR_INVALID_ARG, "histogram shift above 16");
  const int bytes = dtype == TVK_U8 ? 1 : 2;
  // every pointer the kernels dereference must be aligned to its element type:
  // a misaligned one would fault on the GPU instead of returning an error here
  auto misaligned = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) != 0; };
  if (misaligned(raw, bytes) || misaligned(bricks_out, bytes))
    fail(TVK_ERR_INVALID_ARG, "voxel pointers must be aligned to the voxel size (2 bytes for u16)");
  if (misaligned(minmax_out, alignof(double)))
    fail(TVK_ERR_INVALID_ARG, "device_minmax_out must be 8-byte aligned");
  if (misaligned(hist_out, alignof(uint32_t)))
    fail(TVK_ERR_INVALID_ARG, "device_hist_out must be 4-byte aligned");
  BrickGrid g;
  uint64_t lod_size[3];
  for (int a = 0; a < 3; ++a) {
    if (dims[a] < 1) fail(TVK_ERR_INVALID_ARG, "volume dimensions must be >= 1");
    if (bsz[a] <= 2 * ov || bsz[a] > 4096)
      fail(TVK_ERR_INVALID_ARG, "brick size must exceed twice the overlap and be <= 4096");
    const uint64_t usable = bsz[a] - 2ull * ov;
    const uint64_t cnt = (dims[a] + usable - 1) / usable;  // ExtendedOctree.cpp:231-236
    if (cnt >= (1ull << 32)) fail(TVK_ERR_INVALID_ARG, "2^32 or more bricks along one axis");
    g.dims[a] = dims[a];
    g.B[a] = bsz[a];
    g.cnt[a] = uint32_t(cnt);
    lod_size[a] = dims[a];
  }
  if (dims[1] > UINT64_MAX / dims[0] || dims[2] > UINT64_MAX / (dims[0] * dims[1]) ||
      dims[0] * dims[1] * dims[2] > UINT64_MAX / 2)
    fail(TVK_ERR_INVALID_ARG, "volume dimensions overflow 64 bits");
  g.ov = ov;
  g.clamp = clamp ? 1 : 0;
  g.total = dims[0] * dims[1] * dims[2];
  NoAllocBatch batch;
  std::memset(&batch, 0, sizeof(batch));
  batch.count = count;
  uint64_t off = 0;
  uint32_t max_z = 0;
  for (uint32_t b = 0; b < count; ++b) {
    for (int a = 0; a < 3; ++a) {
      const uint64_t c = coords[3 * b + a];
      if (c >= g.cnt[a]) fail(TVK_ERR_INVALID_ARG, "brick coordinate out of range");
      const uint64_t core = bsz[a] - 2ull * ov;
      const bool last = c == g.cnt[a] - 1;  // ExtendedOctree::ComputeBrickSize
      batch.sizes[b][a] =
          uint32_t((last && (lod_size[a] % core)) ? (2ull * ov + lod_size[a] % core) : bsz[a]);
      batch.coords[b][a] = uint32_t(c);
    }
    batch.out_offset[b] = off;
    off += uint64_t(batch.sizes[b][0]) * batch.sizes[b][1] * batch.sizes[b][2];
    max_z = std::max(max_z, batch.sizes[b][2]);
  }
  if (off * bytes > out_bytes)
    fail(TVK_ERR_INVALID_ARG, "output buffer holds " + std::to_string(out_bytes) +
                                  " bytes, the bricks need " + std::to_string(off * bytes));
  uint32_t* scratch = noalloc_scratch_for_current_device();
  noalloc_clear_kernel<<<8, 256, 0, s>>>(scratch, count);
  TVK_CUDA(cudaGetLastError());
  const uint32_t z_chunk = 8;
  const dim3 grid(count, (max_z + z_chunk - 1) / z_chunk);
  if (bytes == 1)
    noalloc_brick_kernel<uint8_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint8_t*>(raw), g, batch, static_cast<uint8_t*>(bricks_out), scratch,
        shift, z_chunk);
  else
    noalloc_brick_kernel<uint16_t><<<grid, kThreads, 0, s>>>(
        static_cast<const uint16_t*>(raw), g, batch, static_cast<uint16_t*>(bricks_out), scratch,
        shift, z_chunk);
  TVK_CUDA(cudaGetLastError());
  noalloc_finish_kernel<<<count, 256, 0, s>>>(scratch, count, minmax_out, hist_out);
  TVK_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace tvk

extern "C" tvk_status tvk_brick_lod0_noalloc(const void* device_voxels, tvk_dtype dtype,
                                             const uint64_t dims[3], const uint32_t brick_size[3],
                                             uint32_t overlap, int clamp_to_edge,
                                             const uint64_t* brick_coords, uint32_t count,
                                             uint32_t hist_shift, void* device_bricks_out,
                                             size_t out_bytes, tvk_minmax* device_minmax_out,
                                             uint32_t* device_hist_out, void* stream) {
  try {
    tvk::brick_lod0_noalloc(device_voxels, dtype, dims, brick_size, overlap, clamp_to_edge,
                            brick_coords, count, hist_shift, device_bricks_out, out_bytes,
                            device_minmax_out, device_hist_out, static_cast<cudaStream_t>(stream));
    tvk::set_last_error("");
    return TVK_OK;
  } catch (const tvk::Error& e) {
    tvk::set_last_error(e.msg);
    return e.status;
  } catch (...) {
    tvk::set_last_error("unknown failure");
    return TVK_ERR_INTERNAL;
  }
}
