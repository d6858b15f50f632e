// lod.cu -- coarser LODs of the brick octree on sm_103a.
//
// ExtendedOctreeConverter::ComputeHierarchy (IO/UVF/ExtendedOctree/
// ExtendedOctreeConverter.inc:358-398) builds LOD l from LOD l-1 brick by brick:
// DownsampleBrick filters up to eight child bricks into each target (2x2x2 mean
// computed in double and truncated, or the 7-value median network of
// VolumeTools::Filter; 4- and 2-sample filters on odd borders), then
// FillOverlap (ExtendedOctreeConverter.cpp:1203-1372) copies the ghost layers
// from up to ten neighbours, bricks in z, y, x order.  FillOverlap is order
// dependent: a brick reads its lower neighbours after they were filled and its
// higher neighbours before (so some corner ghosts end up zero).  Processing the
// bricks in wavefronts of equal x+y+z reproduces exactly that state: a brick's
// lower face neighbours lie on the previous wavefront and every brick it reads
// on the higher side lies on a later one.
//
// Downsampling: one thread per target voxel, mean as integer sum >> k (exact:
// the double sum of at most eight 16-bit values is exact and dividing by a
// power of two then truncating is the same shift).  FillOverlap: one CTA per
// brick of the wavefront; each ghost voxel takes the source of the last copy
// (in the reference's order) whose target region holds it.
#include <algorithm>

#include "tvk_internal.h"

namespace tvk {
namespace {

constexpr int kThreads = 256;

template <class T>
__device__ __forceinline__ void order2(T& a, T& b) {
  if (a > b) { const T t = a; a = b; b = t; }
}

template <class T>
__device__ __forceinline__ T median8(T a, T b, T c, T d, T e, T f, T g) {
  // VolumeTools.h:242-262 (the eighth value is not used)
  order2(a, b); order2(c, d); order2(a, c); order2(b, d); order2(b, c);
  // InsertIntoQuadruple (VolumeTools.h:212-227) of e, then f
  T* p[2] = {&e, &f};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    T& v = *p[q];
    if (v > c) {
      order2(d, v);
    } else if (v < b) {
      d = c; c = b; b = v; order2(a, b);
    } else {
      d = c; c = v;
    }
  }
  return max(min(d, g), c);
}

template <class T>
__device__ __forceinline__ T median4(T a, T b, T c) {
  order2(a, b);
  order2(b, c);
  return max(a, b);
}

// Voxel components: scalar voxels have one; RGBA8 colour voxels (packed in a
// 32-bit word, red in the low byte) four, each filtered on its own like the
// reference's per-component loop (ExtendedOctreeConverter.inc:39-44).
template <class T>
struct Comp {
  static constexpr int n = 1;
  __device__ static uint32_t get(T v, int) { return uint32_t(v); }
  __device__ static void set(T& v, int, uint32_t x) { v = T(x); }
};
struct Rgba8 {
  uint32_t w;
};
template <>
struct Comp<Rgba8> {
  static constexpr int n = 4;
  __device__ static uint32_t get(Rgba8 v, int c) { return (v.w >> (8 * c)) & 0xffu; }
  __device__ static void set(Rgba8& v, int c, uint32_t x) {
    v.w = (v.w & ~(0xffu << (8 * c))) | ((x & 0xffu) << (8 * c));
  }
};

// Geometry of one LOD for the kernels.
struct LodGeom {
  uint32_t cnt[3];        // bricks per axis
  uint32_t lod_size[3];
  uint64_t first;         // TOC index of the first brick
};

__device__ __forceinline__ uint32_t brick_extent(const LodGeom& g, const uint32_t B[3],
                                                 uint32_t ov, int a, uint32_t c) {
  // ExtendedOctree::ComputeBrickSize (ExtendedOctree.cpp:276-285)
  const uint32_t core = B[a] - 2 * ov;
  const bool last = c == g.cnt[a] - 1;
  return (last && (g.lod_size[a] % core)) ? 2 * ov + g.lod_size[a] % core : B[a];
}

template <class T>
__global__ void __launch_bounds__(kThreads)
downsample_kernel(T* __restrict__ pool, const uint64_t* __restrict__ offsets, LodGeom lo,
                  LodGeom hi, uint32_t B0, uint32_t B1, uint32_t B2, uint32_t ov, int median,
                  uint32_t z_chunk) {
  const uint32_t B[3] = {B0, B1, B2};
  const uint32_t b = blockIdx.x;
  const uint32_t c[3] = {b % hi.cnt[0], (b / hi.cnt[0]) % hi.cnt[1], b / (hi.cnt[0] * hi.cnt[1])};
  uint32_t n[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) n[a] = brick_extent(hi, B, ov, a, c[a]);
  T* dst = pool + offsets[hi.first + b];
  const uint32_t z0 = blockIdx.y * z_chunk, z1 = min(n[2], z0 + z_chunk);
  if (z0 >= z1) return;
  const uint32_t sxy = n[0] * n[1];
  // Which child voxels an output voxel filters, axis by axis: outside the
  // inner region (ghost) or beyond the last child nothing (0, FillOverlap
  // writes the ghosts later); else the child, the position in it and whether
  // the axis has a pair of samples or the odd boundary sample.
  auto axis = [&](int a, uint32_t va, uint32_t& child, uint32_t& l, uint32_t& cs,
                  int& pair) -> bool {
    if (va < ov || va >= n[a] - ov) return false;
    const uint32_t tt = va - ov;
    const uint32_t split = (B[a] - 2 * ov + 1) / 2;  // ceil(core / 2)
    const uint32_t cc = tt >= split ? 1u : 0u;
    child = 2 * c[a] + cc;
    if (child >= lo.cnt[a]) return false;
    l = tt - cc * split;
    cs = brick_extent(lo, B, ov, a, child);
    const uint32_t even = (cs - 2 * ov) / 2;
    if (l < even) pair = 1;
    else if (l == even && (cs & 1u)) pair = 0;
    else return false;
    return true;
  };
  // one warp per output row (y, z terms once per row), lanes along x
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t rows = (z1 - z0) * n[1];
  for (uint32_t rr = warp; rr < rows; rr += nwarps) {
    const uint32_t k = z0 + rr / n[1];
    const uint32_t j = rr - (k - z0) * n[1];
    const uint32_t r0 = j * n[0];
    uint32_t child[3], l[3], cs[3];
    int pair[3];  // 1: two samples along the axis, 0: the odd boundary sample
    const bool row_covered = axis(1, j, child[1], l[1], cs[1], pair[1]) &&
                             axis(2, k, child[2], l[2], cs[2], pair[2]);
    // the x axis per row: the two children this row's voxels fall in (the
    // first and second half of the core), their x extents and pair limits
    const uint32_t split0 = (B[0] - 2 * ov + 1) / 2;
    uint32_t cs_a = 0, cs_b = 0, even_a = 0, even_b = 0;
    const T* src_a = nullptr;
    const T* src_b = nullptr;
    if (row_covered) {
      const uint64_t yz = lo.first + child[1] * lo.cnt[0] + child[2] * lo.cnt[0] * lo.cnt[1];
      const uint32_t ch = 2 * c[0];
      if (ch < lo.cnt[0]) {
        cs_a = brick_extent(lo, B, ov, 0, ch);
        even_a = (cs_a - 2 * ov) / 2;
        src_a = pool + offsets[yz + ch];
      }
      if (ch + 1 < lo.cnt[0]) {
        cs_b = brick_extent(lo, B, ov, 0, ch + 1);
        even_b = (cs_b - 2 * ov) / 2;
        src_b = pool + offsets[yz + ch + 1];
      }
    }
   for (uint32_t i = lane; i < n[0]; i += 32) {
    const uint32_t r = r0 + i;
    T out{};
    bool covered = row_covered && i >= ov && i < n[0] - ov;
    const T* src = nullptr;
    if (covered) {  // axis(0, i, ...) from the row's two children
      const uint32_t tt = i - ov;
      const bool second = tt >= split0;
      src = second ? src_b : src_a;
      l[0] = second ? tt - split0 : tt;
      cs[0] = second ? cs_b : cs_a;
      const uint32_t even = second ? even_b : even_a;
      if (!src) covered = false;
      else if (l[0] < even) pair[0] = 1;
      else if (l[0] == even && (cs[0] & 1u)) pair[0] = 0;
      else covered = false;
    }
    if (covered) {
      const uint32_t X = 2 * l[0] + ov, Y = 2 * l[1] + ov, Z = 2 * l[2] + ov;
      auto S = [&](uint32_t x, uint32_t y, uint32_t z) -> T {
        return src[x + (uint64_t(y) + uint64_t(z) * cs[1]) * cs[0]];
      };
      const int np = pair[0] + pair[1] + pair[2];
      if (np == 3) {
        // DownsampleBricktoBrick p0..p7 order (.inc:28-35)
        const T a0 = S(X, Y, Z), a1 = S(X, Y, Z + 1), a2 = S(X, Y + 1, Z), a3 = S(X, Y + 1, Z + 1);
        const T a4 = S(X + 1, Y, Z), a5 = S(X + 1, Y, Z + 1), a6 = S(X + 1, Y + 1, Z),
                a7 = S(X + 1, Y + 1, Z + 1);
#pragma unroll
        for (int q = 0; q < Comp<T>::n; ++q) {
          const uint32_t b0 = Comp<T>::get(a0, q), b1 = Comp<T>::get(a1, q),
                         b2 = Comp<T>::get(a2, q), b3 = Comp<T>::get(a3, q),
                         b4 = Comp<T>::get(a4, q), b5 = Comp<T>::get(a5, q),
                         b6 = Comp<T>::get(a6, q), b7 = Comp<T>::get(a7, q);
          Comp<T>::set(out, q, median ? median8<uint32_t>(b0, b1, b2, b3, b4, b5, b6)
                                      : (b0 + b1 + b2 + b3 + b4 + b5 + b6 + b7) >> 3);
        }
      } else if (np == 2) {
        T a0, a1, a2, a3;
        if (!pair[0]) {  // plane at the end of x: p0, p1, p2, p3
          a0 = S(X, Y, Z); a1 = S(X, Y, Z + 1); a2 = S(X, Y + 1, Z); a3 = S(X, Y + 1, Z + 1);
        } else if (!pair[1]) {  // end of y: p0, p1, p4, p5
          a0 = S(X, Y, Z); a1 = S(X, Y, Z + 1); a2 = S(X + 1, Y, Z); a3 = S(X + 1, Y, Z + 1);
        } else {  // end of z: p0, p2, p4, p6
          a0 = S(X, Y, Z); a1 = S(X, Y + 1, Z); a2 = S(X + 1, Y, Z); a3 = S(X + 1, Y + 1, Z);
        }
#pragma unroll
        for (int q = 0; q < Comp<T>::n; ++q) {
          const uint32_t b0 = Comp<T>::get(a0, q), b1 = Comp<T>::get(a1, q),
                         b2 = Comp<T>::get(a2, q), b3 = Comp<T>::get(a3, q);
          Comp<T>::set(out, q, median ? median4<uint32_t>(b0, b1, b2) : (b0 + b1 + b2 + b3) >> 2);
        }
      } else if (np == 1) {
        T a0 = S(X, Y, Z), a1;
        if (pair[2]) a1 = S(X, Y, Z + 1);       // x/y line: p0, p1
        else if (pair[0]) a1 = S(X + 1, Y, Z);  // y/z line: p0, p4
        else a1 = S(X, Y + 1, Z);               // x/z line: p0, p2
#pragma unroll
        for (int q = 0; q < Comp<T>::n; ++q) {
          const uint32_t b0 = Comp<T>::get(a0, q), b1 = Comp<T>::get(a1, q);
          Comp<T>::set(out, q, median ? b0 : (b0 + b1) >> 1);
        }
      } else {
        out = S(X, Y, Z);  // odd corner copies *p0 (.inc:244-246)
      }
    }
    dst[uint64_t(k) * sxy + r] = out;
   }
  }
}

// The ghost shell of an n0 x n1 x n2 brick (voxels within ov of a face),
// enumerated without visiting the inner voxels: the ghost planes along z,
// then the ghost rows of the other planes, then the ghost x ends of the
// remaining rows.
struct Shell {
  uint32_t n[3], ov, gk, gj, gi, mk, mj;
  uint32_t a, b, total;  // segment ends
};

__device__ __forceinline__ Shell make_shell(const uint32_t n[3], uint32_t ov) {
  Shell s;
  s.n[0] = n[0]; s.n[1] = n[1]; s.n[2] = n[2];
  s.ov = ov;
  s.gk = min(n[2], 2 * ov);
  s.gj = min(n[1], 2 * ov);
  s.gi = min(n[0], 2 * ov);
  s.mk = n[2] - s.gk;
  s.mj = n[1] - s.gj;
  s.a = s.gk * n[1] * n[0];
  s.b = s.a + s.mk * s.gj * n[0];
  s.total = s.b + s.mk * s.mj * s.gi;
  return s;
}

// p-th ghost index of an axis of extent n with g = min(n, 2 ov) ghost layers
__device__ __forceinline__ uint32_t ghost_index(uint32_t p, uint32_t n, uint32_t g, uint32_t ov) {
  return p < min(ov, n) ? p : n - g + p;
}

__device__ __forceinline__ void shell_voxel(const Shell& s, uint32_t t, uint32_t& i, uint32_t& j,
                                            uint32_t& k) {
  if (t < s.a) {
    const uint32_t plane = s.n[1] * s.n[0];
    k = ghost_index(t / plane, s.n[2], s.gk, s.ov);
    const uint32_t r = t % plane;
    j = r / s.n[0];
    i = r % s.n[0];
  } else if (t < s.b) {
    t -= s.a;
    const uint32_t slab = s.gj * s.n[0];
    k = s.ov + t / slab;
    const uint32_t r = t % slab;
    j = ghost_index(r / s.n[0], s.n[1], s.gj, s.ov);
    i = r % s.n[0];
  } else {
    t -= s.b;
    const uint32_t slab = s.mj * s.gi;
    k = s.ov + t / slab;
    const uint32_t r = t % slab;
    j = s.ov + r / s.gi;
    i = ghost_index(r % s.gi, s.n[0], s.gi, s.ov);
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
fill_overlap_kernel(T* __restrict__ pool, const uint64_t* __restrict__ offsets, LodGeom g,
                    const uint32_t* __restrict__ wave, uint32_t B0, uint32_t B1, uint32_t B2,
                    uint32_t ov, int clamp) {
  // Brick wave[blockIdx.x]; its ghost shell is split over gridDim.y CTAs
  // (one CTA when clamping: the clamp steps are ordered by __syncthreads).
  const uint32_t B[3] = {B0, B1, B2};
  const uint32_t b = wave[blockIdx.x];
  const uint32_t c[3] = {b % g.cnt[0], (b / g.cnt[0]) % g.cnt[1], b / (g.cnt[0] * g.cnt[1])};
  uint32_t n[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) n[a] = brick_extent(g, B, ov, a, c[a]);
  T* dst = pool + offsets[g.first + b];
  const bool has_lo[3] = {c[0] > 0, c[1] > 0, c[2] > 0};
  const bool has_hi[3] = {c[0] + 1 < g.cnt[0], c[1] + 1 < g.cnt[1], c[2] + 1 < g.cnt[2]};
  auto brick_ptr = [&](int dx, int dy, int dz) -> const T* {
    return pool + offsets[g.first + (c[0] + dx) + (c[1] + dy) * g.cnt[0] +
                          (c[2] + dz) * g.cnt[0] * g.cnt[1]];
  };
  const Shell sh = make_shell(n, ov);
  const uint32_t t0 = blockIdx.y * blockDim.x + threadIdx.x, dt = gridDim.y * blockDim.x;
  for (uint32_t t = t0; t < sh.total; t += dt) {
    uint32_t i, j, k;
    shell_voxel(sh, t, i, j, k);
    const bool xh = i >= n[0] - ov, yh = j >= n[1] - ov, zh = k >= n[2] - ov;
    const bool xl = i < ov, yl = j < ov, zl = k < ov;
    // the last copy of FillOverlap whose target region holds (i, j, k)
    int dx = 0, dy = 0, dz = 0;
    bool found = true;
    if (has_hi[0] && has_hi[1] && has_hi[2] && xh && yh && zh) { dx = 1; dy = 1; dz = 1; }
    else if (has_hi[1] && has_hi[2] && yh && zh) { dy = 1; dz = 1; }
    else if (has_hi[0] && has_hi[2] && xh && zh) { dx = 1; dz = 1; }
    else if (has_hi[0] && has_hi[1] && xh && yh) { dx = 1; dy = 1; }
    else if (has_lo[2] && zl) { dz = -1; }
    else if (has_lo[1] && yl) { dy = -1; }
    else if (has_lo[0] && xl) { dx = -1; }
    else if (has_hi[2] && zh) { dz = 1; }
    else if (has_hi[1] && yh) { dy = 1; }
    else if (has_hi[0] && xh) { dx = 1; }
    else found = false;
    if (!found) continue;
    // source coordinates: a higher neighbour's first inner layers, a lower
    // neighbour's last inner layers, the same index along the other axes
    uint32_t s[3] = {i, j, k};
    uint32_t ns[3];
    const int d[3] = {dx, dy, dz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      ns[a] = d[a] == 0 ? n[a] : brick_extent(g, B, ov, a, c[a] + d[a]);
      if (d[a] > 0) s[a] = s[a] - (n[a] - ov) + ov;
      else if (d[a] < 0) s[a] = s[a] + ns[a] - 2 * ov;
    }
    const T* src = brick_ptr(dx, dy, dz);
    dst[i + (uint64_t(j) + uint64_t(k) * n[1]) * n[0]] =
        src[s[0] + (uint64_t(s[1]) + uint64_t(s[2]) * ns[1]) * ns[0]];
  }
  if (!clamp) return;
  // ClampToEdge (ExtendedOctreeConverter.cpp:376-462) on sides without a
  // neighbour: x, then y, then z, each reading the previous step's result
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    __syncthreads();
    for (uint32_t t = t0; t < sh.total; t += dt) {
      uint32_t v[3];
      shell_voxel(sh, t, v[0], v[1], v[2]);
      uint32_t from = v[a];
      if (!has_lo[a] && v[a] < ov) from = ov;
      else if (!has_hi[a] && v[a] >= n[a] - ov) from = n[a] - 1 - ov;
      else continue;
      uint32_t s[3] = {v[0], v[1], v[2]};
      s[a] = from;
      dst[v[0] + (uint64_t(v[1]) + uint64_t(v[2]) * n[1]) * n[0]] =
          dst[s[0] + (uint64_t(s[1]) + uint64_t(s[2]) * n[1]) * n[0]];
    }
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
brick_minmax_kernel(const T* __restrict__ pool, const uint64_t* __restrict__ offsets,
                    const uint64_t* __restrict__ voxels, uint64_t first, uint32_t* out_min,
                    uint32_t* out_max) {
  // ComputeBrickStats<T> (.inc:408-444): every voxel of the brick, the brick
  // split over gridDim.y CTAs; 16-byte loads (bricks start 256-byte aligned)
  const uint64_t b = first + blockIdx.x;
  const T* p = pool + offsets[b];
  const uint64_t nv = voxels[b];
  constexpr uint32_t kPer = 16 / sizeof(T);
  const uint64_t nvec = nv / kPer;
  const uint64_t per_cta = (nvec + gridDim.y - 1) / gridDim.y;
  const uint64_t v0 = blockIdx.y * per_cta, v1 = min(nvec, v0 + per_cta);
  const uint4* pv = reinterpret_cast<const uint4*>(p);
  uint32_t lo = 0xffffffffu, hi = 0;
  for (uint64_t t = v0 + threadIdx.x; t < v1; t += blockDim.x) {
    const uint4 w = pv[t];
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (sizeof(T) == 1) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const uint32_t v = (words[q] >> (8 * e)) & 0xffu;
          lo = min(lo, v);
          hi = max(hi, v);
        }
      } else {
        const uint32_t a = words[q] & 0xffffu, c = words[q] >> 16;
        lo = min(lo, min(a, c));
        hi = max(hi, max(a, c));
      }
    }
  }
  if (blockIdx.y == gridDim.y - 1)  // the tail after the last full 16 bytes
    for (uint64_t t = nvec * kPer + threadIdx.x; t < nv; t += blockDim.x) {
      const uint32_t v = p[t];
      lo = min(lo, v);
      hi = max(hi, v);
    }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ uint32_t slo[kThreads / 32], shi[kThreads / 32];
  if ((threadIdx.x & 31) == 0) { slo[threadIdx.x >> 5] = lo; shi[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; ++w) { lo = min(lo, slo[w]); hi = max(hi, shi[w]); }
    atomicMin(&out_min[blockIdx.x], lo);
    atomicMax(&out_max[blockIdx.x], hi);
  }
}

}  // namespace

void build_lod_levels(void* pool, int bytes, const uint64_t* d_offsets, const uint64_t* d_voxels,
                      const std::vector<LodInfo>& lods, const std::vector<uint64_t>& lod_first,
                      const uint32_t B[3], uint32_t ov, bool clamp, bool median,
                      uint32_t* d_min, uint32_t* d_max, uint32_t* d_wave, cudaStream_t s,
                      uint64_t* launches) {
  auto geom = [&](size_t l) {
    LodGeom g;
    for (int a = 0; a < 3; ++a) {
      g.cnt[a] = uint32_t(lods[l].bricks[a]);
      g.lod_size[a] = uint32_t(lods[l].size[a]);
    }
    g.first = lod_first[l];
    return g;
  };
  std::vector<uint32_t> wave_host;
  for (size_t l = 1; l < lods.size(); ++l) {
    const LodGeom lo = geom(l - 1), hi = geom(l);
    const uint64_t nb = uint64_t(hi.cnt[0]) * hi.cnt[1] * hi.cnt[2];
    // z planes per CTA: up to 8, fewer for the coarse levels (few bricks), so
    // that a level still spreads over about 8 CTAs per SM (a CTA's warps walk
    // their rows one after the other)
    const uint32_t z_chunk =
        uint32_t(std::min<uint64_t>(8, std::max<uint64_t>(1, nb * B[2] / (152ull * 8))));
    const dim3 grid(uint32_t(nb), (B[2] + z_chunk - 1) / z_chunk);
    if (bytes == 4)
      downsample_kernel<Rgba8><<<grid, kThreads, 0, s>>>(static_cast<Rgba8*>(pool), d_offsets,
                                                         lo, hi, B[0], B[1], B[2], ov,
                                                         median ? 1 : 0, z_chunk);
    else if (bytes == 1)
      downsample_kernel<uint8_t><<<grid, kThreads, 0, s>>>(static_cast<uint8_t*>(pool), d_offsets,
                                                           lo, hi, B[0], B[1], B[2], ov,
                                                           median ? 1 : 0, z_chunk);
    else
      downsample_kernel<uint16_t><<<grid, kThreads, 0, s>>>(static_cast<uint16_t*>(pool),
                                                            d_offsets, lo, hi, B[0], B[1], B[2],
                                                            ov, median ? 1 : 0, z_chunk);
    TVK_CUDA(cudaGetLastError());
    ++*launches;
    // FillOverlap, one launch per wavefront x + y + z = w, in increasing w
    const uint32_t nw = hi.cnt[0] + hi.cnt[1] + hi.cnt[2] - 2;
    wave_host.clear();
    std::vector<uint32_t> starts;
    for (uint32_t w = 0; w < nw; ++w) {
      starts.push_back(uint32_t(wave_host.size()));
      for (uint32_t z = 0; z < hi.cnt[2]; ++z)
        for (uint32_t y = 0; y < hi.cnt[1]; ++y) {
          if (y + z > w || w - y - z >= hi.cnt[0]) continue;
          const uint32_t x = w - y - z;
          wave_host.push_back(x + y * hi.cnt[0] + z * hi.cnt[0] * hi.cnt[1]);
        }
    }
    starts.push_back(uint32_t(wave_host.size()));
    TVK_CUDA(cudaMemcpyAsync(d_wave, wave_host.data(), wave_host.size() * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, s));
    for (uint32_t w = 0; w < nw; ++w) {
      const uint32_t cnt = starts[w + 1] - starts[w];
      if (!cnt) continue;
      // the shell of a full brick split over enough CTAs to fill the GPU
      // (one CTA per brick when clamping orders its steps with barriers)
      const uint32_t split = clamp ? 1u : std::max(1u, std::min(32u, 1216u / cnt));
      const dim3 fgrid(cnt, split);
      if (bytes == 4)
        fill_overlap_kernel<uint32_t><<<fgrid, kThreads, 0, s>>>(
            static_cast<uint32_t*>(pool), d_offsets, hi, d_wave + starts[w], B[0], B[1], B[2], ov,
            clamp ? 1 : 0);
      else if (bytes == 1)
        fill_overlap_kernel<uint8_t><<<fgrid, kThreads, 0, s>>>(
            static_cast<uint8_t*>(pool), d_offsets, hi, d_wave + starts[w], B[0], B[1], B[2], ov,
            clamp ? 1 : 0);
      else
        fill_overlap_kernel<uint16_t><<<fgrid, kThreads, 0, s>>>(
            static_cast<uint16_t*>(pool), d_offsets, hi, d_wave + starts[w], B[0], B[1], B[2], ov,
            clamp ? 1 : 0);
      TVK_CUDA(cudaGetLastError());
      ++*launches;
    }
    // the wave list is pageable host memory reused by the next level
    TVK_CUDA(cudaStreamSynchronize(s));
    if (bytes == 4) continue;  // colour bricks carry no statistics
    TVK_CUDA(cudaMemsetAsync(d_min + hi.first, 0xff, nb * sizeof(uint32_t), s));
    TVK_CUDA(cudaMemsetAsync(d_max + hi.first, 0, nb * sizeof(uint32_t), s));
    const dim3 mgrid(uint32_t(nb), std::max(1u, std::min(64u, 2432u / uint32_t(nb))));
    if (bytes == 1)
      brick_minmax_kernel<uint8_t><<<mgrid, kThreads, 0, s>>>(
          static_cast<const uint8_t*>(pool), d_offsets, d_voxels, hi.first, d_min + hi.first,
          d_max + hi.first);
    else
      brick_minmax_kernel<uint16_t><<<mgrid, kThreads, 0, s>>>(
          static_cast<const uint16_t*>(pool), d_offsets, d_voxels, hi.first, d_min + hi.first,
          d_max + hi.first);
    TVK_CUDA(cudaGetLastError());
    ++*launches;
  }
}

}  // namespace tvk
