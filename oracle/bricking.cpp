// bricking.cpp -- CPU restatement of Tuvok's LOD-0 bricking, per-brick
// statistics, histograms and brick metadata.
//
// TEST INFRASTRUCTURE ONLY (the checker for tuvok_gb300's CUDA bricking path).
// Each function follows the reference routine named in its comment; paths are
// relative to the Tuvok source tree.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace {

template <class T>
inline const T* as(const void* p) { return static_cast<const T*>(p); }

}  // namespace

extern "C" int orc_lod_table(const uint64_t dims[3], const uint32_t brick_size[3],
                             uint32_t overlap, uint64_t* lod_sizes,
                             uint64_t* brick_counts, int max_lods) {
  // ExtendedOctree::ComputeMetadata, ExtendedOctree.cpp:188-243: halve each
  // axis with ceil until every axis is 1; brick count = ceil(size / usable).
  uint64_t v[3] = {dims[0], dims[1], dims[2]};
  const uint64_t usable[3] = {brick_size[0] - 2ull * overlap,
                              brick_size[1] - 2ull * overlap,
                              brick_size[2] - 2ull * overlap};
  int n = 0;
  bool first = true;
  do {
    if (!first) {
      for (int a = 0; a < 3; ++a)
        if (v[a] > 1) v[a] = uint64_t(std::ceil(v[a] / 2.0));
    }
    first = false;
    if (n < max_lods) {
      for (int a = 0; a < 3; ++a) {
        lod_sizes[3 * n + a] = v[a];
        brick_counts[3 * n + a] = uint64_t(std::ceil(v[a] / double(usable[a])));
      }
    }
    ++n;
  } while (v[0] > 1 || v[1] > 1 || v[2] > 1);
  return n;
}

extern "C" void orc_lod_aspect(const uint64_t dims[3], uint32_t lod, double out[3]) {
  // ExtendedOctree::ComputeMetadata (ExtendedOctree.cpp:188-243): an axis that
  // halves from an odd size gains size / ceil(size / 2) (in float), an even one
  // 2; the result is normalised by its largest component every level.
  uint64_t v[3] = {dims[0], dims[1], dims[2]};
  double asp[3] = {1, 1, 1};
  for (uint32_t l = 1; l <= lod; ++l) {
    for (int a = 0; a < 3; ++a) {
      if (v[a] > 1) {
        const uint64_t h = (v[a] + 1) / 2;
        asp[a] *= (v[a] % 2) ? double(float(v[a]) / float(h)) : 2.0;
        v[a] = h;
      }
    }
    const double m = std::max(asp[0], std::max(asp[1], asp[2]));
    for (int a = 0; a < 3; ++a) asp[a] /= m;
  }
  for (int a = 0; a < 3; ++a) out[a] = asp[a];
}

extern "C" void orc_brick_size(const uint64_t lod_size[3], const uint64_t brick_count[3],
                               const uint32_t brick_size[3], uint32_t overlap,
                               const uint64_t coords[3], uint64_t out[3]) {
  // ExtendedOctree::ComputeBrickSize, ExtendedOctree.cpp:276-285.
  for (int a = 0; a < 3; ++a) {
    const uint64_t core = brick_size[a] - 2ull * overlap;
    const bool last = coords[a] == brick_count[a] - 1;
    out[a] = (last && (lod_size[a] % core)) ? (2ull * overlap + lod_size[a] % core)
                                            : brick_size[a];
  }
}

namespace {

template <class T>
void lod0_brick(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                bool clamp, const uint64_t c[3], T* out) {
  uint64_t lod[3 * 64], cnt[3 * 64];
  orc_lod_table(dims, B, ov, lod, cnt, 64);
  uint64_t bs[3];
  orc_brick_size(lod, cnt, B, ov, c, bs);
  const uint64_t total = dims[0] * dims[1] * dims[2];
  // GetInputBrick, ExtendedOctreeConverter.cpp:288-373.  Without clamping the
  // brick starts zeroed (:300-302).  With clamping the reference leaves the
  // previous brick's bytes in place before ClampToEdge overwrites the borders;
  // those are all overwritten for bricks whose reads stay inside the file, so a
  // zero start gives the same result there.
  std::fill(out, out + bs[0] * bs[1] * bs[2], T(0));
  const uint64_t xs = c[0] == 0 ? ov : 0, ys = c[1] == 0 ? ov : 0, zs = c[2] == 0 ? ov : 0;
  const uint64_t ye = bs[1] - ((c[1] == cnt[1] - 1) ? ov : 0);
  const uint64_t ze = bs[2] - ((c[2] == cnt[2] - 1) ? ov : 0);
  uint64_t line = bs[0];
  if (c[0] == 0) line -= ov;
  if (c[0] == cnt[0] - 1) line -= ov;
  for (uint64_t z = 0; z < ze - zs; ++z) {
    for (uint64_t y = 0; y < ye - ys; ++y) {
      // byte offset into the raw file, in voxels (:335-338); unsigned wrap-around
      // of the "0-(overlap-xStart)" term is intended and cancels out.
      const uint64_t in = (0 - (uint64_t(ov) - xs) + c[0] * (B[0] - 2ull * ov)) +
                          (y - (uint64_t(ov) - ys) + c[1] * (B[1] - 2ull * ov)) * dims[0] +
                          (z - (uint64_t(ov) - zs) + c[2] * (B[2] - 2ull * ov)) * dims[0] * dims[1];
      const uint64_t o = xs + (y + ys) * bs[0] + (z + zs) * bs[0] * bs[1];
      // LargeRAWFile::ReadRAW: a read past the end of the file is short.
      for (uint64_t i = 0; i < line; ++i)
        out[o + i] = (in + i < total) ? raw[in + i] : T(0);
    }
  }
  if (!clamp) return;
  // ClampToEdge, ExtendedOctreeConverter.cpp:376-462, in its order x, y, z.
  const bool s[3] = {c[0] == 0, c[1] == 0, c[2] == 0};
  const bool e[3] = {c[0] == cnt[0] - 1, c[1] == cnt[1] - 1, c[2] == cnt[2] - 1};
  auto at = [&](uint64_t x, uint64_t y, uint64_t z) -> T& {
    return out[x + y * bs[0] + z * bs[0] * bs[1]];
  };
  if (s[0])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t y = 0; y < bs[1]; ++y)
        for (uint64_t o = 0; o < ov; ++o) at(ov - 1 - o, y, z) = at(ov, y, z);
  if (e[0])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t y = 0; y < bs[1]; ++y)
        for (uint64_t o = 0; o < ov; ++o) at(bs[0] - ov + o, y, z) = at(bs[0] - 1 - ov, y, z);
  if (s[1])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, ov - 1 - o, z) = at(x, ov, z);
  if (e[1])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, bs[1] - ov + o, z) = at(x, bs[1] - 1 - ov, z);
  if (s[2])
    for (uint64_t y = 0; y < bs[1]; ++y)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, y, ov - 1 - o) = at(x, y, ov);
  if (e[2])
    for (uint64_t y = 0; y < bs[1]; ++y)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, y, bs[2] - ov + o) = at(x, y, bs[2] - 1 - ov);
}

template <class T>
void stats(const T* p, uint64_t n, double* mn, double* mx) {
  // ComputeBrickStats<T>, ExtendedOctreeConverter.inc:408-444: every voxel of
  // the brick, ghost included, compared as double.
  double lo = std::numeric_limits<double>::max();
  double hi = -std::numeric_limits<double>::max();
  for (uint64_t i = 0; i < n; ++i) {
    const double cur = static_cast<double>(p[i]);
    lo = cur < lo ? cur : lo;
    hi = cur > hi ? cur : hi;
  }
  *mn = lo;
  *mx = hi;
}

template <class T>
uint64_t hist1d(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                uint64_t* hist) {
  // Histogram1DDataBlock::ComputeTemplate<T>, Histogram1DDataBlock.cpp:120-161:
  // every LOD-0 brick, inner voxels only.
  const uint64_t nb = uint64_t(1) << (8 * sizeof(T));
  std::fill(hist, hist + nb, 0ull);
  uint64_t lod[3 * 64], cnt[3 * 64];
  orc_lod_table(dims, B, ov, lod, cnt, 64);
  std::vector<T> brick(uint64_t(B[0]) * B[1] * B[2]);
  for (uint64_t bz = 0; bz < cnt[2]; ++bz)
    for (uint64_t by = 0; by < cnt[1]; ++by)
      for (uint64_t bx = 0; bx < cnt[0]; ++bx) {
        const uint64_t c[3] = {bx, by, bz};
        uint64_t bs[3];
        orc_brick_size(lod, cnt, B, ov, c, bs);
        lod0_brick<T>(raw, dims, B, ov, false, c, brick.data());
        for (uint64_t z = ov; z < bs[2] - ov; ++z)
          for (uint64_t y = ov; y < bs[1] - ov; ++y)
            for (uint64_t x = ov; x < bs[0] - ov; ++x)
              hist[size_t(brick[x + y * bs[0] + z * bs[0] * bs[1]])]++;
      }
  uint64_t len = nb;
  while (len > 0 && hist[len - 1] == 0) --len;
  return len;
}

template <class T>
void hist256(const T* p, const uint64_t n[3], uint32_t ov, uint32_t shift, uint32_t* h) {
  std::fill(h, h + 256, 0u);
  for (uint64_t z = ov; z < n[2] - ov; ++z)
    for (uint64_t y = ov; y < n[1] - ov; ++y)
      for (uint64_t x = ov; x < n[0] - ov; ++x) {
        const uint32_t v = uint32_t(p[x + y * n[0] + z * n[0] * n[1]]) >> shift;
        h[v > 255 ? 255 : v]++;
      }
}

}  // namespace

extern "C" void orc_lod0_brick(const void* raw, int dtype, const uint64_t dims[3],
                               const uint32_t brick_size[3], uint32_t overlap,
                               int clamp_to_edge, const uint64_t coords[3], void* out) {
  if (dtype == 2)  // RGBA8: the same copy of 4-byte voxels
    lod0_brick<uint32_t>(as<uint32_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                         coords, static_cast<uint32_t*>(out));
  else if (dtype == 0)
    lod0_brick<uint8_t>(as<uint8_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                        coords, static_cast<uint8_t*>(out));
  else
    lod0_brick<uint16_t>(as<uint16_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                         coords, static_cast<uint16_t*>(out));
}

extern "C" void orc_brick_stats(const void* brick, int dtype, uint64_t n_voxels,
                                double* min_out, double* max_out) {
  if (dtype == 0)
    stats<uint8_t>(as<uint8_t>(brick), n_voxels, min_out, max_out);
  else
    stats<uint16_t>(as<uint16_t>(brick), n_voxels, min_out, max_out);
}

extern "C" uint64_t orc_histogram1d(const void* raw, int dtype, const uint64_t dims[3],
                                    const uint32_t brick_size[3], uint32_t overlap,
                                    uint64_t* hist) {
  if (dtype == 0) return hist1d<uint8_t>(as<uint8_t>(raw), dims, brick_size, overlap, hist);
  return hist1d<uint16_t>(as<uint16_t>(raw), dims, brick_size, overlap, hist);
}

extern "C" void orc_brick_hist256(const void* brick, int dtype, const uint64_t n[3],
                                  uint32_t overlap, uint32_t shift, uint32_t* hist) {
  if (dtype == 0)
    hist256<uint8_t>(as<uint8_t>(brick), n, overlap, shift, hist);
  else
    hist256<uint16_t>(as<uint16_t>(brick), n, overlap, shift, hist);
}

extern "C" void orc_brick_metadata(const uint64_t lod_size[3], const uint64_t brick_count[3],
                                   const uint32_t brick_size[3], uint32_t overlap,
                                   const double aspect[3], float* centers, float* extents,
                                   uint32_t* n_voxels) {
  // UVFDataset::ComputeMetadataTOC, uvfDataset.cpp:242-288.  Loop order x, y, z
  // with the corner accumulated in float, exactly as the reference does.
  const float asp[3] = {float(aspect[0]), float(aspect[1]), float(aspect[2])};
  float nd[3] = {float(lod_size[0]) * asp[0], float(lod_size[1]) * asp[1],
                 float(lod_size[2]) * asp[2]};
  const float maxv = std::max(nd[0], std::max(nd[1], nd[2]));
  for (int a = 0; a < 3; ++a) nd[a] /= maxv;
  float corner[3] = {0, 0, 0};
  float ext[3] = {0, 0, 0};
  for (uint64_t x = 0; x < brick_count[0]; ++x) {
    corner[1] = 0;
    for (uint64_t y = 0; y < brick_count[1]; ++y) {
      corner[2] = 0;
      for (uint64_t z = 0; z < brick_count[2]; ++z) {
        const uint64_t c[3] = {x, y, z};
        uint64_t bs[3];
        orc_brick_size(lod_size, brick_count, brick_size, overlap, c, bs);
        const uint64_t k = z * brick_count[0] * brick_count[1] + y * brick_count[0] + x;
        for (int a = 0; a < 3; ++a) {
          ext[a] = float(bs[a] - 2ull * overlap) * asp[a] / maxv;
          centers[3 * k + a] = (corner[a] + ext[a] / 2.0f) - nd[a] * 0.5f;
          extents[3 * k + a] = ext[a];
          n_voxels[3 * k + a] = uint32_t(bs[a]);
        }
        corner[2] += ext[2];
      }
      corner[1] += ext[1];
    }
    corner[0] += ext[0];
  }
}

namespace {
// Visits every inner voxel of every LOD-0 brick (bricks in TOC order, voxels z, y,
// x) with its value and |gradient|: Histogram2DDataBlock::ComputeGradient
// (Histogram2DDataBlock.cpp:327-345), central differences normalised by
// 2 * max(T) in double, DOUBLEVECTOR3::length() = sqrt(x*x + y*y + z*z).
template <class T, class F>
void for_each_gradient(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                       bool clamp, F&& f) {
  uint64_t lod[3 * 64], cnt[3 * 64];
  orc_lod_table(dims, B, ov, lod, cnt, 64);
  std::vector<T> brick(uint64_t(B[0]) * B[1] * B[2]);
  const double nf = double(std::numeric_limits<T>::max());
  for (uint64_t bz = 0; bz < cnt[2]; ++bz)
    for (uint64_t by = 0; by < cnt[1]; ++by)
      for (uint64_t bx = 0; bx < cnt[0]; ++bx) {
        const uint64_t c[3] = {bx, by, bz};
        uint64_t bs[3];
        orc_brick_size(lod, cnt, B, ov, c, bs);
        lod0_brick<T>(raw, dims, B, ov, clamp, c, brick.data());
        const uint64_t sx = bs[0], sxy = bs[0] * bs[1];
        for (uint64_t z = ov; z < bs[2] - ov; ++z)
          for (uint64_t y = ov; y < bs[1] - ov; ++y)
            for (uint64_t x = ov; x < bs[0] - ov; ++x) {
              const uint64_t i = x + y * sx + z * sxy;
              const double gx = (double(brick[i - 1]) - double(brick[i + 1])) / (nf * 2);
              const double gy = (double(brick[i - sx]) - double(brick[i + sx])) / (nf * 2);
              const double gz = (double(brick[i - sxy]) - double(brick[i + sxy])) / (nf * 2);
              f(brick[i], std::sqrt(gx * gx + gy * gy + gz * gz));
            }
      }
}

template <class T>
double max_gradient(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                    bool clamp) {
  // Histogram2DDataBlock::ComputeTemplate<T> first loop (Histogram2DDataBlock.cpp:363-397)
  double best = 0;
  for_each_gradient<T>(raw, dims, B, ov, clamp, [&](T, double l) {
    if (l > best) best = l;
  });
  return best;
}

template <class T>
double histogram2d(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                   bool clamp, uint64_t value_bins, double max_nonzero, uint64_t* hist) {
  // Histogram2DDataBlock::ComputeTemplate<T> second loop (Histogram2DDataBlock.cpp:399-435):
  // gradient bin = min(255, size_t(|g| / max|g| * 255.0f)); value bin = the raw
  // value, or value * (bins - 1) / max_nonzero when the value range exceeds the
  // bins; both clamped to the table.  A constant volume (max |g| = 0) divides
  // 0 by 0 there, which C++ leaves undefined; this restatement puts those
  // voxels in gradient bin 0.
  const double gmax = max_gradient<T>(raw, dims, B, ov, clamp);
  std::fill(hist, hist + value_bins * 256, uint64_t(0));
  for_each_gradient<T>(raw, dims, B, ov, clamp, [&](T v, double l) {
    uint64_t g = 0;
    if (gmax > 0) g = std::min<uint64_t>(255, uint64_t(l / gmax * 255.0f));
    uint64_t vb = (max_nonzero <= double(value_bins - 1))
                      ? uint64_t(v)
                      : uint64_t(double(v) * double(value_bins - 1) / max_nonzero);
    if (vb > value_bins - 1) vb = value_bins - 1;
    hist[vb * 256 + g]++;
  });
  return gmax;
}
}  // namespace

extern "C" double orc_histogram2d(const void* raw, int dtype, const uint64_t dims[3],
                                  const uint32_t brick_size[3], uint32_t overlap,
                                  int clamp_to_edge, uint64_t value_bins, double max_nonzero,
                                  uint64_t* hist) {
  if (dtype == 0)
    return histogram2d<uint8_t>(as<uint8_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                                value_bins, max_nonzero, hist);
  return histogram2d<uint16_t>(as<uint16_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                               value_bins, max_nonzero, hist);
}

extern "C" double orc_max_gradient(const void* raw, int dtype, const uint64_t dims[3],
                                   const uint32_t brick_size[3], uint32_t overlap,
                                   int clamp_to_edge) {
  if (dtype == 0)
    return max_gradient<uint8_t>(as<uint8_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0);
  return max_gradient<uint16_t>(as<uint16_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0);
}

// ---------------------------------------------------------------- LOD hierarchy

namespace {

template <class T>
void order2(T& a, T& b) { if (a > b) std::swap(a, b); }

// VolumeTools.h:196-210: median of a, b, c (d ignored) or the mean of four
template <class T>
T filter4(T a, T b, T c, T d, bool median) {
  if (median) {
    order2(a, b);
    order2(b, c);
    return std::max(a, b);
  }
  return T((double(a) + double(b) + double(c) + double(d)) / double(4));
}

template <class T>
T filter2(T a, T b, bool median) {
  if (median) return a;
  return T((double(a) + double(b)) / double(2));
}

template <class T>
void insert4(T& a, T& b, T& c, T& d, T& p) {
  // VolumeTools.h:212-227 InsertIntoQuadruple
  if (p > c) {
    order2(d, p);
  } else {
    if (p < b) {
      d = c;
      c = b;
      b = p;
      order2(a, b);
    } else {
      d = c;
      c = p;
    }
  }
}

template <class T>
T filter8(T a, T b, T c, T d, T e, T f, T g, T h, bool median) {
  // VolumeTools.h:242-262: 7-value median network, or the mean of eight
  if (median) {
    order2(a, b);
    order2(c, d);
    order2(a, c);
    order2(b, d);
    order2(b, c);
    insert4(a, b, c, d, e);
    insert4(a, b, c, d, f);
    return std::max(std::min(d, g), c);
  }
  return T((double(a) + double(b) + double(c) + double(d) + double(e) + double(f) + double(g) +
            double(h)) / double(8));
}

struct Tree {
  uint64_t dims[3];
  uint32_t B[3];
  uint32_t ov;
  std::vector<std::array<uint64_t, 3>> lod_size, lod_cnt;
  std::vector<uint64_t> lod_first;  // TOC index of each LOD's first brick
  std::vector<uint64_t> off;        // voxel offset per TOC index
  std::array<uint64_t, 3> size(uint64_t l, uint64_t x, uint64_t y, uint64_t z) const {
    uint64_t ls[3] = {lod_size[l][0], lod_size[l][1], lod_size[l][2]};
    uint64_t lc[3] = {lod_cnt[l][0], lod_cnt[l][1], lod_cnt[l][2]};
    uint64_t c[3] = {x, y, z}, o[3];
    orc_brick_size(ls, lc, B, ov, c, o);
    return {o[0], o[1], o[2]};
  }
  uint64_t index(uint64_t l, uint64_t x, uint64_t y, uint64_t z) const {
    return lod_first[l] + x + y * lod_cnt[l][0] + z * lod_cnt[l][0] * lod_cnt[l][1];
  }
};

// DownsampleBricktoBrick (.inc:1-248): one child brick into the target.
template <class T>
void downsample_child(const Tree& t, T* target, const std::array<uint64_t, 3>& ts,
                      const T* src, const std::array<uint64_t, 3>& ss, const uint64_t toff[3],
                      bool median) {
  const uint64_t ov = t.ov;
  const uint64_t ex = (ss[0] - 2 * ov) / 2, ey = (ss[1] - 2 * ov) / 2, ez = (ss[2] - 2 * ov) / 2;
  const bool odx = ss[0] % 2, ody = ss[1] % 2, odz = ss[2] % 2;
  auto S = [&](uint64_t x, uint64_t y, uint64_t z) -> T {
    return src[x + y * ss[0] + z * ss[0] * ss[1]];
  };
  auto D = [&](uint64_t x, uint64_t y, uint64_t z) -> T& {
    return target[(x + ov + toff[0]) + (y + ov + toff[1]) * ts[0] +
                  (z + ov + toff[2]) * ts[0] * ts[1]];
  };
  for (uint64_t z = 0; z < ez; ++z)
    for (uint64_t y = 0; y < ey; ++y)
      for (uint64_t x = 0; x < ex; ++x) {
        const uint64_t X = 2 * x + ov, Y = 2 * y + ov, Z = 2 * z + ov;
        D(x, y, z) = filter8<T>(S(X, Y, Z), S(X, Y, Z + 1), S(X, Y + 1, Z), S(X, Y + 1, Z + 1),
                                S(X + 1, Y, Z), S(X + 1, Y, Z + 1), S(X + 1, Y + 1, Z),
                                S(X + 1, Y + 1, Z + 1), median);
      }
  if (odx)
    for (uint64_t z = 0; z < ez; ++z)
      for (uint64_t y = 0; y < ey; ++y) {
        const uint64_t X = 2 * ex + ov, Y = 2 * y + ov, Z = 2 * z + ov;
        D(ex, y, z) = filter4<T>(S(X, Y, Z), S(X, Y, Z + 1), S(X, Y + 1, Z), S(X, Y + 1, Z + 1),
                                 median);
      }
  if (ody)
    for (uint64_t z = 0; z < ez; ++z)
      for (uint64_t x = 0; x < ex; ++x) {
        const uint64_t X = 2 * x + ov, Y = 2 * ey + ov, Z = 2 * z + ov;
        D(x, ey, z) = filter4<T>(S(X, Y, Z), S(X, Y, Z + 1), S(X + 1, Y, Z), S(X + 1, Y, Z + 1),
                                 median);
      }
  if (odz)
    for (uint64_t y = 0; y < ey; ++y)
      for (uint64_t x = 0; x < ex; ++x) {
        const uint64_t X = 2 * x + ov, Y = 2 * y + ov, Z = 2 * ez + ov;
        D(x, y, ez) = filter4<T>(S(X, Y, Z), S(X, Y + 1, Z), S(X + 1, Y, Z), S(X + 1, Y + 1, Z),
                                 median);
      }
  if (odx && ody)
    for (uint64_t z = 0; z < ez; ++z) {
      const uint64_t X = 2 * ex + ov, Y = 2 * ey + ov, Z = 2 * z + ov;
      D(ex, ey, z) = filter2<T>(S(X, Y, Z), S(X, Y, Z + 1), median);
    }
  if (ody && odz)
    for (uint64_t x = 0; x < ex; ++x) {
      const uint64_t X = 2 * x + ov, Y = 2 * ey + ov, Z = 2 * ez + ov;
      D(x, ey, ez) = filter2<T>(S(X, Y, Z), S(X + 1, Y, Z), median);
    }
  if (odx && odz)
    for (uint64_t y = 0; y < ey; ++y) {
      const uint64_t X = 2 * ex + ov, Y = 2 * y + ov, Z = 2 * ez + ov;
      D(ex, y, ez) = filter2<T>(S(X, Y, Z), S(X, Y + 1, Z), median);
    }
  if (odx && ody && odz) D(ex, ey, ez) = S(2 * ex + ov, 2 * ey + ov, 2 * ez + ov);
}

// CopyBrickToBrick (.cpp:1153-1202)
template <class T>
void copy_region(const T* src, const std::array<uint64_t, 3>& ss, T* dst,
                 const std::array<uint64_t, 3>& ds, const uint64_t so[3], const uint64_t dof[3],
                 const uint64_t r[3]) {
  for (uint64_t z = 0; z < r[2]; ++z)
    for (uint64_t y = 0; y < r[1]; ++y)
      for (uint64_t x = 0; x < r[0]; ++x)
        dst[(dof[0] + x) + (dof[1] + y) * ds[0] + (dof[2] + z) * ds[0] * ds[1]] =
            src[(so[0] + x) + (so[1] + y) * ss[0] + (so[2] + z) * ss[0] * ss[1]];
}

template <class T>
void clamp_brick(T* d, const std::array<uint64_t, 3>& bs, uint64_t ov, const bool s[3],
                 const bool e[3]) {
  // ClampToEdge (.cpp:376-462), same order as for LOD 0
  auto at = [&](uint64_t x, uint64_t y, uint64_t z) -> T& {
    return d[x + y * bs[0] + z * bs[0] * bs[1]];
  };
  if (s[0])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t y = 0; y < bs[1]; ++y)
        for (uint64_t o = 0; o < ov; ++o) at(ov - 1 - o, y, z) = at(ov, y, z);
  if (e[0])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t y = 0; y < bs[1]; ++y)
        for (uint64_t o = 0; o < ov; ++o) at(bs[0] - ov + o, y, z) = at(bs[0] - 1 - ov, y, z);
  if (s[1])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, ov - 1 - o, z) = at(x, ov, z);
  if (e[1])
    for (uint64_t z = 0; z < bs[2]; ++z)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, bs[1] - ov + o, z) = at(x, bs[1] - 1 - ov, z);
  if (s[2])
    for (uint64_t y = 0; y < bs[1]; ++y)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, y, ov - 1 - o) = at(x, y, ov);
  if (e[2])
    for (uint64_t y = 0; y < bs[1]; ++y)
      for (uint64_t o = 0; o < ov; ++o)
        for (uint64_t x = 0; x < bs[0]; ++x) at(x, y, bs[2] - ov + o) = at(x, y, bs[2] - 1 - ov);
}

// FillOverlap (.cpp:1203-1372) for one LOD, bricks in z, y, x order
template <class T>
void fill_overlap(const Tree& t, T* pool, uint64_t l, bool clamp) {
  const uint64_t ov = t.ov;
  const auto& cnt = t.lod_cnt[l];
  for (uint64_t z = 0; z < cnt[2]; ++z)
    for (uint64_t y = 0; y < cnt[1]; ++y)
      for (uint64_t x = 0; x < cnt[0]; ++x) {
        const bool lf = x > 0, rt = x < cnt[0] - 1, tp = y > 0, bt = y < cnt[1] - 1;
        const bool fr = z > 0, bk = z < cnt[2] - 1;
        const auto ts = t.size(l, x, y, z);
        T* dst = pool + t.off[t.index(l, x, y, z)];
        auto copy = [&](int64_t dx, int64_t dy, int64_t dz, uint64_t sx0, uint64_t sy0,
                        uint64_t sz0, uint64_t dx0, uint64_t dy0, uint64_t dz0, uint64_t rx,
                        uint64_t ry, uint64_t rz) {
          const uint64_t nx = x + dx, ny = y + dy, nz = z + dz;
          const auto ss = t.size(l, nx, ny, nz);
          const T* src = pool + t.off[t.index(l, nx, ny, nz)];
          const uint64_t so[3] = {sx0, sy0, sz0}, dof[3] = {dx0, dy0, dz0};
          const uint64_t r[3] = {rx == ~0ull ? ss[0] : rx, ry == ~0ull ? ss[1] : ry,
                                 rz == ~0ull ? ss[2] : rz};
          copy_region<T>(src, ss, dst, ts, so, dof, r);
        };
        const uint64_t A = ~0ull;
        if (rt) copy(1, 0, 0, ov, 0, 0, ts[0] - ov, 0, 0, ov, A, A);
        if (bt) copy(0, 1, 0, 0, ov, 0, 0, ts[1] - ov, 0, A, ov, A);
        if (bk) copy(0, 0, 1, 0, 0, ov, 0, 0, ts[2] - ov, A, A, ov);
        if (lf) copy(-1, 0, 0, t.size(l, x - 1, y, z)[0] - 2 * ov, 0, 0, 0, 0, 0, ov, A, A);
        if (tp) copy(0, -1, 0, 0, t.size(l, x, y - 1, z)[1] - 2 * ov, 0, 0, 0, 0, A, ov, A);
        if (fr) copy(0, 0, -1, 0, 0, t.size(l, x, y, z - 1)[2] - 2 * ov, 0, 0, 0, A, A, ov);
        if (bt && rt) copy(1, 1, 0, ov, ov, 0, ts[0] - ov, ts[1] - ov, 0, ov, ov, A);
        if (rt && bk) copy(1, 0, 1, ov, 0, ov, ts[0] - ov, 0, ts[2] - ov, ov, A, ov);
        if (bt && bk) copy(0, 1, 1, 0, ov, ov, 0, ts[1] - ov, ts[2] - ov, A, ov, ov);
        if (rt && bt && bk) copy(1, 1, 1, ov, ov, ov, ts[0] - ov, ts[1] - ov, ts[2] - ov, ov, ov, ov);
        if (clamp) {
          const bool s[3] = {!lf, !tp, !fr}, e[3] = {!rt, !bt, !bk};
          clamp_brick<T>(dst, ts, ov, s, e);
        }
      }
}

template <class T>
int64_t build_octree(const T* raw, const uint64_t dims[3], const uint32_t B[3], uint32_t ov,
                     bool clamp, bool median, T* pool, uint64_t pool_voxels, uint64_t* offsets,
                     uint64_t max_bricks) {
  Tree t;
  for (int a = 0; a < 3; ++a) {
    t.dims[a] = dims[a];
    t.B[a] = B[a];
  }
  t.ov = ov;
  uint64_t ls[3 * 64], lc[3 * 64];
  const int nl = orc_lod_table(dims, B, ov, ls, lc, 64);
  uint64_t n = 0, vox = 0;
  for (int l = 0; l < nl; ++l) {
    t.lod_size.push_back({ls[3 * l], ls[3 * l + 1], ls[3 * l + 2]});
    t.lod_cnt.push_back({lc[3 * l], lc[3 * l + 1], lc[3 * l + 2]});
    t.lod_first.push_back(n);
    for (uint64_t z = 0; z < lc[3 * l + 2]; ++z)
      for (uint64_t y = 0; y < lc[3 * l + 1]; ++y)
        for (uint64_t x = 0; x < lc[3 * l]; ++x) {
          const auto s = t.size(l, x, y, z);
          t.off.push_back(vox);
          vox += s[0] * s[1] * s[2];
          ++n;
        }
  }
  if (n > max_bricks || vox > pool_voxels) return -1;
  std::fill(pool, pool + vox, T(0));
  for (uint64_t i = 0; i < n; ++i) offsets[i] = t.off[i];
  // LOD 0 (PermuteInputData)
  for (uint64_t z = 0; z < lc[2]; ++z)
    for (uint64_t y = 0; y < lc[1]; ++y)
      for (uint64_t x = 0; x < lc[0]; ++x) {
        const uint64_t c[3] = {x, y, z};
        lod0_brick<T>(raw, dims, B, ov, clamp, c, pool + t.off[t.index(0, x, y, z)]);
      }
  // ComputeHierarchy (.inc:358-398)
  const uint64_t split[3] = {uint64_t(std::ceil((B[0] - 2.0 * ov) / 2.0)),
                             uint64_t(std::ceil((B[1] - 2.0 * ov) / 2.0)),
                             uint64_t(std::ceil((B[2] - 2.0 * ov) / 2.0))};
  for (int l = 1; l < nl; ++l) {
    const auto& cnt = t.lod_cnt[l];
    const auto& lower = t.lod_cnt[l - 1];
    for (uint64_t z = 0; z < cnt[2]; ++z)
      for (uint64_t y = 0; y < cnt[1]; ++y)
        for (uint64_t x = 0; x < cnt[0]; ++x) {
          const auto ts = t.size(l, x, y, z);
          T* dst = pool + t.off[t.index(l, x, y, z)];
          const bool hr = x * 2 + 1 < lower[0], hb = y * 2 + 1 < lower[1], hk = z * 2 + 1 < lower[2];
          for (int k = 0; k < 8; ++k) {
            const uint64_t cx = k & 1, cy = (k >> 1) & 1, cz = (k >> 2) & 1;
            if ((cx && !hr) || (cy && !hb) || (cz && !hk)) continue;
            const uint64_t toff[3] = {cx ? split[0] : 0, cy ? split[1] : 0, cz ? split[2] : 0};
            const uint64_t sx = 2 * x + cx, sy = 2 * y + cy, sz = 2 * z + cz;
            downsample_child<T>(t, dst, ts, pool + t.off[t.index(l - 1, sx, sy, sz)],
                                t.size(l - 1, sx, sy, sz), toff, median);
          }
        }
    fill_overlap<T>(t, pool, l, clamp);
  }
  return int64_t(n);
}

}  // namespace

extern "C" int64_t orc_build_octree(const void* raw, int dtype, const uint64_t dims[3],
                                    const uint32_t brick_size[3], uint32_t overlap,
                                    int clamp_to_edge, int median, void* pool,
                                    uint64_t pool_voxels, uint64_t* brick_offsets,
                                    uint64_t max_bricks) {
  if (dtype == 2) {
    // RGBA8: every step filters or copies each component on its own
    // (ExtendedOctreeConverter.inc:39-44), so the octree is the four
    // single-channel octrees interleaved
    const uint64_t n = dims[0] * dims[1] * dims[2];
    std::vector<uint8_t> chan(n), part(pool_voxels);
    uint8_t* out = static_cast<uint8_t*>(pool);
    int64_t bricks = -1;
    for (int c = 0; c < 4; ++c) {
      for (uint64_t i = 0; i < n; ++i) chan[i] = as<uint8_t>(raw)[4 * i + uint64_t(c)];
      bricks = build_octree<uint8_t>(chan.data(), dims, brick_size, overlap, clamp_to_edge != 0,
                                     median != 0, part.data(), pool_voxels, brick_offsets,
                                     max_bricks);
      if (bricks < 0) return bricks;
      for (uint64_t i = 0; i < pool_voxels; ++i) out[4 * i + uint64_t(c)] = part[i];
    }
    return bricks;
  }
  if (dtype == 0)
    return build_octree<uint8_t>(as<uint8_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                                 median != 0, static_cast<uint8_t*>(pool), pool_voxels,
                                 brick_offsets, max_bricks);
  return build_octree<uint16_t>(as<uint16_t>(raw), dims, brick_size, overlap, clamp_to_edge != 0,
                                median != 0, static_cast<uint16_t*>(pool), pool_voxels,
                                brick_offsets, max_bricks);
}

// The CPU bricking baseline: the serial work of ExtendedOctreeConverter::Convert
// (ExtendedOctreeConverter.cpp:128-280) restated -- every brick of every LOD
// with its ghost voxels (the octree above), ComputeBrickStats per brick
// (.inc:408-444) -- plus the 1D histogram of Histogram1DDataBlock
// (Histogram1DDataBlock.cpp:120-161), on one thread, timed without file IO.
// Returns the bricks built (negative on failure); *seconds = wall time.
extern "C" int64_t orc_convert_timed(const void* raw, int dtype, const uint64_t dims[3],
                                     const uint32_t brick_size[3], uint32_t overlap,
                                     int clamp_to_edge, double* seconds,
                                     uint64_t* pool_bytes_out) {
  if (dtype != 0 && dtype != 1) return -1;
  const size_t bytes = dtype == 0 ? 1 : 2;
  uint64_t lod[3 * 64], cnt[3 * 64];
  const int n_lods = orc_lod_table(dims, brick_size, overlap, lod, cnt, 64);
  uint64_t n_bricks = 0, total = 0;
  for (int l = 0; l < n_lods; ++l)
    for (uint64_t z = 0; z < cnt[3 * l + 2]; ++z)
      for (uint64_t y = 0; y < cnt[3 * l + 1]; ++y)
        for (uint64_t x = 0; x < cnt[3 * l]; ++x) {
          const uint64_t c[3] = {x, y, z};
          uint64_t bs[3];
          orc_brick_size(&lod[3 * l], &cnt[3 * l], brick_size, overlap, c, bs);
          total += bs[0] * bs[1] * bs[2];
          ++n_bricks;
        }
  std::vector<uint8_t> pool(total * bytes);
  std::vector<uint64_t> off(n_bricks);
  std::vector<uint64_t> hist(size_t(1) << (8 * bytes));
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = orc_build_octree(raw, dtype, dims, brick_size, overlap, clamp_to_edge, 0,
                                     pool.data(), total, off.data(), n_bricks);
  if (n < 0) return n;
  double acc = 0.0;
  for (uint64_t b = 0; b < n_bricks; ++b) {
    const uint64_t end = b + 1 < n_bricks ? off[b + 1] : total;
    double mn, mx;
    orc_brick_stats(pool.data() + off[b] * bytes, dtype, end - off[b], &mn, &mx);
    acc += mn + mx;
  }
  orc_histogram1d(raw, dtype, dims, brick_size, overlap, hist.data());
  const auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count() + (acc < 0 ? 1 : 0);
  if (pool_bytes_out) *pool_bytes_out = total * bytes;
  return n;
}
