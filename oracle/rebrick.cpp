// rebrick.cpp -- CPU restatement of the reference's DynamicBrickingDS
// (IO/DynamicBrickingDS.cpp) and minmax_brick (IO/BMinMax.cpp:8-47).
//
// TEST INFRASTRUCTURE ONLY: the tests check the GPU rebricking against it.
//
// The source dataset is an ExtendedOctree brick pool as orc_build_octree writes
// it (every built LOD in TOC order).  DynamicBrickingDS re-cuts it into bricks of
// a requested size (ghost voxels included) that must divide the source bricks:
//   * Rebrick (:1090-1180) checks integer_multiple (:963-971) per axis and lists
//     the target bricks of every source LOD, laid out with the real ghost width
//     (dbinfo::BrickSansGhost :218-223, GenericBrickLayout :226-239);
//   * ComputedTargetBrickSize (:414-434), SourceBrickIndex (:272-303),
//     OffsetIntoSource (:305-335) and BrickMetadata (:1034-1088) use the static
//     BrickSansGhost (:208-217), which subtracts a hard-coded 4;
//   * Brick/CopyBrick (:495-538, :566-620) copy tgt_bs[0]-long scanlines from the
//     source brick at the offset, with linear source indexing (a scanline that
//     runs past the source's x extent continues on the next line);
//   * MaxMinForKey (:862-875): MM_SOURCE = the source brick's min/max,
//     MM_DYNAMIC / MM_PRECOMPUTE = std::minmax_element over the copied brick
//     (GetBrick resizes the buffer to the brick, so nothing else enters).
// The layout helpers divide in float (layout :113-121) and the metadata lerps
// mix float and double exactly as MathTools::lerp (Basics/MathTools.h:79-92).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "oracle.h"

namespace {

using U3 = std::array<uint64_t, 3>;

// layout(): static_cast<float>(voxels) / bsize, then ceil
U3 layout_f(const U3& voxels, const U3& bs) {
  U3 r;
  for (int a = 0; a < 3; ++a)
    r[a] = uint64_t(std::ceil(static_cast<float>(voxels[a]) / float(bs[a])));
  return r;
}

U3 sans_static(U3 b) {
  for (int a = 0; a < 3; ++a) b[a] = b[a] > 4 ? b[a] - 4 : b[a];
  return b;
}

// integer_multiple(a, b): b == a * i for some i < 128
bool integer_multiple(uint64_t a, uint64_t b) {
  for (uint64_t i = 0; i < 128; ++i)
    if (a * i == b) return true;
  return false;
}

template <class In>
float lerp_ref(In value, In imin, In imax, float omin, float omax) {
  return float(omin + (value - imin) * (static_cast<double>(omax - omin) / (imax - imin)));
}

template <class T>
int64_t rebrick(const uint64_t dims[3], const uint32_t src_brick[3], uint32_t ov,
                uint32_t n_built, const T* src_pool, const uint64_t* src_offsets,
                const double* src_min, const double* src_max, const uint32_t tgt_brick[3],
                int mm_mode, uint64_t max_out, uint32_t* info, float* geom, uint64_t* src_index,
                double* mm, T* out_pool, uint64_t pool_cap, uint64_t* out_offsets,
                uint64_t* pool_needed) {
  const uint64_t ghost = 2ull * ov;
  const U3 B = {tgt_brick[0], tgt_brick[1], tgt_brick[2]};
  // SourceMaxBrickSize: the converter's brick size minus the ghost width
  const U3 src_bs = {src_brick[0] - ghost, src_brick[1] - ghost, src_brick[2] - ghost};
  for (int a = 0; a < 3; ++a) {
    if (B[a] <= ghost) return -1;
    if (!integer_multiple(B[a] - ghost, src_bs[a])) return -1;  // std::runtime_error
  }
  uint64_t lsz[3 * 64], lcnt[3 * 64];
  const int n_lods = orc_lod_table(dims, src_brick, ov, lsz, lcnt, 64);
  const int lods = std::min<int>(n_lods, int(n_built));
  double asp_single[3];
  // source TOC index of each LOD's first brick
  std::vector<uint64_t> src_first(n_lods + 1, 0);
  for (int l = 0; l < n_lods; ++l)
    src_first[l + 1] = src_first[l] + lcnt[3 * l] * lcnt[3 * l + 1] * lcnt[3 * l + 2];

  // DatasetExtents (:993-1014): brick 0 of the first LOD with a single brick
  int single = 0;
  for (int l = 0; l < n_lods; ++l)
    if (lcnt[3 * l] * lcnt[3 * l + 1] * lcnt[3 * l + 2] == 1) { single = l; break; }
  float ext_full[3];
  {
    float c[3], e[3];
    uint32_t n[3];
    orc_lod_aspect(dims, uint32_t(single), asp_single);
    orc_brick_metadata(&lsz[3 * single], &lcnt[3 * single], src_brick, ov, asp_single, c, e, n);
    for (int a = 0; a < 3; ++a) ext_full[a] = e[a];
  }
  const float elow[3] = {-(ext_full[0] / 2.0f), -(ext_full[1] / 2.0f), -(ext_full[2] / 2.0f)};
  const float ehigh[3] = {ext_full[0] / 2.0f, ext_full[1] / 2.0f, ext_full[2] / 2.0f};

  const U3 real_sans = {B[0] - ghost, B[1] - ghost, B[2] - ghost};
  const U3 ssans = sans_static(B);
  uint64_t count = 0, need = 0;
  for (int l = 0; l < lods; ++l) {
    const U3 vox = {lsz[3 * l], lsz[3 * l + 1], lsz[3 * l + 2]};
    const U3 bl = layout_f(vox, real_sans);   // Rebrick's loop bounds
    const U3 bls = layout_f(vox, ssans);      // ComputedTargetBrickSize / SourceBrickIndex
    const U3 src_lay = layout_f(vox, src_bs); // SourceKey
    for (uint64_t idx = 0; idx < bl[0] * bl[1] * bl[2]; ++idx) {
      const U3 bi = {idx % bl[0], (idx / bl[0]) % bl[1], idx / (bl[0] * bl[1])};
      U3 cur;
      for (int a = 0; a < 3; ++a) {
        const bool last = bi[a] == bls[a] - 1;
        const uint64_t extra = vox[a] % ssans[a];
        cur[a] = (last && extra) ? 4 + extra : B[a];
      }
      // source brick and offset (SourceBrickIndex / OffsetIntoSource / SourceKey)
      if (idx >= bls[0] * bls[1] * bls[2]) return -2;
      const U3 i3 = {idx % bls[0], (idx / bls[0]) % bls[1], idx / (bls[0] * bls[1])};
      U3 bps, sidx, off;
      for (int a = 0; a < 3; ++a) {
        bps[a] = src_bs[a] / ssans[a];
        if (bps[a] == 0) return -2;
        sidx[a] = i3[a] / bps[a];
        off[a] = (i3[a] % bps[a]) * ssans[a];
        if (sidx[a] >= src_lay[a] || sidx[a] >= lcnt[3 * l + a]) return -2;
      }
      const uint64_t sk = sidx[0] + sidx[1] * src_lay[0] + sidx[2] * src_lay[0] * src_lay[1];
      uint64_t sbs[3];
      orc_brick_size(&lsz[3 * l], &lcnt[3 * l], src_brick, ov, sidx.data(), sbs);
      // the copy reads src[(off.z+z)*sx*sy + (off.y+y)*sx + off.x + x]; past the
      // source buffer the reference reads outside its vector
      const uint64_t last_read = (off[2] + cur[2] - 1) * sbs[0] * sbs[1] +
                                 (off[1] + cur[1] - 1) * sbs[0] + off[0] + cur[0] - 1;
      if (last_read >= sbs[0] * sbs[1] * sbs[2]) return -2;

      const uint64_t nv = cur[0] * cur[1] * cur[2];
      if (count < max_out && need + nv <= pool_cap) {
        const uint64_t t = count;
        info[4 * t + 0] = uint32_t(l);
        for (int a = 0; a < 3; ++a) info[4 * t + 1 + a] = uint32_t(cur[a]);
        // BrickMetadata with size = BrickSansGhost(cur), bsize = BrickSansGhost(B)
        const U3 size = sans_static(cur);
        for (int a = 0; a < 3; ++a) {
          const uint64_t lo = bi[a] * ssans[a];
          const uint64_t hi = lo + size[a];
          const float vc = ((hi - lo) / 2.0f) + lo;
          const float vf = static_cast<float>(vox[a]);
          geom[6 * t + a] = lerp_ref<float>(vc, 0.0f, vf, elow[a], ehigh[a]);
          const float wl = lerp_ref<uint64_t>(lo, 0ull, vox[a], elow[a], ehigh[a]);
          const float wh = lerp_ref<uint64_t>(hi, 0ull, vox[a], elow[a], ehigh[a]);
          geom[6 * t + 3 + a] = wh - wl;
        }
        const uint64_t s_toc = src_first[l] + sk;
        src_index[t] = s_toc;
        out_offsets[t] = need;
        const T* s = src_pool + src_offsets[s_toc];
        T* d = out_pool + need;
        for (uint64_t z = 0; z < cur[2]; ++z)
          for (uint64_t y = 0; y < cur[1]; ++y) {
            const uint64_t so = (off[2] + z) * sbs[0] * sbs[1] + (off[1] + y) * sbs[0] + off[0];
            std::copy(s + so, s + so + cur[0], d + (z * cur[1] + y) * cur[0]);
          }
        if (mm_mode == 0) {  // MM_SOURCE
          mm[2 * t] = src_min[s_toc];
          mm[2 * t + 1] = src_max[s_toc];
        } else {             // MM_DYNAMIC / MM_PRECOMPUTE: minmax_brick
          const auto r = std::minmax_element(d, d + nv);
          mm[2 * t] = double(*r.first);
          mm[2 * t + 1] = double(*r.second);
        }
      }
      ++count;
      need += nv;
    }
  }
  *pool_needed = need;
  return int64_t(count);
}

}  // namespace

extern "C" int64_t orc_rebrick(int dtype, const uint64_t dims[3], const uint32_t src_brick[3],
                               uint32_t overlap, uint32_t n_built_lods, const void* src_pool,
                               const uint64_t* src_offsets, const double* src_min,
                               const double* src_max, const uint32_t tgt_brick[3], int mm_mode,
                               uint64_t max_out, uint32_t* info, float* geom,
                               uint64_t* src_index, double* minmax, void* out_pool,
                               uint64_t pool_cap, uint64_t* out_offsets, uint64_t* pool_needed) {
  if (dtype == 0)
    return rebrick<uint8_t>(dims, src_brick, overlap, n_built_lods,
                            static_cast<const uint8_t*>(src_pool), src_offsets, src_min, src_max,
                            tgt_brick, mm_mode, max_out, info, geom, src_index, minmax,
                            static_cast<uint8_t*>(out_pool), pool_cap, out_offsets, pool_needed);
  return rebrick<uint16_t>(dims, src_brick, overlap, n_built_lods,
                           static_cast<const uint16_t*>(src_pool), src_offsets, src_min, src_max,
                           tgt_brick, mm_mode, max_out, info, geom, src_index, minmax,
                           static_cast<uint16_t*>(out_pool), pool_cap, out_offsets, pool_needed);
}
