// volgen.cpp -- host restatement of tuvok_gb300's seeded volume generator
// (tvk_generate_volume), so that a CPU-only program (the reference arm of the
// benchmark) renders the very bytes the GPU run renders, and a digest of the
// bytes that both record.
//
// TEST INFRASTRUCTURE ONLY (input creation for the CPU baseline and the
// reference arm; the checks that GPU and host generate the same volume).
//
// value(x,y,z) = sum over blobs b (in order) of peak_b * ((ex_b(x) * ey_b(y)) * ez_b(z))
//                for ((qx_b(x) + qy_b(y)) + qz_b(z)) < 32 sigma_b^2
//              + value noise or integer noise, floor(v + 1/2), clamped to [0, vmax],
// with q_b(i) = (i - c_b)^2 and e_b(i) = exp(-q_b(i) / (2 sigma_b^2)) per axis
// (the exponential in double from its Taylor series, no libm), every other
// step a plain float or integer operation in a fixed order.  Built with
// -ffp-contract=off, so no multiply-add is fused.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

inline uint64_t hash4(uint64_t seed, uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
  uint64_t h = mix64(seed + 0x9e3779b97f4a7c15ull);
  h = mix64(h ^ (a + 0x9e3779b97f4a7c15ull));
  h = mix64(h ^ (b + 0x632be59bd9b4e019ull));
  h = mix64(h ^ (c + 0x85157af5ull));
  return mix64(h ^ d);
}

inline float lattice(uint64_t seed, uint32_t oct, int64_t x, int64_t y, int64_t z) {
  const uint64_t h = hash4(seed, uint64_t(x), uint64_t(y), uint64_t(z), oct);
  return float(h >> 40) * (2.0f / 16777216.0f) - 1.0f;
}

// e^x, x <= 0: k = floor(x / ln 2 + 1/2), r = x - k ln 2, Taylor series of
// e^r to r^11, times 2^k.
double exp_nonpositive(double x) {
  if (!(x > -700.0)) return 0.0;
  const double k = std::floor(x * 1.4426950408889634 + 0.5);
  const double r = x - k * 0.69314718055994531;
  const double c[12] = {1.0 / 39916800.0, 1.0 / 3628800.0, 1.0 / 362880.0, 1.0 / 40320.0,
                        1.0 / 5040.0,     1.0 / 720.0,     1.0 / 120.0,    1.0 / 24.0,
                        1.0 / 6.0,        0.5,             1.0,            1.0};
  double p = c[0];
  for (int i = 1; i < 12; ++i) p = std::fma(p, r, c[i]);
  const uint64_t bits = uint64_t(int64_t(k) + 1023) << 52;
  double two_k;
  std::memcpy(&two_k, &bits, sizeof two_k);
  return p * two_k;
}

template <class T>
void generate(T* out, const uint64_t dims[3], const float* blobs, uint32_t nb, float amp,
              uint32_t octaves, float cell, uint64_t seed, int int_noise, float vmax,
              int threads) {
  const uint64_t nx = dims[0], ny = dims[1], nz = dims[2];
  std::vector<float> q[3], e[3], lim(nb), pk(nb);
  for (int a = 0; a < 3; ++a) {
    q[a].resize(size_t(nb) * dims[a]);
    e[a].resize(q[a].size());
  }
  for (uint32_t b = 0; b < nb; ++b) {
    const float* B = blobs + 7 * size_t(b);
    const float s2 = B[3] * B[3];
    lim[b] = 32.0f * s2;
    pk[b] = B[4];
    const double den = 2.0 * double(s2);
    for (int a = 0; a < 3; ++a)
      for (uint64_t i = 0; i < dims[a]; ++i) {
        const float d = float(i) - B[a];
        const float qq = d * d;
        q[a][size_t(b) * dims[a] + i] = qq;
        e[a][size_t(b) * dims[a] + i] = float(exp_nonpositive(-double(qq) / den));
      }
  }
  // value noise: per axis and octave the smoothstep weight and lattice index,
  // and per octave the lattice values over the index range the volume uses
  std::vector<float> sm[3];
  std::vector<int64_t> ix[3];
  std::vector<float> lat;
  std::vector<size_t> lat_off(octaves + 1, 0);
  std::vector<int64_t> lat_n(3 * size_t(octaves), 0);
  float nscale = 0.0f;
  if (!int_noise && octaves > 0) {
    float wsum = 0.0f;
    for (uint32_t k = 0; k < octaves; ++k) wsum = wsum + std::ldexp(1.0f, -int(k));
    nscale = amp / wsum;
    for (int a = 0; a < 3; ++a) {
      sm[a].resize(size_t(octaves) * dims[a]);
      ix[a].resize(sm[a].size());
    }
    float c = cell;
    for (uint32_t k = 0; k < octaves; ++k, c = c * 0.5f) {
      for (int a = 0; a < 3; ++a) {
        int64_t mx = 0;
        for (uint64_t i = 0; i < dims[a]; ++i) {
          const float g = float(i) / c;
          const float f = std::floor(g);
          const float t = g - f;
          sm[a][size_t(k) * dims[a] + i] = (t * t) * (3.0f - 2.0f * t);
          ix[a][size_t(k) * dims[a] + i] = int64_t(f);
          mx = std::max(mx, int64_t(f));
        }
        lat_n[3 * k + a] = mx + 2;
      }
      lat_off[k + 1] = lat_off[k] + size_t(lat_n[3 * k]) * lat_n[3 * k + 1] * lat_n[3 * k + 2];
    }
    lat.resize(lat_off[octaves]);
    for (uint32_t k = 0; k < octaves; ++k) {
      const int64_t Lx = lat_n[3 * k], Ly = lat_n[3 * k + 1], Lz = lat_n[3 * k + 2];
#pragma omp parallel for num_threads(threads > 0 ? threads : omp_get_max_threads()) schedule(static)
      for (int64_t Z = 0; Z < Lz; ++Z)
        for (int64_t Y = 0; Y < Ly; ++Y)
          for (int64_t X = 0; X < Lx; ++X)
            lat[lat_off[k] + size_t((Z * Ly + Y) * Lx + X)] = lattice(seed, k, X, Y, Z);
    }
  }
  const int64_t rows = int64_t(ny * nz);
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads())
  {
    std::vector<float> v(nx);
#pragma omp for schedule(dynamic, 16)
    for (int64_t row = 0; row < rows; ++row) {
      const uint64_t y = uint64_t(row) % ny, z = uint64_t(row) / ny;
      std::fill(v.begin(), v.end(), 0.0f);
      for (uint32_t b = 0; b < nb; ++b) {
        const float qy = q[1][size_t(b) * ny + y], qz = q[2][size_t(b) * nz + z];
        // the x term is >= 0: a blob whose y and z terms reach the limit adds nothing
        if (!(qy + qz < lim[b])) continue;
        const float ey = e[1][size_t(b) * ny + y], ez = e[2][size_t(b) * nz + z];
        // x range that can pass the test (its rounding is below the margin)
        const double rem = double(lim[b]) * (1.0 + 1e-6) - (double(qy) + double(qz));
        const double r = std::sqrt(std::max(rem, 0.0)) + 2.0;
        const double cx = double(blobs[7 * size_t(b)]);
        const int64_t x0 = std::max<int64_t>(0, int64_t(std::floor(cx - r)));
        const int64_t x1 = std::min<int64_t>(int64_t(nx) - 1, int64_t(std::ceil(cx + r)));
        const float* qx = &q[0][size_t(b) * nx];
        const float* ex = &e[0][size_t(b) * nx];
        for (int64_t x = x0; x <= x1; ++x) {
          const float d2 = (qx[x] + qy) + qz;
          if (d2 < lim[b]) {
            const float g = (ex[x] * ey) * ez;
            v[x] = v[x] + pk[b] * g;
          }
        }
      }
      T* dst = out + (z * ny + y) * nx;
      for (uint64_t x = 0; x < nx; ++x) {
        float val = v[x];
        if (int_noise) {
          const int64_t span = int64_t(2.0f * amp + 1.0f);
          const uint64_t h = hash4(seed, x, y, z, 0xabcdefull);
          val = val + float(int64_t(h % uint64_t(span)) - int64_t(amp));
        } else if (octaves > 0) {
          float nv = 0.0f;
          for (uint32_t k = 0; k < octaves; ++k) {
            const float sx = sm[0][size_t(k) * nx + x], sy = sm[1][size_t(k) * ny + y],
                        sz = sm[2][size_t(k) * nz + z];
            const int64_t X = ix[0][size_t(k) * nx + x], Y = ix[1][size_t(k) * ny + y],
                          Z = ix[2][size_t(k) * nz + z];
            const int64_t Lx = lat_n[3 * k], Ly = lat_n[3 * k + 1];
            const float* L = &lat[lat_off[k]];
            float acc = 0.0f;
            for (int cz = 0; cz < 2; ++cz)
              for (int cy = 0; cy < 2; ++cy)
                for (int cxx = 0; cxx < 2; ++cxx) {
                  const float w = ((cxx ? sx : 1.0f - sx) * (cy ? sy : 1.0f - sy)) *
                                  (cz ? sz : 1.0f - sz);
                  acc = acc + w * L[size_t(((Z + cz) * Ly + (Y + cy)) * Lx + (X + cxx))];
                }
            nv = nv + acc * std::ldexp(1.0f, -int(k));
          }
          val = val + nv * nscale;
        }
        val = std::floor(val + 0.5f);
        val = std::fmin(std::fmax(val, 0.0f), vmax);
        dst[x] = T(val);
      }
    }
  }
}

inline uint64_t fnv1a(const uint8_t* p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

}  // namespace

extern "C" {

// dtype 0 = u8, 1 = u16; out holds dims[0]*dims[1]*dims[2] voxels (x fastest).
// threads <= 0: all of OpenMP's threads.
int orc_generate_volume(void* out, int dtype, const uint64_t dims[3], const float* blobs,
                        uint32_t n_blobs, float noise_amp, uint32_t octaves, float cell,
                        uint64_t seed, int int_noise, float vmax, int threads) {
  if (!out || !dims || (n_blobs && !blobs) || (dtype != 0 && dtype != 1)) return -1;
  if (octaves > 0 && !(cell > 0.0f)) return -1;
  if (dtype == 0)
    generate(static_cast<uint8_t*>(out), dims, blobs, n_blobs, noise_amp, octaves, cell, seed,
             int_noise, vmax, threads);
  else
    generate(static_cast<uint16_t*>(out), dims, blobs, n_blobs, noise_amp, octaves, cell, seed,
             int_noise, vmax, threads);
  return 0;
}

// Digest of a volume's bytes: FNV-1a (64-bit) of every 1 MiB chunk, then
// FNV-1a of those digests' little-endian bytes in chunk order.
uint64_t orc_volume_hash(const void* data, uint64_t n, int threads) {
  const uint8_t* p = static_cast<const uint8_t*>(data);
  const uint64_t chunk = 1ull << 20;
  const int64_t nc = int64_t((n + chunk - 1) / chunk);
  std::vector<uint64_t> h(size_t(std::max<int64_t>(nc, 0)));
#pragma omp parallel for num_threads(threads > 0 ? threads : omp_get_max_threads()) schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    const uint64_t off = uint64_t(c) * chunk;
    h[size_t(c)] = fnv1a(p + off, size_t(std::min(chunk, n - off)));
  }
  uint64_t d = 0xcbf29ce484222325ull;
  for (uint64_t v : h) {
    uint8_t le[8];
    for (int i = 0; i < 8; ++i) le[i] = uint8_t(v >> (8 * i));
    d = fnv1a(le, 8, d);
  }
  return d;
}

}  // extern "C"
