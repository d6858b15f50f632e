// volgen.cu -- seeded synthetic volumes (input creation for tests and benchmarks).
//
// value(x,y,z) = sum over blobs b of  peak_b * ex_b(x) * ey_b(y) * ez_b(z)
//                where (x - cx_b)^2 + (y - cy_b)^2 + (z - cz_b)^2 < 32 sigma_b^2,
//              + noise(x,y,z),  rounded to nearest and clamped to [0, vmax].
// e_b(i) = exp(-(i - c_b)^2 / (2 sigma_b^2)) per axis (the Gaussian is
// separable).  Noise is either value noise (lattice values in [-1,1] from a
// 64-bit hash of (seed, octave, lattice point), smoothstep-interpolated,
// octave k at cell size cell/2^k with weight 2^-k, scaled so the weights sum
// to noise_amp) or uniform integer noise in [-noise_amp, noise_amp] from the
// hash of the voxel.
//
// The volume is a function of its parameters alone, bit for bit on any IEEE
// machine: the per-axis tables (squared distances and Gaussian factors) are
// computed here on the host in double with an exponential written out below
// (no libm), the kernel combines them in a fixed order of float operations
// (this file is built with -fmad=false), and everything else is integer
// hashing.  A host program that restates the same steps gets the same bytes.
#include <cmath>
#include <cstring>
#include <vector>

#include "tvk_internal.h"

namespace tvk {
namespace {

constexpr uint32_t kMaxBlobs = 2048;
constexpr uint32_t kGenThreads = 256;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t hash4(uint64_t seed, uint64_t a, uint64_t b, uint64_t c,
                                          uint64_t d) {
  uint64_t h = mix64(seed + 0x9e3779b97f4a7c15ull);
  h = mix64(h ^ (a + 0x9e3779b97f4a7c15ull));
  h = mix64(h ^ (b + 0x632be59bd9b4e019ull));
  h = mix64(h ^ (c + 0x85157af5ull));
  return mix64(h ^ d);
}

__device__ __forceinline__ float lattice(uint64_t seed, uint32_t oct, int64_t x, int64_t y,
                                         int64_t z) {
  const uint64_t h = hash4(seed, uint64_t(x), uint64_t(y), uint64_t(z), oct);
  return float(h >> 40) * (2.0f / 16777216.0f) - 1.0f;
}

// e^x for x <= 0 in double: x = k ln 2 + r with k = floor(x / ln 2 + 1/2),
// |r| <= ln 2 / 2, and the Taylor series of e^r to r^11 (truncation below
// 1e-14 relative), scaled by 2^k.  Every operation is a plain IEEE double
// operation, so any machine gives the same bits.
double exp_nonpositive(double x) {
  if (!(x > -700.0)) return 0.0;
  const double k = std::floor(x * 1.4426950408889634 + 0.5);
  const double r = x - k * 0.69314718055994531;
  static const double inv_fact[12] = {1.0 / 39916800.0, 1.0 / 3628800.0, 1.0 / 362880.0,
                                      1.0 / 40320.0,    1.0 / 5040.0,    1.0 / 720.0,
                                      1.0 / 120.0,      1.0 / 24.0,      1.0 / 6.0,
                                      0.5,              1.0,             1.0};
  double p = inv_fact[0];
  for (int i = 1; i < 12; ++i) p = std::fma(p, r, inv_fact[i]);
  const uint64_t bits = uint64_t(int64_t(k) + 1023) << 52;
  double two_k;
  std::memcpy(&two_k, &bits, sizeof two_k);
  return p * two_k;
}

struct GenTables {
  const float* q[3];   // [axis][blob * dim + i]: squared distance to the centre
  const float* e[3];   // [axis][blob * dim + i]: Gaussian factor
  const float* lim;    // [blob]: 32 sigma^2
  const float* peak;   // [blob]
};

// One CTA per (y, z) row at a time: the blobs that can reach the row are
// listed first (their y and z terms alone already reach the limit otherwise:
// IEEE addition of the non-negative x term cannot lower the sum), in blob
// order, then every voxel of the row adds their contributions in that order.
template <class T>
__global__ void __launch_bounds__(kGenThreads)
generate_kernel(T* __restrict__ out, uint64_t nx, uint64_t ny, uint64_t nz, GenTables tb,
                uint32_t n_blobs, float noise_amp, uint32_t octaves, float cell, uint64_t seed,
                int int_noise, float vmax) {
  extern __shared__ float sm[];
  float* s_qy = sm;
  float* s_qz = s_qy + n_blobs;
  float* s_ey = s_qz + n_blobs;
  float* s_ez = s_ey + n_blobs;
  float* s_lim = s_ez + n_blobs;
  float* s_pk = s_lim + n_blobs;
  uint32_t* s_id = reinterpret_cast<uint32_t*>(s_pk + n_blobs);
  __shared__ uint32_t warp_cnt[kGenThreads / 32];
  __shared__ uint32_t n_kept;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float wsum = 0.0f;
  for (uint32_t k = 0; k < octaves; ++k) wsum = wsum + ldexpf(1.0f, -int(k));
  const float nscale = octaves > 0 ? noise_amp / wsum : 0.0f;
  const uint64_t rows = ny * nz;
  for (uint64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const uint64_t y = row % ny, z = row / ny;
    __syncthreads();  // the previous row's list is no longer read
    if (tid == 0) n_kept = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_blobs; base += kGenThreads) {
      const uint32_t b = base + tid;
      float qy = 0.f, qz = 0.f;
      bool keep = false;
      if (b < n_blobs) {
        qy = tb.q[1][uint64_t(b) * ny + y];
        qz = tb.q[2][uint64_t(b) * nz + z];
        keep = qy + qz < tb.lim[b];
      }
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warp_cnt[warp] = __popc(m);
      __syncthreads();
      uint32_t off = n_kept;
      for (uint32_t w = 0; w < warp; ++w) off += warp_cnt[w];
      if (keep) {
        const uint32_t j = off + __popc(m & ((1u << lane) - 1u));
        s_qy[j] = qy;
        s_qz[j] = qz;
        s_ey[j] = tb.e[1][uint64_t(b) * ny + y];
        s_ez[j] = tb.e[2][uint64_t(b) * nz + z];
        s_lim[j] = tb.lim[b];
        s_pk[j] = tb.peak[b];
        s_id[j] = b;
      }
      __syncthreads();
      if (tid == 0) {
        uint32_t t = n_kept;
        for (uint32_t w = 0; w < kGenThreads / 32; ++w) t += warp_cnt[w];
        n_kept = t;
      }
      __syncthreads();
    }
    const uint32_t nk = n_kept;
    for (uint64_t x = tid; x < nx; x += kGenThreads) {
      float v = 0.0f;
      for (uint32_t j = 0; j < nk; ++j) {
        const uint64_t bx = uint64_t(s_id[j]) * nx + x;
        const float d2 = (__ldg(&tb.q[0][bx]) + s_qy[j]) + s_qz[j];
        if (d2 < s_lim[j]) {
          const float g = (__ldg(&tb.e[0][bx]) * s_ey[j]) * s_ez[j];
          v = v + s_pk[j] * g;
        }
      }
      if (int_noise) {
        const int64_t span = int64_t(2.0f * noise_amp + 1.0f);
        const uint64_t h = hash4(seed, x, y, z, 0xabcdefull);
        v = v + float(int64_t(h % uint64_t(span)) - int64_t(noise_amp));
      } else if (octaves > 0) {
        float nv = 0.0f;
        float c = cell;
        for (uint32_t k = 0; k < octaves; ++k, c = c * 0.5f) {
          const float gx = float(x) / c, gy = float(y) / c, gz = float(z) / c;
          const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
          const float tx = gx - fx, ty = gy - fy, tz = gz - fz;
          const float sx = (tx * tx) * (3.0f - 2.0f * tx);
          const float sy = (ty * ty) * (3.0f - 2.0f * ty);
          const float sz = (tz * tz) * (3.0f - 2.0f * tz);
          const int64_t X = int64_t(fx), Y = int64_t(fy), Z = int64_t(fz);
          float acc = 0.0f;
          for (int cz = 0; cz < 2; ++cz)
            for (int cy = 0; cy < 2; ++cy)
              for (int cx = 0; cx < 2; ++cx) {
                const float w = ((cx ? sx : 1.0f - sx) * (cy ? sy : 1.0f - sy)) *
                                (cz ? sz : 1.0f - sz);
                acc = acc + w * lattice(seed, k, X + cx, Y + cy, Z + cz);
              }
          nv = nv + acc * ldexpf(1.0f, -int(k));
        }
        v = v + nv * nscale;
      }
      v = floorf(v + 0.5f);
      v = fminf(fmaxf(v, 0.0f), vmax);
      out[(z * ny + y) * nx + x] = T(v);
    }
  }
}

}  // namespace

void launch_generate(void* out, int bytes, const uint64_t dims[3], const float* host_blobs,
                     uint32_t n_blobs, float noise_amp, uint32_t octaves, float cell,
                     uint64_t seed, int int_noise, float vmax, cudaStream_t s) {
  if (n_blobs > kMaxBlobs) fail(TVK_ERR_INVALID_ARG, "too many blobs (max 2048)");
  // per-axis tables, blob-major: q = (i - c)^2 and e = exp(-q / (2 sigma^2))
  std::vector<float> q[3], e[3];
  std::vector<float> lim(std::max<uint32_t>(n_blobs, 1)), peak(std::max<uint32_t>(n_blobs, 1));
  for (int a = 0; a < 3; ++a) {
    q[a].resize(size_t(std::max<uint32_t>(n_blobs, 1)) * dims[a]);
    e[a].resize(q[a].size());
  }
  for (uint32_t b = 0; b < n_blobs; ++b) {
    const float* B = host_blobs + 7 * size_t(b);
    const float s2 = B[3] * B[3];
    lim[b] = 32.0f * s2;
    peak[b] = B[4];
    const double den = 2.0 * double(s2);
    for (int a = 0; a < 3; ++a)
      for (uint64_t i = 0; i < dims[a]; ++i) {
        const float d = float(i) - B[a];
        const float qq = d * d;
        q[a][size_t(b) * dims[a] + i] = qq;
        e[a][size_t(b) * dims[a] + i] = float(exp_nonpositive(-double(qq) / den));
      }
  }
  size_t total = 2 * lim.size();
  for (int a = 0; a < 3; ++a) total += 2 * q[a].size();
  void* dtab = nullptr;
  TVK_CUDA(cudaMalloc(&dtab, total * sizeof(float)));
  float* p = static_cast<float*>(dtab);
  GenTables tb;
  auto put = [&](const std::vector<float>& v) {
    float* d = p;
    const cudaError_t err =
        cudaMemcpyAsync(d, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (err != cudaSuccess) {
      cudaFree(dtab);
      check_cuda(err, "cudaMemcpyAsync(generator tables)");
    }
    p += v.size();
    return d;
  };
  for (int a = 0; a < 3; ++a) tb.q[a] = put(q[a]);
  for (int a = 0; a < 3; ++a) tb.e[a] = put(e[a]);
  tb.lim = put(lim);
  tb.peak = put(peak);
  const size_t smem = size_t(std::max<uint32_t>(n_blobs, 1)) * 7 * sizeof(float);
  const uint32_t grid = 152 * 8;
  cudaError_t err = cudaSuccess;
  if (bytes == 1) {
    err = cudaFuncSetAttribute(generate_kernel<uint8_t>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (err == cudaSuccess)
      generate_kernel<uint8_t><<<grid, kGenThreads, smem, s>>>(
          static_cast<uint8_t*>(out), dims[0], dims[1], dims[2], tb, n_blobs, noise_amp,
          octaves, cell, seed, int_noise, vmax);
  } else {
    err = cudaFuncSetAttribute(generate_kernel<uint16_t>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (err == cudaSuccess)
      generate_kernel<uint16_t><<<grid, kGenThreads, smem, s>>>(
          static_cast<uint16_t*>(out), dims[0], dims[1], dims[2], tb, n_blobs, noise_amp,
          octaves, cell, seed, int_noise, vmax);
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  cudaFree(dtab);
  check_cuda(err, "generate_kernel");
}

}  // namespace tvk
