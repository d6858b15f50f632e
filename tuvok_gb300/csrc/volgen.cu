// volgen.cu -- seeded synthetic volumes (input creation for tests and benchmarks).
//
// value(x,y,z) = sum_b peak_b * exp(-|p - c_b|^2 / (2 sigma_b^2))
//              + noise(x,y,z),  rounded to nearest and clamped to [0, vmax].
// Noise is either value noise (lattice values in [-1,1] from a 64-bit hash of
// (seed, octave, lattice point), smoothstep-interpolated, octave k at cell
// size cell/2^k with weight 2^-k, scaled so the weights sum to noise_amp) or
// uniform integer noise in [-noise_amp, noise_amp] from the hash of the voxel.
#include "tvk_internal.h"

namespace tvk {
namespace {

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

__device__ __forceinline__ float smooth(float t) { return t * t * (3.0f - 2.0f * t); }

template <class T>
__global__ void generate_kernel(T* __restrict__ out, uint64_t nx, uint64_t ny, uint64_t nz,
                                const float* __restrict__ blobs, uint32_t n_blobs,
                                float noise_amp, uint32_t octaves, float cell, uint64_t seed,
                                int int_noise, float vmax) {
  extern __shared__ float sb[];
  for (uint32_t i = threadIdx.x; i < 7 * n_blobs; i += blockDim.x) sb[i] = blobs[i];
  __syncthreads();
  const uint64_t n = nx * ny * nz;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  float wsum = 0.f;
  for (uint32_t k = 0; k < octaves; ++k) wsum += ldexpf(1.0f, -int(k));
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
    const float fx = float(x), fy = float(y), fz = float(z);
    float v = 0.f;
    for (uint32_t b = 0; b < n_blobs; ++b) {
      const float* B = sb + 7 * b;
      const float dx = fx - B[0], dy = fy - B[1], dz = fz - B[2];
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float s2 = B[3] * B[3];
      if (d2 < 32.0f * s2) v += B[4] * expf(-d2 / (2.0f * s2));
    }
    if (int_noise) {
      const int64_t span = int64_t(2.0f * noise_amp + 1.0f);
      const uint64_t h = hash4(seed, x, y, z, 0xabcdefull);
      v += float(int64_t(h % uint64_t(span)) - int64_t(noise_amp));
    } else if (octaves > 0) {
      float nv = 0.f;
      float c = cell;
      for (uint32_t k = 0; k < octaves; ++k, c *= 0.5f) {
        const float gx = fx / c, gy = fy / c, gz = fz / c;
        const float ix = floorf(gx), iy = floorf(gy), iz = floorf(gz);
        const float tx = smooth(gx - ix), ty = smooth(gy - iy), tz = smooth(gz - iz);
        const int64_t X = int64_t(ix), Y = int64_t(iy), Z = int64_t(iz);
        float acc = 0.f;
        for (int cz = 0; cz < 2; ++cz)
          for (int cy = 0; cy < 2; ++cy)
            for (int cx = 0; cx < 2; ++cx) {
              const float w = (cx ? tx : 1.f - tx) * (cy ? ty : 1.f - ty) * (cz ? tz : 1.f - tz);
              acc += w * lattice(seed, k, X + cx, Y + cy, Z + cz);
            }
        nv += acc * ldexpf(1.0f, -int(k));
      }
      v += nv * (noise_amp / wsum);
    }
    v = floorf(v + 0.5f);
    v = fminf(fmaxf(v, 0.0f), vmax);
    out[i] = T(v);
  }
}

}  // namespace

void launch_generate(void* out, int bytes, const uint64_t dims[3], const float* d_blobs,
                     uint32_t n_blobs, float noise_amp, uint32_t octaves, float cell,
                     uint64_t seed, int int_noise, float vmax, cudaStream_t s) {
  const size_t smem = size_t(7) * n_blobs * sizeof(float);
  if (smem > 48 * 1024) fail(TVK_ERR_INVALID_ARG, "too many blobs (max 1755)");
  const uint32_t grid = 152 * 8;
  if (bytes == 1)
    generate_kernel<uint8_t><<<grid, 256, smem, s>>>(static_cast<uint8_t*>(out), dims[0], dims[1],
                                                     dims[2], d_blobs, n_blobs, noise_amp,
                                                     octaves, cell, seed, int_noise, vmax);
  else
    generate_kernel<uint16_t><<<grid, 256, smem, s>>>(static_cast<uint16_t*>(out), dims[0],
                                                      dims[1], dims[2], d_blobs, n_blobs,
                                                      noise_amp, octaves, cell, seed, int_noise,
                                                      vmax);
  TVK_CUDA(cudaGetLastError());
}

}  // namespace tvk
