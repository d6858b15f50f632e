// raycast.cu -- brick-by-brick front-to-back ray march on sm_103a.
//
// Restates Tuvok's GLRaycaster: for every pixel, every non-empty LOD-0 brick the
// pixel's ray crosses is marched on its own (Shaders/GLRaycaster-1D-FS.glsl:51-82,
// -1D-light-FS.glsl:84-134, -2D-FS.glsl:53-94, -2D-light-FS.glsl:61-117) from its
// RGBA16F-rounded entry point (Renderer/GL/GLRaycaster.cpp:93-99) with the brick's
// own step size and opacity correction (:239-300), and the per-brick colour is
// blended into the frame with (ONE_MINUS_DST_ALPHA, ONE) (GLRenderer.cpp:151-153)
// in the order the ray meets the bricks.
//
// One thread per pixel, warps on 8x4 pixel tiles so neighbouring rays touch the
// same brick cache lines.  The arithmetic is the oracle's, operation for
// operation: this file is compiled with -fmad=false, every fused multiply-add is
// an explicit fmaf, sqrt and division are IEEE, and opacity correction comes from
// a host-built table (1 - powf(1 - a, s) per TF entry).  Work the reference does
// but that cannot change the pixel is skipped: gradients and lighting of samples
// whose corrected alpha is 0 (their compositing adds exactly zero).
#include <cuda_fp16.h>
#include <type_traits>

#include "tvk_internal.h"

// 1: the lit march batches the gradient and lighting of pending samples
// across the warp (same per-ray arithmetic, other interleaving); measured
// 12 % faster on the 1024^3 lit frame (4.26 -> 3.76 ms), 20 % on 512^3.
// TVK_DEFER_NUM / TVK_DEFER_DEN: the pending share of the marching lanes that
// starts a batch (1/3: 3.93, 1/2: 3.84, 2/3: 3.77, 3/4: 3.77, 7/8: 3.79 ms).
#ifndef TVK_DEFER_LIGHT
#define TVK_DEFER_LIGHT 1
#endif
#ifndef TVK_DEFER_NUM
#define TVK_DEFER_NUM 3
#endif
#ifndef TVK_DEFER_DEN
#define TVK_DEFER_DEN 4
#endif
// 1: the centre samples are batched the same way (a lane that reached a
// non-empty cell waits while the others leap); measured slower (4.59 against
// 3.76 ms on the 1024^3 lit frame), so off
#ifndef TVK_DEFER_SAMPLE
#define TVK_DEFER_SAMPLE 0
#endif

// 1: count leap iterations, the steps they skip, candidate-brick slab tests
// and brick marches into the frame's counters [4..7] (one global atomic per
// event: a profiling build, not for timing).
#ifndef TVK_PROFILE_COUNTS
#define TVK_PROFILE_COUNTS 0
#endif
#if TVK_PROFILE_COUNTS
#define TVK_PROF(P, i, n) atomicAdd(&(P).counters[i], (unsigned long long)(n))
#else
#define TVK_PROF(P, i, n) ((void)0)
#endif

namespace tvk {
namespace {

// CTAs of 128 threads the register allocation must leave room for per SM
// (occupancy against spills; measured on GB300 with the 1024^3 lit frames:
// 6 CTAs 3.42 ms, 5 3.48, 7 3.46, 8 3.61, 4 3.86).
#ifndef TVK_RAYCAST_MIN_BLOCKS
#define TVK_RAYCAST_MIN_BLOCKS 6
#endif

__device__ __forceinline__ float affine_row(const float r[4], float x, float y, float z) {
  return fmaf(r[0], x, fmaf(r[1], y, fmaf(r[2], z, r[3])));
}

__device__ __forceinline__ float len3(float x, float y, float z) {
  return sqrtf((x * x + y * y) + z * z);
}

template <class T>
struct BrickView {
  const T* __restrict__ p;
  int n0, n1, n2;
  float fn0, fn1, fn2;
  uint32_t sx, sxy;

  __device__ __forceinline__ float fetch(int x, int y, int z) const {
    // 32-bit voxel offset: a brick holds fewer than 2^32 voxels (at most 1023 per axis)
    return float(__ldg(p + (uint32_t(x) + uint32_t(y) * sx + uint32_t(z) * sxy)));
  }
  // texel-centre trilinear, clamp to edge, raw units
  __device__ __forceinline__ float sample_raw(float tx, float ty, float tz) const {
    float u0 = fmaf(tx, fn0, -0.5f);
    float u1 = fmaf(ty, fn1, -0.5f);
    float u2 = fmaf(tz, fn2, -0.5f);
    u0 = fminf(fmaxf(u0, 0.0f), float(n0 - 1));
    u1 = fminf(fmaxf(u1, 0.0f), float(n1 - 1));
    u2 = fminf(fmaxf(u2, 0.0f), float(n2 - 1));
    return sample_u(u0, u1, u2);
  }
  // the same from voxel coordinates already clamped to [0, n-1]
  __device__ __forceinline__ float sample_u(float u0, float u1, float u2) const {
    const int x0 = int(u0), y0 = int(u1), z0 = int(u2);
    const float fx = u0 - float(x0), fy = u1 - float(y0), fz = u2 - float(z0);
    const int x1 = min(x0 + 1, n0 - 1), y1 = min(y0 + 1, n1 - 1), z1 = min(z0 + 1, n2 - 1);
    const float v000 = fetch(x0, y0, z0), v100 = fetch(x1, y0, z0);
    const float v010 = fetch(x0, y1, z0), v110 = fetch(x1, y1, z0);
    const float v001 = fetch(x0, y0, z1), v101 = fetch(x1, y0, z1);
    const float v011 = fetch(x0, y1, z1), v111 = fetch(x1, y1, z1);
    const float c00 = fmaf(fx, v100 - v000, v000);
    const float c10 = fmaf(fx, v110 - v010, v010);
    const float c01 = fmaf(fx, v101 - v001, v001);
    const float c11 = fmaf(fx, v111 - v011, v011);
    const float c0 = fmaf(fy, c10 - c00, c00);
    const float c1 = fmaf(fy, c11 - c01, c01);
    return fmaf(fz, c1 - c0, c0);
  }
};

// RGBA8 bricks (colour volumes, four unsigned-normalised channels): every
// channel filtered exactly like the scalar lookup.
struct ColorView {
  const uchar4* __restrict__ p;
  int n0, n1, n2;
  float fn0, fn1, fn2;
  uint32_t sx, sxy;

  __device__ __forceinline__ uchar4 fetch(int x, int y, int z) const {
    return __ldg(p + (uint32_t(x) + uint32_t(y) * sx + uint32_t(z) * sxy));
  }
  __device__ __forceinline__ static float tri(float fx, float fy, float fz, float v000,
                                              float v100, float v010, float v110, float v001,
                                              float v101, float v011, float v111) {
    const float c00 = fmaf(fx, v100 - v000, v000);
    const float c10 = fmaf(fx, v110 - v010, v010);
    const float c01 = fmaf(fx, v101 - v001, v001);
    const float c11 = fmaf(fx, v111 - v011, v011);
    const float c0 = fmaf(fy, c10 - c00, c00);
    const float c1 = fmaf(fy, c11 - c01, c01);
    return fmaf(fz, c1 - c0, c0);
  }
  // channel mask: bit c set = filter channel c (others returned as 0); raw units
  template <int kMask>
  __device__ __forceinline__ float4 sample_raw(float tx, float ty, float tz) const {
    const float u0 = fminf(fmaxf(fmaf(tx, fn0, -0.5f), 0.0f), float(n0 - 1));
    const float u1 = fminf(fmaxf(fmaf(ty, fn1, -0.5f), 0.0f), float(n1 - 1));
    const float u2 = fminf(fmaxf(fmaf(tz, fn2, -0.5f), 0.0f), float(n2 - 1));
    return sample_u<kMask>(u0, u1, u2);
  }
  // the same from voxel coordinates already clamped to [0, n-1]
  template <int kMask>
  __device__ __forceinline__ float4 sample_u(float u0, float u1, float u2) const {
    const int x0 = int(u0), y0 = int(u1), z0 = int(u2);
    const float fx = u0 - float(x0), fy = u1 - float(y0), fz = u2 - float(z0);
    const int x1 = min(x0 + 1, n0 - 1), y1 = min(y0 + 1, n1 - 1), z1 = min(z0 + 1, n2 - 1);
    const uchar4 a = fetch(x0, y0, z0), b = fetch(x1, y0, z0), c = fetch(x0, y1, z0),
                 d = fetch(x1, y1, z0), e = fetch(x0, y0, z1), f = fetch(x1, y0, z1),
                 g = fetch(x0, y1, z1), h = fetch(x1, y1, z1);
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (kMask & 1)
      r.x = tri(fx, fy, fz, a.x, b.x, c.x, d.x, e.x, f.x, g.x, h.x);
    if (kMask & 2)
      r.y = tri(fx, fy, fz, a.y, b.y, c.y, d.y, e.y, f.y, g.y, h.y);
    if (kMask & 4)
      r.z = tri(fx, fy, fz, a.z, b.z, c.z, d.z, e.z, f.z, g.z, h.z);
    if (kMask & 8)
      r.w = tri(fx, fy, fz, a.w, b.w, c.w, d.w, e.w, f.w, g.w, h.w);
    return r;
  }
};

__device__ __forceinline__ ColorView color_view(const RenderParams& P, const DevBrick& b) {
  ColorView v;
  v.p = static_cast<const uchar4*>(P.pool) + b.off;
  v.n0 = int(b.n[0]); v.n1 = int(b.n[1]); v.n2 = int(b.n[2]);
  v.fn0 = float(b.n[0]); v.fn1 = float(b.n[1]); v.fn2 = float(b.n[2]);
  v.sx = b.n[0]; v.sxy = b.n[0] * b.n[1];
  return v;
}

// Footprint of a centre sample, kept so the six central-difference lookups
// (each one voxel away along one axis) reuse its index math and its voxels.
// Every lookup still evaluates exactly the oracle's trilinear: the unshifted
// axes' coordinates are the centre's (the same float expression), and a
// voxel is taken from the centre's registers only when its index is equal.
struct Foot {
  int x0, x1, y0, y1, z0, z1;
  float fx, fy, fz;
  float v000, v100, v010, v110, v001, v101, v011, v111;
};

template <class T>
__device__ __forceinline__ float centre_sample(const BrickView<T>& B, float u0, float u1,
                                               float u2, Foot& f) {
  f.x0 = int(u0); f.y0 = int(u1); f.z0 = int(u2);
  f.fx = u0 - float(f.x0); f.fy = u1 - float(f.y0); f.fz = u2 - float(f.z0);
  f.x1 = min(f.x0 + 1, B.n0 - 1); f.y1 = min(f.y0 + 1, B.n1 - 1); f.z1 = min(f.z0 + 1, B.n2 - 1);
  f.v000 = B.fetch(f.x0, f.y0, f.z0); f.v100 = B.fetch(f.x1, f.y0, f.z0);
  f.v010 = B.fetch(f.x0, f.y1, f.z0); f.v110 = B.fetch(f.x1, f.y1, f.z0);
  f.v001 = B.fetch(f.x0, f.y0, f.z1); f.v101 = B.fetch(f.x1, f.y0, f.z1);
  f.v011 = B.fetch(f.x0, f.y1, f.z1); f.v111 = B.fetch(f.x1, f.y1, f.z1);
  const float c00 = fmaf(f.fx, f.v100 - f.v000, f.v000);
  const float c10 = fmaf(f.fx, f.v110 - f.v010, f.v010);
  const float c01 = fmaf(f.fx, f.v101 - f.v001, f.v001);
  const float c11 = fmaf(f.fx, f.v111 - f.v011, f.v011);
  const float c0 = fmaf(f.fy, c10 - c00, c00);
  const float c1 = fmaf(f.fy, c11 - c01, c01);
  return fmaf(f.fz, c1 - c0, c0);
}

// lookup with the x coordinate replaced by u (clamped voxel coordinate)
template <class T>
__device__ __forceinline__ float shifted_x(const BrickView<T>& B, const Foot& f, float u) {
  const int a = int(u), b = min(a + 1, B.n0 - 1);
  const float w = u - float(a);
  float a00, a10, a01, a11, b00, b10, b01, b11;  // [y][z]
  if (a == f.x0) { a00 = f.v000; a10 = f.v010; a01 = f.v001; a11 = f.v011; }
  else if (a == f.x1) { a00 = f.v100; a10 = f.v110; a01 = f.v101; a11 = f.v111; }
  else { a00 = B.fetch(a, f.y0, f.z0); a10 = B.fetch(a, f.y1, f.z0);
         a01 = B.fetch(a, f.y0, f.z1); a11 = B.fetch(a, f.y1, f.z1); }
  if (b == f.x1) { b00 = f.v100; b10 = f.v110; b01 = f.v101; b11 = f.v111; }
  else if (b == f.x0) { b00 = f.v000; b10 = f.v010; b01 = f.v001; b11 = f.v011; }
  else { b00 = B.fetch(b, f.y0, f.z0); b10 = B.fetch(b, f.y1, f.z0);
         b01 = B.fetch(b, f.y0, f.z1); b11 = B.fetch(b, f.y1, f.z1); }
  const float c00 = fmaf(w, b00 - a00, a00), c10 = fmaf(w, b10 - a10, a10);
  const float c01 = fmaf(w, b01 - a01, a01), c11 = fmaf(w, b11 - a11, a11);
  const float c0 = fmaf(f.fy, c10 - c00, c00), c1 = fmaf(f.fy, c11 - c01, c01);
  return fmaf(f.fz, c1 - c0, c0);
}

template <class T>
__device__ __forceinline__ float shifted_y(const BrickView<T>& B, const Foot& f, float u) {
  const int a = int(u), b = min(a + 1, B.n1 - 1);
  const float w = u - float(a);
  float a00, a10, a01, a11, b00, b10, b01, b11;  // [x][z]
  if (a == f.y0) { a00 = f.v000; a10 = f.v100; a01 = f.v001; a11 = f.v101; }
  else if (a == f.y1) { a00 = f.v010; a10 = f.v110; a01 = f.v011; a11 = f.v111; }
  else { a00 = B.fetch(f.x0, a, f.z0); a10 = B.fetch(f.x1, a, f.z0);
         a01 = B.fetch(f.x0, a, f.z1); a11 = B.fetch(f.x1, a, f.z1); }
  if (b == f.y1) { b00 = f.v010; b10 = f.v110; b01 = f.v011; b11 = f.v111; }
  else if (b == f.y0) { b00 = f.v000; b10 = f.v100; b01 = f.v001; b11 = f.v101; }
  else { b00 = B.fetch(f.x0, b, f.z0); b10 = B.fetch(f.x1, b, f.z0);
         b01 = B.fetch(f.x0, b, f.z1); b11 = B.fetch(f.x1, b, f.z1); }
  const float c00 = fmaf(f.fx, a10 - a00, a00), c10 = fmaf(f.fx, b10 - b00, b00);
  const float c01 = fmaf(f.fx, a11 - a01, a01), c11 = fmaf(f.fx, b11 - b01, b01);
  const float c0 = fmaf(w, c10 - c00, c00), c1 = fmaf(w, c11 - c01, c01);
  return fmaf(f.fz, c1 - c0, c0);
}

template <class T>
__device__ __forceinline__ float shifted_z(const BrickView<T>& B, const Foot& f, float u) {
  const int a = int(u), b = min(a + 1, B.n2 - 1);
  const float w = u - float(a);
  float a00, a10, a01, a11, b00, b10, b01, b11;  // [x][y]
  if (a == f.z0) { a00 = f.v000; a10 = f.v100; a01 = f.v010; a11 = f.v110; }
  else if (a == f.z1) { a00 = f.v001; a10 = f.v101; a01 = f.v011; a11 = f.v111; }
  else { a00 = B.fetch(f.x0, f.y0, a); a10 = B.fetch(f.x1, f.y0, a);
         a01 = B.fetch(f.x0, f.y1, a); a11 = B.fetch(f.x1, f.y1, a); }
  if (b == f.z1) { b00 = f.v001; b10 = f.v101; b01 = f.v011; b11 = f.v111; }
  else if (b == f.z0) { b00 = f.v000; b10 = f.v100; b01 = f.v010; b11 = f.v110; }
  else { b00 = B.fetch(f.x0, f.y0, b); b10 = B.fetch(f.x1, f.y0, b);
         b01 = B.fetch(f.x0, f.y1, b); b11 = B.fetch(f.x1, f.y1, b); }
  const float c00 = fmaf(f.fx, a10 - a00, a00), c10 = fmaf(f.fx, a11 - a01, a01);
  const float c01 = fmaf(f.fx, b10 - b00, b00), c11 = fmaf(f.fx, b11 - b01, b01);
  const float c0 = fmaf(f.fy, c10 - c00, c00), c1 = fmaf(f.fy, c11 - c01, c01);
  return fmaf(w, c1 - c0, c0);
}

// Hardware-filtered bricks (the measured alternative to the exact lookups): a
// brick's copy in a 3D CUDA array read through a texture object with linear
// filtering, clamp to edge and normalised reads, at unnormalised coordinates
// u + 0.5 (texel i's centre is at i + 0.5), so a lookup at clamped voxel
// coordinate u filters the same eight texels as the exact path, with the
// texture unit's fixed-point weights; `scale` (255 or 65535) returns raw
// units.  Not bit-exact: its distance to the oracle is measured and reported.
struct TexView {
  cudaTextureObject_t obj;
  int n0, n1, n2;
  float fn0, fn1, fn2;
  float scale;
  __device__ __forceinline__ float sample_u(float u0, float u1, float u2) const {
    return tex3D<float>(obj, u0 + 0.5f, u1 + 0.5f, u2 + 0.5f) * scale;
  }
  __device__ __forceinline__ float sample_raw(float tx, float ty, float tz) const {
    const float u0 = fminf(fmaxf(fmaf(tx, fn0, -0.5f), 0.0f), float(n0 - 1));
    const float u1 = fminf(fmaxf(fmaf(ty, fn1, -0.5f), 0.0f), float(n1 - 1));
    const float u2 = fminf(fmaxf(fmaf(tz, fn2, -0.5f), 0.0f), float(n2 - 1));
    return sample_u(u0, u1, u2);
  }
};

// The centre sample and the shifted lookups of the gradient for a texture
// view: the footprint keeps only the centre's coordinates (in fx, fy, fz).
__device__ __forceinline__ float centre_sample(const TexView& B, float u0, float u1, float u2,
                                               Foot& f) {
  f.fx = u0; f.fy = u1; f.fz = u2;
  return B.sample_u(u0, u1, u2);
}
__device__ __forceinline__ float shifted_x(const TexView& B, const Foot& f, float u) {
  return B.sample_u(u, f.fy, f.fz);
}
__device__ __forceinline__ float shifted_y(const TexView& B, const Foot& f, float u) {
  return B.sample_u(f.fx, u, f.fz);
}
__device__ __forceinline__ float shifted_z(const TexView& B, const Foot& f, float u) {
  return B.sample_u(f.fx, f.fy, u);
}

// The brick's view for the march: its pool voxels, or its texture.
template <class V, class T>
__device__ __forceinline__ V brick_view(const RenderParams& P, const DevBrick& b) {
  V v;
  if constexpr (std::is_same<V, TexView>::value) {
    v.obj = P.tex[b.id];
    v.scale = sizeof(T) == 1 ? 255.0f : 65535.0f;
  } else {
    v.p = static_cast<const T*>(P.pool) + b.off;
    v.sx = b.n[0];
    v.sxy = b.n[0] * b.n[1];
  }
  v.n0 = int(b.n[0]); v.n1 = int(b.n[1]); v.n2 = int(b.n[2]);
  v.fn0 = float(b.n[0]); v.fn1 = float(b.n[1]); v.fn2 = float(b.n[2]);
  return v;
}

// (fn - 1.0f is float(n - 1) exactly: n < 2^24)
__device__ __forceinline__ float clamp_u(float t, float fn, int n) {
  (void)n;
  return fminf(fmaxf(fmaf(t, fn, -0.5f), 0.0f), fn - 1.0f);
}

// x^y for x in [0, 1] as exp2(y * log2(x)) (GLSL defines pow as that
// composition and leaves its precision to the implementation), in double
// operations that give the same bits on any IEEE machine, rounded to float:
//  * log2(x) = e + (2 / ln 2) * atanh(s), x = m * 2^e with m in [sqrt(1/2),
//    sqrt(2)), s = (m - 1) / (m + 1) (|s| <= 0.172), the atanh series
//    s + s^3/3 + ... + s^13/13 (truncation below 1e-12);
//  * exp2(t) = 2^k * e^(f ln 2), k = floor(t + 1/2), |f| <= 1/2, the Taylor
//    series of e^z to z^9 (truncation below 1e-10).
// Within one float ulp of the exact power.  Results below 2^-125 are
// returned as 0: callers use 1 - x^y, which that leaves unchanged.
__device__ __forceinline__ float pow01(float xf, float yf) {
  if (yf == 0.0f || xf == 1.0f) return 1.0f;
  if (!(xf > 0.0f)) return 0.0f;
  if (xf > 1.0f) return 1.0f;  // a rounded dot product of unit vectors
  const double x = double(xf);
  const uint64_t bits = uint64_t(__double_as_longlong(x));
  double e = double(int((bits >> 52) & 0x7ffu) - 1022);  // float inputs: never subnormal here
  double m = __longlong_as_double(
      (long long)((bits & 0x000fffffffffffffull) | 0x3fe0000000000000ull));  // [0.5, 1)
  if (m < 0.70710678118654752) { m = m * 2.0; e = e - 1.0; }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 1.0 / 13.0;
  p = fma(p, s2, 1.0 / 11.0);
  p = fma(p, s2, 1.0 / 9.0);
  p = fma(p, s2, 1.0 / 7.0);
  p = fma(p, s2, 1.0 / 5.0);
  p = fma(p, s2, 1.0 / 3.0);
  p = fma(p, s2, 1.0);
  const double lg = fma(2.8853900817779268 * s, p, e);  // 2 / ln 2
  const double t = double(yf) * lg;
  if (!(t > -125.0)) return 0.0f;
  if (t >= 128.0) return INFINITY;  // y < 0
  const double k = floor(t + 0.5);
  const double z = (t - k) * 0.69314718055994531;  // ln 2
  double q = 1.0 / 362880.0;
  q = fma(q, z, 1.0 / 40320.0);
  q = fma(q, z, 1.0 / 5040.0);
  q = fma(q, z, 1.0 / 720.0);
  q = fma(q, z, 1.0 / 120.0);
  q = fma(q, z, 1.0 / 24.0);
  q = fma(q, z, 1.0 / 6.0);
  q = fma(q, z, 0.5);
  q = fma(q, z, 1.0);
  q = fma(q, z, 1.0);
  const double two_k = __longlong_as_double((long long)(uint64_t(int(k) + 1023) << 52));
  return float(q * two_k);
}

__device__ __forceinline__ float pow_int_or_real(float x, float e) {
  if (e == 8.0f) { float a = x * x; a = a * a; return a * a; }
  if (e == 32.0f) { float a = x * x; a = a * a; a = a * a; a = a * a; return a * a; }
  return pow01(x, e);
}

__device__ __forceinline__ void lighting_ref(const RenderParams& P, const float pos[3],
                                             const float N[3], const float tfc[3], float out[3]) {
  // Shaders/lighting.glsl:33-43
  const float p0 = -pos[0], p1 = -pos[1], p2 = -pos[2];
  // normalize() as a multiply by the correctly rounded reciprocal length
  const float ilp = 1.0f / len3(p0, p1, p2);
  const float V0 = p0 * ilp, V1 = p1 * ilp, V2 = p2 * ilp;
  const float d = (N[0] * V0 + N[1] * V1) + N[2] * V2;
  float R0 = V0 - (2.0f * d) * N[0];
  float R1 = V1 - (2.0f * d) * N[1];
  float R2 = V2 - (2.0f * d) * N[2];
  const float ilr = 1.0f / len3(R0, R1, R2);
  R0 = R0 * ilr; R1 = R1 * ilr; R2 = R2 * ilr;
  const float* L = P.light_dir;
  const float diff = fmaxf(fabsf((N[0] * L[0] + N[1] * L[1]) + N[2] * L[2]), 0.0f);
  const float spec = pow_int_or_real(fmaxf((R0 * L[0] + R1 * L[1]) + R2 * L[2], 0.0f), 8.0f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float dcol = P.light_d[i] * tfc[i];
    float c = P.light_a[i] + dcol * diff;
    c = c + P.light_s[i] * spec;
    out[i] = fminf(fmaxf(c, 0.0f), 1.0f);
  }
}

__device__ __forceinline__ void lighting_bp(const RenderParams& P, const float pos[3],
                                            const float Nin[3], const float tfc[3], float out[3]) {
  const float p0 = -pos[0], p1 = -pos[1], p2 = -pos[2];
  const float ilp = 1.0f / len3(p0, p1, p2);
  const float V0 = p0 * ilp, V1 = p1 * ilp, V2 = p2 * ilp;
  float N0 = Nin[0], N1 = Nin[1], N2 = Nin[2];
  if ((N0 * V0 + N1 * V1) + N2 * V2 < 0.0f) { N0 = -N0; N1 = -N1; N2 = -N2; }
  const float L0 = -P.light_dir[0], L1 = -P.light_dir[1], L2 = -P.light_dir[2];
  float H0 = L0 + V0, H1 = L1 + V1, H2 = L2 + V2;
  const float ilh = 1.0f / len3(H0, H1, H2);
  H0 = H0 * ilh; H1 = H1 * ilh; H2 = H2 * ilh;
  const float diff = fmaxf((N0 * L0 + N1 * L1) + N2 * L2, 0.0f);
  const float spec = pow_int_or_real(fmaxf((N0 * H0 + N1 * H1) + N2 * H2, 0.0f), P.bp_shininess);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float c = P.bp_ka * tfc[i];
    c = c + (P.bp_kd * tfc[i]) * diff;
    c = c + P.bp_ks * spec;
    out[i] = fminf(fmaxf(c, 0.0f), 1.0f);
  }
}

// Marches one brick; returns the brick's premultiplied RGBA.  kTex: lookups
// through the brick's texture (TexView) instead of its pool voxels.
template <class T, bool kTex = false>
__device__ __forceinline__ float4 march_brick(const RenderParams& P, const DevBrick& b,
                                              const float dir[3], float t_in, float t_out,
                                              uint32_t& samples, uint32_t& shaded,
                                              uint32_t& graded, float& first_t) {
  float en[3], ex[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    en[a] = __half2float(__float2half_rn(dir[a] * t_in));
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const float q = len / b.step;
  float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(q < P.max_q)) {
    atomicAdd(&P.counters[2], 1ull);
    return c;
  }
  const int n = int(q) + 1;
  float pos[3], inc[3], epos[3], einc[3];
  // the increment divides by the step count: a multiply by its reciprocal
  const float iq = 1.0f / q;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    inc[a] = (tout[a] - tin[a]) * iq;
    pos[a] = tin[a];
    epos[a] = en[a];
  }
  const float ilen = 1.0f / len;
  einc[0] = (dx * ilen) * b.step;
  einc[1] = (dy * ilen) * b.step;
  einc[2] = (dz * ilen) * b.step;

  using View = typename std::conditional<kTex, TexView, BrickView<T>>::type;
  const View vol = brick_view<View, T>(P, b);
  const float vs0 = 1.0f / float(b.n[0]), vs1 = 1.0f / float(b.n[1]), vs2 = 1.0f / float(b.n[2]);
  const bool lit = P.lighting != 0;
  const bool two_d = P.mode == TVK_RM_2DTRANS;
  const float W = float(P.tf_w), H = float(P.tf_h);
  const float im = P.inv_max_raw;
  // macro cells of kCell^3 voxel positions (see DevBrick::cells)
  const uint8_t* __restrict__ dist = P.cell_dist ? P.cell_dist + b.cell_off : nullptr;
  const int ncx = int(b.cells & 1023u), ncy = int((b.cells >> 10) & 1023u),
            ncz = int(b.cells >> 20);
  const float du0 = inc[0] * vol.fn0, du1 = inc[1] * vol.fn1, du2 = inc[2] * vol.fn2;
  const float idu0 = 1.0f / fabsf(du0), idu1 = 1.0f / fabsf(du1), idu2 = 1.0f / fabsf(du2);

#if TVK_DEFER_LIGHT
  // The same per-ray sequence as below (a cell test before every step, leaps
  // over empty cubes, one sample per non-empty step), scheduled so that the
  // expensive part of a sample -- the six gradient lookups, the 2D lookup and
  // the lighting -- runs for many lanes of the warp together: a lane whose
  // sample needs it waits (pending) while the other lanes leap or take cheap
  // samples, until at least half of the lanes still marching are pending.
  // Every lane's arithmetic is unchanged; only the interleaving differs.
  int i = 0;
  int epend = 0;  // additions of einc owed to epos (made before its next use)
  bool pend = false;
  Foot foot;
  float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
  float fx = 0.0f;
  bool ready = false;  // at a non-empty step, its sample not taken yet
  float u0 = 0.f, u1 = 0.f, u2 = 0.f;
  for (;;) {
    bool fin = false;     // a sample is complete: composite it and advance
    bool leaped = false;  // this lane leapt over empty cells in this round
    if (!pend && !ready) {
      if (i >= n) break;
      const float uu0 = fmaf(pos[0], vol.fn0, -0.5f);
      const float uu1 = fmaf(pos[1], vol.fn1, -0.5f);
      const float uu2 = fmaf(pos[2], vol.fn2, -0.5f);
      u0 = fminf(fmaxf(uu0, 0.0f), (vol.fn0 - 1.0f));
      u1 = fminf(fmaxf(uu1, 0.0f), (vol.fn1 - 1.0f));
      u2 = fminf(fmaxf(uu2, 0.0f), (vol.fn2 - 1.0f));
      int dd = 0;
      int cx = 0, cy = 0, cz = 0;
      if (dist) {
        cx = int(u0) >> kCellShift; cy = int(u1) >> kCellShift; cz = int(u2) >> kCellShift;
        dd = __ldg(&dist[(cz * ncy + cy) * ncx + cx]);
      }
      if (dd != 0) {
        int k = 0;
        if (uu0 == u0 && uu1 == u1 && uu2 == u2) {
          const int r = dd - 1;
          const float lo0 = float(max(cx - r, 0) << kCellShift),
                      lo1 = float(max(cy - r, 0) << kCellShift),
                      lo2 = float(max(cz - r, 0) << kCellShift);
          const float hi0 = float(min(cx + r + 1, ncx) << kCellShift),
                      hi1 = float(min(cy + r + 1, ncy) << kCellShift),
                      hi2 = float(min(cz + r + 1, ncz) << kCellShift);
          const float d0 = du0 > 0.0f ? hi0 - uu0 : uu0 - lo0;
          const float d1 = du1 > 0.0f ? hi1 - uu1 : uu1 - lo1;
          const float d2 = du2 > 0.0f ? hi2 - uu2 : uu2 - lo2;
          const float m = fminf(fminf((d0 - 0.015625f) * idu0, (d1 - 0.015625f) * idu1),
                                (d2 - 0.015625f) * idu2);
          k = m > 0.0f ? int(fminf(m, float(n - 1 - i))) : 0;
        }
        samples += uint32_t(k + 1);
        TVK_PROF(P, 4, 1);
        TVK_PROF(P, 5, k + 1);
        // the chain of k + 1 additions, unrolled (the same sums in order);
        // the eye-space position's own chain waits for a lit sample (epend)
#pragma unroll 4
        for (int j = 0; j <= k; ++j) {
#pragma unroll
          for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
        }
        epend += k + 1;
        i += k + 1;
        leaped = true;
      } else {
        ready = true;
      }
    }
    // Progress: leaping lanes advance; when no lane leapt in a round, every
    // waiting lane goes ahead, so no round passes without progress.
    bool take = ready;
    bool stalled = false;
#if TVK_DEFER_SAMPLE
    {
      const unsigned am = __activemask();
      const unsigned rm = __ballot_sync(am, ready);
      stalled = __ballot_sync(am, leaped) == 0u;
      take = ready && (stalled || TVK_DEFER_DEN * __popc(rm) >= TVK_DEFER_NUM * __popc(am));
    }
#endif
    if (take) {
      {
        ready = false;
        ++samples;
        ++shaded;
        const float v = centre_sample(vol, u0, u1, u2, foot) * im;
        const float u = v * P.trans_scale;
        fx = floorf(u * W);
        fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
        bool need;
        if (two_d) {
          need = P.tf_col_nonzero[int(fx)] != 0;
          src = make_float4(0.f, 0.f, 0.f, 0.f);  // whole column transparent
        } else {
          src = __ldg(&P.tf[int(fx)]);
          need = lit && src.w != 0.0f;
        }
        if (need) pend = true;
        else fin = true;
      }
    }
    const unsigned am = __activemask();
    const unsigned pm = __ballot_sync(am, pend);
    if (pend && (stalled || TVK_DEFER_DEN * __popc(pm) >= TVK_DEFER_NUM * __popc(am))) {
      ++graded;
      // Volume3D.glsl:43-54 (Yp sampled at -step.y)
      const float xp = shifted_x(vol, foot, clamp_u(pos[0] + vs0, vol.fn0, vol.n0)) * im;
      const float xm = shifted_x(vol, foot, clamp_u(pos[0] + (-vs0), vol.fn0, vol.n0)) * im;
      const float yp = shifted_y(vol, foot, clamp_u(pos[1] + (-vs1), vol.fn1, vol.n1)) * im;
      const float ym = shifted_y(vol, foot, clamp_u(pos[1] + vs1, vol.fn1, vol.n1)) * im;
      const float zp = shifted_z(vol, foot, clamp_u(pos[2] + vs2, vol.fn2, vol.n2)) * im;
      const float zm = shifted_z(vol, foot, clamp_u(pos[2] + (-vs2), vol.fn2, vol.n2)) * im;
      const float g0 = (xm - xp) / 2.0f, g1 = (yp - ym) / 2.0f, g2 = (zm - zp) / 2.0f;
      bool shade = lit;
      if (two_d) {
        const float mag = len3(g0, g1, g2);
        const float w = 1.0f - mag * P.grad_scale;
        float fy = floorf(w * H);
        fy = fminf(fmaxf(fy, 0.0f), H - 1.0f);
        src = __ldg(&P.tf[int(fy) * P.tf_w + int(fx)]);
        shade = lit && src.w != 0.0f;
      }
      if (shade) {
        const float gs0 = g0 * P.domain_scale[0], gs1 = g1 * P.domain_scale[1],
                    gs2 = g2 * P.domain_scale[2];
        float N[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          N[r] = fmaf(P.norm_mat[r][2], gs2, fmaf(P.norm_mat[r][1], gs1, P.norm_mat[r][0] * gs0));
        const float l = len3(N[0], N[1], N[2]);
        if (l > 0.0f) {
          const float il = 1.0f / l;
          N[0] = N[0] * il; N[1] = N[1] * il; N[2] = N[2] * il;
        }
        const float tfc[3] = {src.x, src.y, src.z};
        float lc[3];
        // the eye-space position of this step: its pending additions, in order
        for (; epend > 0; --epend) {
#pragma unroll
          for (int a = 0; a < 3; ++a) epos[a] = epos[a] + einc[a];
        }
        if (P.light_model == TVK_LIGHT_BLINN_PHONG)
          lighting_bp(P, epos, N, tfc, lc);
        else
          lighting_ref(P, epos, N, tfc, lc);
        src.x = lc[0]; src.y = lc[1]; src.z = lc[2];
        if (two_d) src.w = fminf(fmaxf(src.w, 0.0f), 1.0f);
      }
      pend = false;
      fin = true;
    }
    if (fin) {
      if (src.w != 0.0f && first_t == INFINITY) first_t = t_in + float(i) * ((t_out - t_in) / q);
      // Compositing.glsl:33-38 UnderCompositing
      const float w = 1.0f - c.w;
      c.x = fmaf(src.x * w, src.w, c.x);
      c.y = fmaf(src.y * w, src.w, c.y);
      c.z = fmaf(src.z * w, src.w, c.z);
      c.w = fmaf(src.w, w, c.w);
#pragma unroll
      for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
      ++epend;
      ++i;
      if (c.w >= 0.99f) break;
    }
  }
#else
  int i = 0;
  while (i < n) {
    // Phase 1: leap over empty macro cells.  Every voxel a trilinear lookup
    // from an empty cell can touch maps to TF entries with zero corrected
    // alpha, so those steps add exactly zero.  A cell at Chebyshev distance d
    // from the nearest non-empty cell sits in an empty cube of 2d - 1 cells;
    // the steps that provably stay inside it are skipped at once, with a
    // margin of 1/64 voxel for the rounding of the accumulated position
    // (< 2e-3 voxel across the largest cube); the position keeps the
    // reference's chain of additions.  Lanes of a warp reconverge before
    // shading.
    float u0, u1, u2;
    for (;;) {
      const float uu0 = fmaf(pos[0], vol.fn0, -0.5f);
      const float uu1 = fmaf(pos[1], vol.fn1, -0.5f);
      const float uu2 = fmaf(pos[2], vol.fn2, -0.5f);
      u0 = fminf(fmaxf(uu0, 0.0f), (vol.fn0 - 1.0f));
      u1 = fminf(fmaxf(uu1, 0.0f), (vol.fn1 - 1.0f));
      u2 = fminf(fmaxf(uu2, 0.0f), (vol.fn2 - 1.0f));
      if (!dist) break;
      const int cx = int(u0) >> kCellShift, cy = int(u1) >> kCellShift,
                cz = int(u2) >> kCellShift;
      const int dd = __ldg(&dist[(cz * ncy + cy) * ncx + cx]);
      if (dd == 0) break;
      int k = 0;
      if (uu0 == u0 && uu1 == u1 && uu2 == u2) {
        const int r = dd - 1;
        const float lo0 = float(max(cx - r, 0) << kCellShift),
                    lo1 = float(max(cy - r, 0) << kCellShift),
                    lo2 = float(max(cz - r, 0) << kCellShift);
        const float hi0 = float(min(cx + r + 1, ncx) << kCellShift),
                    hi1 = float(min(cy + r + 1, ncy) << kCellShift),
                    hi2 = float(min(cz + r + 1, ncz) << kCellShift);
        const float d0 = du0 > 0.0f ? hi0 - uu0 : uu0 - lo0;
        const float d1 = du1 > 0.0f ? hi1 - uu1 : uu1 - lo1;
        const float d2 = du2 > 0.0f ? hi2 - uu2 : uu2 - lo2;
        const float m = fminf(fminf((d0 - 0.015625f) * idu0, (d1 - 0.015625f) * idu1),
                              (d2 - 0.015625f) * idu2);
        k = m > 0.0f ? int(fminf(m, float(n - 1 - i))) : 0;
      }
      samples += uint32_t(k + 1);
      TVK_PROF(P, 4, 1);
      TVK_PROF(P, 5, k + 1);
      // the chain of k + 1 additions, unrolled (the same sums in order)
      if (lit) {
#pragma unroll 4
        for (int j = 0; j <= k; ++j) {
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            pos[a] = pos[a] + inc[a];
            epos[a] = epos[a] + einc[a];
          }
        }
      } else {
#pragma unroll 4
        for (int j = 0; j <= k; ++j) {
#pragma unroll
          for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
        }
      }
      i += k + 1;
      if (i >= n) break;
    }
    if (i >= n) break;
    // Phase 2: the reference's step i
    ++samples;
    ++shaded;
    Foot foot;
    const float v = centre_sample(vol, u0, u1, u2, foot) * im;
    const float u = v * P.trans_scale;
    float fx = floorf(u * W);
    fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
    float4 src;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
    bool need_grad = lit;
    if (two_d) need_grad = P.tf_col_nonzero[int(fx)] != 0;
    if (!two_d) {
      src = __ldg(&P.tf[int(fx)]);
      need_grad = lit && src.w != 0.0f;
    }
    if (need_grad) {
      ++graded;
      // Volume3D.glsl:43-54 (Yp sampled at -step.y)
      const float xp = shifted_x(vol, foot, clamp_u(pos[0] + vs0, vol.fn0, vol.n0)) * im;
      const float xm = shifted_x(vol, foot, clamp_u(pos[0] + (-vs0), vol.fn0, vol.n0)) * im;
      const float yp = shifted_y(vol, foot, clamp_u(pos[1] + (-vs1), vol.fn1, vol.n1)) * im;
      const float ym = shifted_y(vol, foot, clamp_u(pos[1] + vs1, vol.fn1, vol.n1)) * im;
      const float zp = shifted_z(vol, foot, clamp_u(pos[2] + vs2, vol.fn2, vol.n2)) * im;
      const float zm = shifted_z(vol, foot, clamp_u(pos[2] + (-vs2), vol.fn2, vol.n2)) * im;
      g0 = (xm - xp) / 2.0f;
      g1 = (yp - ym) / 2.0f;
      g2 = (zm - zp) / 2.0f;
    }
    if (two_d) {
      if (need_grad) {
        const float mag = len3(g0, g1, g2);
        const float w = 1.0f - mag * P.grad_scale;
        float fy = floorf(w * H);
        fy = fminf(fmaxf(fy, 0.0f), H - 1.0f);
        src = __ldg(&P.tf[int(fy) * P.tf_w + int(fx)]);
      } else {
        src = make_float4(0.f, 0.f, 0.f, 0.f);  // whole column transparent
      }
      need_grad = need_grad && lit && src.w != 0.0f;
    }
    if (lit && need_grad) {
      const float gs0 = g0 * P.domain_scale[0], gs1 = g1 * P.domain_scale[1],
                  gs2 = g2 * P.domain_scale[2];
      float N[3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
        N[r] = fmaf(P.norm_mat[r][2], gs2, fmaf(P.norm_mat[r][1], gs1, P.norm_mat[r][0] * gs0));
      const float l = len3(N[0], N[1], N[2]);
      if (l > 0.0f) {
        const float il = 1.0f / l;
        N[0] = N[0] * il; N[1] = N[1] * il; N[2] = N[2] * il;
      }
      const float tfc[3] = {src.x, src.y, src.z};
      float lc[3];
      if (P.light_model == TVK_LIGHT_BLINN_PHONG)
        lighting_bp(P, epos, N, tfc, lc);
      else
        lighting_ref(P, epos, N, tfc, lc);
      src.x = lc[0]; src.y = lc[1]; src.z = lc[2];
      if (two_d) src.w = fminf(fmaxf(src.w, 0.0f), 1.0f);
    }
    // the first sample that adds anything (the ray's first hit, a network input)
    if (src.w != 0.0f && first_t == INFINITY) first_t = t_in + float(i) * ((t_out - t_in) / q);
    // Compositing.glsl:33-38 UnderCompositing
    const float w = 1.0f - c.w;
    c.x = fmaf(src.x * w, src.w, c.x);
    c.y = fmaf(src.y * w, src.w, c.y);
    c.z = fmaf(src.z * w, src.w, c.z);
    c.w = fmaf(src.w, w, c.w);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      pos[a] = pos[a] + inc[a];
      epos[a] = epos[a] + einc[a];
    }
    ++i;
    if (c.w >= 0.99f) break;
  }
#endif
  return c;
}

// GLRaycaster-ISO-FS.glsl:51-105 for one brick: first step whose sample is
// >= fIsoval, RefineIsosurface.glsl:37-52, the eye-space hit interpolated by
// |hit - entry| / |exit - entry| in texture space, its non-linear depth and the
// normal at the refined position.  Returns false when the ray misses.
struct IsoHit {
  float pos[3];  // eye space
  float f;       // interpolation parameter (alpha of the hit buffer)
  float n[3];
  float depth;
  float enc_r, enc_gb;  // colour volumes: the packed hit colour
};

//
// kCV: the focus-surface pass of GLRaycaster-ISO-CV-FS.glsl:56-115 with
// isovalue `iso_cv`.  Its texture-space entry moves to the parameter p_start of
// the brick (the context hit, when that hit lies in this brick); the eye-space
// entry does not move (the shader blends vRayEntry with itself), so the step
// count and the eye-space hit interpolation keep the whole brick's entry.  The
// hit's depth (of the brick's exit) is not computed: along a ray the first
// brick with a focus hit wins the depth test.
template <class T, bool kCV = false, bool kTex = false>
__device__ __forceinline__ bool iso_brick(const RenderParams& P, const DevBrick& b,
                                          const float dir[3], float t_in, float t_out,
                                          IsoHit& h, uint32_t& samples, uint32_t& shaded,
                                          float iso_cv = 0.0f, float p_start = 0.0f) {
  float en[3], ex[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    en[a] = __half2float(__float2half_rn(dir[a] * t_in));
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row(b.tex[a], ex[0], ex[1], ex[2]);
  }
  if (kCV) {
#pragma unroll
    for (int a = 0; a < 3; ++a) tin[a] = tin[a] * (1.0f - p_start) + tout[a] * p_start;
  }
  const float len_tex = len3(tout[0] - tin[0], tout[1] - tin[1], tout[2] - tin[2]);
  const float q = len / b.step;
  if (!(q < P.max_q)) return false;
  const int n = int(q) + 1;
  float pos[3], inc[3];
  // the increment divides by the step count: a multiply by its reciprocal
  const float iq = 1.0f / q;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    inc[a] = (tout[a] - tin[a]) * iq;
    pos[a] = tin[a];
  }
  using View = typename std::conditional<kTex, TexView, BrickView<T>>::type;
  const View vol = brick_view<View, T>(P, b);
  const float im = P.inv_max_raw;
  const float iso = kCV ? iso_cv : P.iso_norm;
  // cells whose maximum stays below the isovalue cannot produce a hit
  const uint8_t* __restrict__ dist =
      (P.cell_dist && (!kCV || P.cv_cell_skip)) ? P.cell_dist + b.cell_off : nullptr;
  const int ncx = int(b.cells & 1023u), ncy = int((b.cells >> 10) & 1023u),
            ncz = int(b.cells >> 20);
  const float du0 = inc[0] * vol.fn0, du1 = inc[1] * vol.fn1, du2 = inc[2] * vol.fn2;
  const float idu0 = 1.0f / fabsf(du0), idu1 = 1.0f / fabsf(du1), idu2 = 1.0f / fabsf(du2);
  bool hit = false;
  int i = 0;
  while (i < n) {
    const float uu0 = fmaf(pos[0], vol.fn0, -0.5f);
    const float uu1 = fmaf(pos[1], vol.fn1, -0.5f);
    const float uu2 = fmaf(pos[2], vol.fn2, -0.5f);
    const float u0 = fminf(fmaxf(uu0, 0.0f), (vol.fn0 - 1.0f));
    const float u1 = fminf(fmaxf(uu1, 0.0f), (vol.fn1 - 1.0f));
    const float u2 = fminf(fmaxf(uu2, 0.0f), (vol.fn2 - 1.0f));
    if (dist) {
      const int cx = int(u0) >> kCellShift, cy = int(u1) >> kCellShift,
                cz = int(u2) >> kCellShift;
      const int dd = __ldg(&dist[(cz * ncy + cy) * ncx + cx]);
      if (dd != 0) {
        int k = 0;
        if (uu0 == u0 && uu1 == u1 && uu2 == u2) {
          const int r = dd - 1;
          const float lo0 = float(max(cx - r, 0) << kCellShift),
                      lo1 = float(max(cy - r, 0) << kCellShift),
                      lo2 = float(max(cz - r, 0) << kCellShift);
          const float hi0 = float(min(cx + r + 1, ncx) << kCellShift),
                      hi1 = float(min(cy + r + 1, ncy) << kCellShift),
                      hi2 = float(min(cz + r + 1, ncz) << kCellShift);
          const float d0 = du0 > 0.0f ? hi0 - uu0 : uu0 - lo0;
          const float d1 = du1 > 0.0f ? hi1 - uu1 : uu1 - lo1;
          const float d2 = du2 > 0.0f ? hi2 - uu2 : uu2 - lo2;
          const float m = fminf(fminf((d0 - 0.015625f) * idu0, (d1 - 0.015625f) * idu1),
                                (d2 - 0.015625f) * idu2);
          k = m > 0.0f ? int(fminf(m, float(n - 1 - i))) : 0;
        }
        samples += uint32_t(k + 1);
#pragma unroll 4
        for (int j = 0; j <= k; ++j) {
#pragma unroll
          for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
        }
        i += k + 1;
        continue;
      }
    }
    ++samples;
    ++shaded;
    if (vol.sample_u(u0, u1, u2) * im >= iso) { hit = true; break; }
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
    ++i;
  }
  if (!hit) return false;
  float d[3], cur[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    d[a] = inc[a] / 2.0f;
    cur[a] = pos[a] - d[a];
  }
  for (int k = 0; k < 5; ++k) {
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = d[a] / 2.0f;
    const bool above = vol.sample_raw(cur[0], cur[1], cur[2]) * im >= iso;
#pragma unroll
    for (int a = 0; a < 3; ++a) cur[a] = above ? cur[a] - d[a] : cur[a] + d[a];
  }
  h.f = len3(cur[0] - tin[0], cur[1] - tin[1], cur[2] - tin[2]) / len_tex;
#pragma unroll
  for (int a = 0; a < 3; ++a) h.pos[a] = en[a] * (1.0f - h.f) + ex[a] * h.f;
  h.depth = kCV ? 0.0f : P.proj_x + (P.proj_y / -h.pos[2]);
  const float vs0 = 1.0f / float(b.n[0]), vs1 = 1.0f / float(b.n[1]), vs2 = 1.0f / float(b.n[2]);
  const float xp = vol.sample_raw(cur[0] + vs0, cur[1], cur[2]) * im;
  const float xm = vol.sample_raw(cur[0] + (-vs0), cur[1], cur[2]) * im;
  const float yp = vol.sample_raw(cur[0], cur[1] + (-vs1), cur[2]) * im;
  const float ym = vol.sample_raw(cur[0], cur[1] + vs1, cur[2]) * im;
  const float zp = vol.sample_raw(cur[0], cur[1], cur[2] + vs2) * im;
  const float zm = vol.sample_raw(cur[0], cur[1], cur[2] + (-vs2)) * im;
  const float gs0 = ((xm - xp) / 2.0f) * P.domain_scale[0];
  const float gs1 = ((yp - ym) / 2.0f) * P.domain_scale[1];
  const float gs2 = ((zm - zp) / 2.0f) * P.domain_scale[2];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    h.n[r] = fmaf(P.norm_mat[r][2], gs2, fmaf(P.norm_mat[r][1], gs1, P.norm_mat[r][0] * gs0));
  const float l = len3(h.n[0], h.n[1], h.n[2]);
  if (l > 0.0f) { h.n[0] = h.n[0] / l; h.n[1] = h.n[1] / l; h.n[2] = h.n[2] / l; }
  return true;
}

// Lighting of Compose-FS.glsl:40-48 (and Compose-CV-FS.glsl:48-56) at the
// eye-space position pos with normal n: N.z made non-negative, diffuse from
// |N . -L|, specular exponent 8, clamped to [0, 1].
__device__ __forceinline__ void surface_lighting(const float pos[3], const float n[3],
                                                 const float* light_a, const float* diffuse,
                                                 const float* light_s, const float* L,
                                                 float c[3]) {
  const float N0 = n[0], N1 = n[1], N2 = fabsf(n[2]);
  const float p0 = 0.0f - pos[0], p1 = 0.0f - pos[1], p2 = 0.0f - pos[2];
  const float lp = len3(p0, p1, p2);
  const float V0 = p0 / lp, V1 = p1 / lp, V2 = p2 / lp;
  const float d = (N0 * V0 + N1 * V1) + N2 * V2;
  float R0 = V0 - (2.0f * d) * N0, R1 = V1 - (2.0f * d) * N1, R2 = V2 - (2.0f * d) * N2;
  const float lr = len3(R0, R1, R2);
  R0 = R0 / lr; R1 = R1 / lr; R2 = R2 / lr;
  const float nl0 = -L[0], nl1 = -L[1], nl2 = -L[2];
  const float diff = fmaxf(fabsf((N0 * nl0 + N1 * nl1) + N2 * nl2), 0.0f);
  const float spec = pow_int_or_real(fmaxf((R0 * L[0] + R1 * L[1]) + R2 * L[2], 0.0f), 8.0f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float x = light_a[i] + diffuse[i] * diff;
    x = x + light_s[i] * spec;
    c[i] = fminf(fmaxf(x, 0.0f), 1.0f);
  }
}

// Compose-FS.glsl:40-63: lighting of the nearest hit.
__device__ __forceinline__ float4 iso_compose(const RenderParams& P, const IsoHit& h) {
  const float N0 = h.n[0], N1 = h.n[1], N2 = fabsf(h.n[2]);
  const float p0 = 0.0f - h.pos[0], p1 = 0.0f - h.pos[1], p2 = 0.0f - h.pos[2];
  const float lp = len3(p0, p1, p2);
  const float V0 = p0 / lp, V1 = p1 / lp, V2 = p2 / lp;
  const float d = (N0 * V0 + N1 * V1) + N2 * V2;
  float R0 = V0 - (2.0f * d) * N0, R1 = V1 - (2.0f * d) * N1, R2 = V2 - (2.0f * d) * N2;
  const float lr = len3(R0, R1, R2);
  R0 = R0 / lr; R1 = R1 / lr; R2 = R2 / lr;
  const float* L = P.light_dir;
  const float nl0 = -L[0], nl1 = -L[1], nl2 = -L[2];
  const float diff = fmaxf(fabsf((N0 * nl0 + N1 * nl1) + N2 * nl2), 0.0f);
  const float spec = pow_int_or_real(fmaxf((R0 * L[0] + R1 * L[1]) + R2 * L[2], 0.0f), 8.0f);
  float c[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float x = P.light_a[i] + P.iso_diffuse[i] * diff;
    x = x + P.light_s[i] * spec;
    c[i] = fminf(fmaxf(x, 0.0f), 1.0f);
  }
  return make_float4(c[0], c[1], c[2], 1.0f);
}

// Normal from the red channel's central differences (Volume3D.glsl:43-60:
// sampleVolume(...).x of a colour volume), in eye space, safely normalised.
__device__ __forceinline__ void color_normal(const RenderParams& P, const ColorView& vol,
                                             const float pos[3], float N[3]) {
  const float vs0 = 1.0f / vol.fn0, vs1 = 1.0f / vol.fn1, vs2 = 1.0f / vol.fn2;
  const float im = P.inv_max_raw;
  const float xp = vol.sample_raw<1>(pos[0] + vs0, pos[1], pos[2]).x * im;
  const float xm = vol.sample_raw<1>(pos[0] + (-vs0), pos[1], pos[2]).x * im;
  const float yp = vol.sample_raw<1>(pos[0], pos[1] + (-vs1), pos[2]).x * im;
  const float ym = vol.sample_raw<1>(pos[0], pos[1] + vs1, pos[2]).x * im;
  const float zp = vol.sample_raw<1>(pos[0], pos[1], pos[2] + vs2).x * im;
  const float zm = vol.sample_raw<1>(pos[0], pos[1], pos[2] + (-vs2)).x * im;
  const float gs0 = ((xm - xp) / 2.0f) * P.domain_scale[0];
  const float gs1 = ((yp - ym) / 2.0f) * P.domain_scale[1];
  const float gs2 = ((zm - zp) / 2.0f) * P.domain_scale[2];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    N[r] = fmaf(P.norm_mat[r][2], gs2, fmaf(P.norm_mat[r][1], gs1, P.norm_mat[r][0] * gs0));
  const float l = len3(N[0], N[1], N[2]);
  if (l > 0.0f) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
}

// One brick of a colour volume in 1D mode (GLRaycaster-1D-FS /
// -1D-light-FS with VRender1D-Color.glsl:44-53 / VRender1DLit-Color.glsl:
// 44-62): the filtered RGBA times the TF entry at (r + g + b) / 3, opacity
// correction of the product's alpha (P.tf holds uncorrected entries), lit
// with the product's colour as the diffuse colour.  No macro-cell leaps:
// colour bricks are never empty (AbstrRenderer::ContainsData).
__device__ __forceinline__ float4 march_brick_color(const RenderParams& P, const DevBrick& b,
                                                    const float dir[3], float t_in, float t_out,
                                                    uint32_t& samples, uint32_t& shaded,
                                                    uint32_t& graded, float& first_t) {
  float en[3], ex[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    en[a] = __half2float(__float2half_rn(dir[a] * t_in));
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const float q = len / b.step;
  float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(q < P.max_q)) {
    atomicAdd(&P.counters[2], 1ull);
    return c;
  }
  const int n = int(q) + 1;
  float pos[3], inc[3], epos[3], einc[3];
  // the increment divides by the step count: a multiply by its reciprocal
  const float iq = 1.0f / q;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    inc[a] = (tout[a] - tin[a]) * iq;
    pos[a] = tin[a];
    epos[a] = en[a];
  }
  const float ilen = 1.0f / len;
  einc[0] = (dx * ilen) * b.step;
  einc[1] = (dy * ilen) * b.step;
  einc[2] = (dz * ilen) * b.step;
  const ColorView vol = color_view(P, b);
  const float im = P.inv_max_raw;
  const float W = float(P.tf_w);
  const bool lit = P.lighting != 0;
  for (int i = 0; i < n; ++i) {
    ++samples;
    ++shaded;
    const float4 raw = vol.sample_raw<15>(pos[0], pos[1], pos[2]);
    const float v0 = raw.x * im, v1 = raw.y * im, v2 = raw.z * im, v3 = raw.w * im;
    const float u = ((v0 + v1) + v2) / 3.0f;
    float fx = floorf(u * W);
    fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
    const float4 t = __ldg(&P.tf[int(fx)]);
    float4 src = make_float4(v0 * t.x, v1 * t.y, v2 * t.z, v3 * t.w);
    src.w = 1.0f - pow01(1.0f - src.w, P.step_scale);
    if (lit && src.w != 0.0f) {
      ++graded;
      float N[3];
      color_normal(P, vol, pos, N);
      const float tfc[3] = {src.x, src.y, src.z};
      float lc[3];
      if (P.light_model == TVK_LIGHT_BLINN_PHONG)
        lighting_bp(P, epos, N, tfc, lc);
      else
        lighting_ref(P, epos, N, tfc, lc);
      src.x = lc[0]; src.y = lc[1]; src.z = lc[2];
    }
    if (src.w != 0.0f && first_t == INFINITY) first_t = t_in + float(i) * ((t_out - t_in) / q);
    const float w = 1.0f - c.w;
    c.x = fmaf(src.x * w, src.w, c.x);
    c.y = fmaf(src.y * w, src.w, c.y);
    c.z = fmaf(src.z * w, src.w, c.z);
    c.w = fmaf(src.w, w, c.w);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      pos[a] = pos[a] + inc[a];
      epos[a] = epos[a] + einc[a];
    }
    if (c.w >= 0.99f) break;
  }
  return c;
}

// GLRaycaster-Color-FS.glsl for one brick: the first step whose alpha is >=
// fIsoval, RefineIsosurface.glsl on the red channel (its sampleVolume(...).x),
// the normal from the red channel, and the colour at the unrefined step,
// packed as the shader packs it: red + 1 in the hit's alpha, floor(green *
// 512) + blue in the normal's alpha.
__device__ __forceinline__ bool iso_brick_color(const RenderParams& P, const DevBrick& b,
                                                const float dir[3], float t_in, float t_out,
                                                IsoHit& h, uint32_t& samples,
                                                uint32_t& shaded) {
  float en[3], ex[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    en[a] = __half2float(__float2half_rn(dir[a] * t_in));
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const float len_tex = len3(tout[0] - tin[0], tout[1] - tin[1], tout[2] - tin[2]);
  const float q = len / b.step;
  if (!(q < P.max_q)) return false;
  const int n = int(q) + 1;
  float pos[3], inc[3];
  // the increment divides by the step count: a multiply by its reciprocal
  const float iq = 1.0f / q;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    inc[a] = (tout[a] - tin[a]) * iq;
    pos[a] = tin[a];
  }
  const ColorView vol = color_view(P, b);
  const float im = P.inv_max_raw;
  const float iso = P.iso_norm;
  bool hit = false;
  for (int i = 0; i < n; ++i) {
    ++samples;
    ++shaded;
    if (vol.sample_raw<8>(pos[0], pos[1], pos[2]).w * im >= iso) { hit = true; break; }
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
  }
  if (!hit) return false;
  float d[3], cur[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    d[a] = inc[a] / 2.0f;
    cur[a] = pos[a] - d[a];
  }
  for (int k = 0; k < 5; ++k) {
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = d[a] / 2.0f;
    const bool above = vol.sample_raw<1>(cur[0], cur[1], cur[2]).x * im >= iso;
#pragma unroll
    for (int a = 0; a < 3; ++a) cur[a] = above ? cur[a] - d[a] : cur[a] + d[a];
  }
  const float4 col = vol.sample_raw<7>(pos[0], pos[1], pos[2]);
  h.f = len3(cur[0] - tin[0], cur[1] - tin[1], cur[2] - tin[2]) / len_tex;
#pragma unroll
  for (int a = 0; a < 3; ++a) h.pos[a] = en[a] * (1.0f - h.f) + ex[a] * h.f;
  h.depth = P.proj_x + (P.proj_y / -h.pos[2]);
  color_normal(P, vol, cur, h.n);
  h.enc_r = col.x * im + 1.0f;
  h.enc_gb = floorf((col.y * im) * 512.0f) + col.z * im;
  return true;
}

// Compose-Color-FS.glsl:60-88: the colour recovered from the two packed
// channels lights the hit (diffuse = colour * the diffuse light).
__device__ __forceinline__ float4 iso_compose_color(const RenderParams& P, const IsoHit& h) {
  const float rgb[3] = {h.enc_r - 1.0f, floorf(h.enc_gb / 2.0f) / 256.0f,
                        h.enc_gb - floorf(h.enc_gb)};
  const float n[3] = {h.n[0], h.n[1], fabsf(h.n[2])};
  float dcol[3], c[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dcol[i] = rgb[i] * P.light_d[i];
  surface_lighting(h.pos, n, P.light_a, dcol, P.light_s, P.light_dir, c);
  return make_float4(c[0], c[1], c[2], 1.0f);
}

constexpr uint32_t kCandChunk = 1024;

// Conservative: can any pixel ray of the 16x8 tile at (tx0, ty0) meet brick b?
// A ray through a pixel centre meets the box only if the centre lies in the
// box's projection, hence in the bounding rectangle of its projected corners;
// a 2-pixel margin covers rounding.  Bricks reaching behind the near plane
// are always kept (the per-ray slab test decides).
__device__ __forceinline__ bool footprint_touches_tile(const RenderParams& P, const DevBrick& b,
                                                       float tx0, float ty0, float span_x,
                                                       float span_y) {
  float xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  const float hw = 0.5f * float(P.width), hh = 0.5f * float(P.height);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float x = (c & 1) ? b.pmax[0] : b.pmin[0];
    const float y = (c & 2) ? b.pmax[1] : b.pmin[1];
    const float z = (c & 4) ? b.pmax[2] : b.pmin[2];
    const float ex = fmaf(P.mv[0][0], x, fmaf(P.mv[0][1], y, fmaf(P.mv[0][2], z, P.mv[0][3])));
    const float ey = fmaf(P.mv[1][0], x, fmaf(P.mv[1][1], y, fmaf(P.mv[1][2], z, P.mv[1][3])));
    const float ez = fmaf(P.mv[2][0], x, fmaf(P.mv[2][1], y, fmaf(P.mv[2][2], z, P.mv[2][3])));
    if (ez > -0.5f * P.znear) return true;
    const float iz = 1.0f / (-ez);
    const float sx = (ex * iz / P.kx + 1.0f) * hw - 0.5f;
    const float sy = (ey * iz / P.ky + 1.0f) * hh - 0.5f;
    xmin = fminf(xmin, sx); xmax = fmaxf(xmax, sx);
    ymin = fminf(ymin, sy); ymax = fmaxf(ymax, sy);
  }
  return xmax >= tx0 - 2.0f && xmin <= tx0 + span_x + 2.0f && ymax >= ty0 - 2.0f &&
         ymin <= ty0 + span_y + 2.0f;
}

// Shared-memory state of one 16x8-pixel tile: the candidate brick list.
struct TileShared {
  uint16_t cand[kCandChunk];
  uint32_t warp_cnt[4];
  uint32_t n_cand;
};

// One tile of (16 * kRPT) x 8 pixels (tile coordinates bx, by) of the frame P
// describes; all 128 threads of the CTA take part, each marching kRPT rays
// one after the other (pixel columns 16 r + ...).  kIso: isosurface mode
// (nearest refined hit + compose); otherwise the compositing modes (1D/2D TF,
// lit or unlit).  Every pixel's value does not depend on kRPT.  kCV (with
// kIso): ClearView, both surfaces' hits go to P.cv_hits for cv_compose.
template <class T, bool kIso, int kRPT, bool kCV = false, bool kTex = false>
__device__ __forceinline__ void render_tile(const RenderParams& P, uint32_t bx, uint32_t by,
                                            TileShared& sh) {
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t kW = 16 * kRPT;
  constexpr bool kColor = std::is_same<T, uchar4>::value;  // RGBA8 colour volume

  // The host lists the visible bricks in a front-to-back order that holds for
  // every ray (increasing L1 grid distance from the eye's brick cell, which
  // strictly grows whenever a ray crosses into the next brick).  Each CTA
  // keeps, in that order, the bricks whose screen footprint can touch its
  // tile; each ray then marches those its own slab test hits.
  const float tx0 = float(bx * kW * P.stride + P.off_x), ty0 = float(by * 8 * P.stride + P.off_y);
  const float span_x = float((kW - 1) * P.stride), span_y = float(7 * P.stride);

  float4 frame[kRPT];
  float first_t[kRPT];
  uint32_t ray_samples[kRPT];
  uint32_t shaded = 0, graded = 0;
  constexpr bool iso_mode = kIso;
  IsoHit best[kRPT];
  float best_depth[kRPT];  // depth buffer cleared to 1, test DF_LESS
  bool have_hit[kRPT];
  IsoHit focus[kRPT];      // ClearView: the focus surface's hit
  bool have_focus[kRPT];
#pragma unroll
  for (int r = 0; r < kRPT; ++r) {
    frame[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    first_t[r] = INFINITY;
    ray_samples[r] = 0;
    best_depth[r] = 1.0f;
    have_hit[r] = false;
    have_focus[r] = false;
  }
  for (uint32_t base = 0; base < P.n_bricks; base += kCandChunk) {
    const uint32_t end = min(P.n_bricks, base + kCandChunk);
    __syncthreads();  // the previous chunk's list is no longer read
    if (tid == 0) sh.n_cand = 0;
    for (uint32_t s = base; s < end; s += blockDim.x) {
      const uint32_t i = s + tid;
      const bool keep = i < end && footprint_touches_tile(P, P.bricks[i], tx0, ty0, span_x, span_y);
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      __syncthreads();
      if (lane == 0) sh.warp_cnt[warp] = __popc(m);
      __syncthreads();
      uint32_t off = sh.n_cand;
      for (uint32_t w2 = 0; w2 < warp; ++w2) off += sh.warp_cnt[w2];
      if (keep) sh.cand[off + __popc(m & ((1u << lane) - 1u))] = uint16_t(i - base);
      __syncthreads();
      if (tid == 0)
        sh.n_cand += sh.warp_cnt[0] + sh.warp_cnt[1] + sh.warp_cnt[2] + sh.warp_cnt[3];
    }
    __syncthreads();
    const uint32_t nc = sh.n_cand;
#pragma unroll 1
    for (int r = 0; r < kRPT; ++r) {
      const uint32_t px = bx * kW + uint32_t(r) * 16 + (warp & 1) * 8 + (lane & 7);
      const uint32_t py = by * 8 + (warp >> 1) * 4 + (lane >> 3);
      // the frame pixel this ray marches (stride 1, offset 0 for whole frames)
      const uint32_t fx = px * P.stride + P.off_x, fy = py * P.stride + P.off_y;
      const bool active = px < P.out_w && py < P.out_h && fx < P.width && fy < P.height;
      if (!active) continue;
      const float nx = (float(fx) + 0.5f) * P.inv_w2 - 1.0f;
      const float ny = (float(fy) + 0.5f) * P.inv_h2 - 1.0f;
      const float dir[3] = {nx * P.kx, ny * P.ky, -1.0f};
      float o[3], inv[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        o[a] = P.inv[a][3];
        const float d = fmaf(P.inv[a][2], dir[2], fmaf(P.inv[a][1], dir[1], P.inv[a][0] * dir[0]));
        inv[a] = 1.0f / d;
      }
      // the clip plane keeps the ray parameters [clip_lo, clip_hi]
      // (GLRaycaster.cpp:328-337 caps each brick box with the plane)
      float clip_lo = -INFINITY, clip_hi = INFINITY;
      if (P.clip_on) {
        const float cs = fmaf(P.clip_eye[2], dir[2], fmaf(P.clip_eye[1], dir[1],
                                                          P.clip_eye[0] * dir[0]));
        if (cs > 0.0f) clip_hi = -P.clip_eye[3] / cs;
        else if (cs < 0.0f) clip_lo = -P.clip_eye[3] / cs;
        else if (P.clip_eye[3] > 0.0f) { clip_lo = INFINITY; clip_hi = -INFINITY; }
      }
      uint32_t samples = ray_samples[r];
      for (uint32_t c = 0; c < nc; ++c) {
        if (frame[r].w >= P.frame_ert) break;
        const DevBrick& bg = P.bricks[base + sh.cand[c]];
        TVK_PROF(P, 6, 1);
        float tn = -INFINITY, tf = INFINITY;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float t0 = (__ldg(&bg.pmin[a]) - o[a]) * inv[a];
          const float t1 = (__ldg(&bg.pmax[a]) - o[a]) * inv[a];
          tn = fmaxf(tn, fminf(t0, t1));
          tf = fminf(tf, fmaxf(t0, t1));
        }
        const float t_near = fmaxf(tn, P.znear);
        if (!(tf > t_near) || tf > P.zfar) continue;
        const float ti = fmaxf(t_near, clip_lo), tc = fminf(tf, clip_hi);
        if (!(tc > ti)) continue;
        const DevBrick b = bg;
        if (iso_mode) {
          // A later brick's hit lies beyond its (RGBA16F-rounded) entry, so
          // once that entry is behind the nearest hit it cannot pass the
          // depth test; bricks come in increasing entry order along the ray.
          const bool settled = have_hit[r] && ti * (1.0f - 2e-3f) - 1e-4f > -best[r].pos[2];
          if constexpr (kColor) {
            if (settled) break;
            IsoHit h;
            if (iso_brick_color(P, b, dir, ti, tc, h, samples, shaded) &&
                h.depth < best_depth[r]) {
              best[r] = h;
              best_depth[r] = h.depth;
              have_hit[r] = true;
            }
            continue;
          } else {
          if (!kCV) {
            if (settled) break;
            IsoHit h;
            if (iso_brick<T, false, kTex>(P, b, dir, ti, tc, h, samples, shaded) &&
                h.depth < best_depth[r]) {
              best[r] = h;
              best_depth[r] = h.depth;
              have_hit[r] = true;
            }
            continue;
          }
          // ClearView (GLRaycaster.cpp:421-436): per brick the context pass,
          // then the focus pass, which starts at the context hit when the
          // nearest context hit so far is this brick's (its tile ID).  The
          // focus pass writes the brick's exit depth, so the first brick
          // along the ray with a focus hit keeps it.
          if (settled && have_focus[r]) break;
          bool here = false;
          if (!settled) {
            IsoHit h;
            if (iso_brick<T, false, kTex>(P, b, dir, ti, tc, h, samples, shaded) &&
                h.depth < best_depth[r]) {
              best[r] = h;
              best_depth[r] = h.depth;
              have_hit[r] = true;
              here = true;
            }
          }
          if (!have_focus[r] &&
              iso_brick<T, true>(P, b, dir, ti, tc, focus[r], samples, shaded, P.cv_iso,
                                 here ? best[r].f : 0.0f))
            have_focus[r] = true;
          continue;
          }
        }
        float4 col;
        if constexpr (kColor)
          col = march_brick_color(P, b, dir, ti, tc, samples, shaded, graded, first_t[r]);
        else
          col = march_brick<T, kTex>(P, b, dir, ti, tc, samples, shaded, graded, first_t[r]);
        TVK_PROF(P, 7, 1);
        const float w = 1.0f - frame[r].w;
        frame[r].x = fmaf(col.x, w, frame[r].x);
        frame[r].y = fmaf(col.y, w, frame[r].y);
        frame[r].z = fmaf(col.z, w, frame[r].z);
        frame[r].w = fmaf(col.w, w, frame[r].w);
      }
      ray_samples[r] = samples;
    }
  }
  uint32_t samples = 0;
#pragma unroll
  for (int r = 0; r < kRPT; ++r) {
    const uint32_t px = bx * kW + uint32_t(r) * 16 + (warp & 1) * 8 + (lane & 7);
    const uint32_t py = by * 8 + (warp >> 1) * 4 + (lane >> 3);
    const uint32_t fx = px * P.stride + P.off_x, fy = py * P.stride + P.off_y;
    const bool active = px < P.out_w && py < P.out_h && fx < P.width && fy < P.height;
    // Compose-FS.glsl:58-61: no hit, or an interpolation parameter of exactly
    // 0, leaves the pixel empty
    float4 out = frame[r];
    if constexpr (kColor) {
      if (iso_mode && have_hit[r]) {
        // the packed red + 1 is the hit buffer's alpha: never 0
        out = iso_compose_color(P, best[r]);
        first_t[r] = -best[r].pos[2];
      }
    } else if (iso_mode && have_hit[r] && best[r].f != 0.0f) {
      if (!kCV) out = iso_compose(P, best[r]);
      first_t[r] = -best[r].pos[2];
    }
    if (active) {
      const size_t pix = size_t(py) * P.out_w + px;
      if (kCV) {
        // the two hit buffers of GLRenderer (m_pFBOIsoHit, m_pFBOCVHit):
        // position + interpolation parameter, normal; cleared to zero
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        float4* H = P.cv_hits + 4 * pix;
        H[0] = have_hit[r] ? make_float4(best[r].pos[0], best[r].pos[1], best[r].pos[2], best[r].f) : z;
        H[1] = have_hit[r] ? make_float4(best[r].n[0], best[r].n[1], best[r].n[2], 0.f) : z;
        H[2] = have_focus[r] ? make_float4(focus[r].pos[0], focus[r].pos[1], focus[r].pos[2],
                                           focus[r].f) : z;
        H[3] = have_focus[r] ? make_float4(focus[r].n[0], focus[r].n[1], focus[r].n[2], 0.f) : z;
      } else {
        P.out[pix] = out;
      }
      if (P.spp) P.spp[pix] = ray_samples[r];
      if (P.depth) P.depth[pix] = first_t[r] == INFINITY ? 0.0f : 1.0f / (1.0f + first_t[r]);
    }
    samples += ray_samples[r];
  }
  // frame totals: one atomic per warp
  const uint32_t s = __reduce_add_sync(0xffffffffu, samples);
  const uint32_t shd = __reduce_add_sync(0xffffffffu, shaded);
  const uint32_t gr = __reduce_add_sync(0xffffffffu, graded);
  if (lane == 0) {
    atomicAdd(&P.counters[0], (unsigned long long)s);
    atomicAdd(&P.counters[1], (unsigned long long)shd);
    atomicAdd(&P.counters[3], (unsigned long long)gr);
  }
}

// Rays per thread of the single-frame kernel (tiles of 16 x TVK_RAYCAST_RPT by 8 pixels).
#ifndef TVK_RAYCAST_RPT
#define TVK_RAYCAST_RPT 1
#endif

template <class T, bool kIso, bool kCV = false, bool kTex = false>
__global__ void __launch_bounds__(128, TVK_RAYCAST_MIN_BLOCKS) raycast_kernel(const RenderParams P) {
  __shared__ TileShared sh;
  render_tile<T, kIso, TVK_RAYCAST_RPT, kCV, kTex>(P, blockIdx.x, blockIdx.y, sh);
}

// Compose-CV-FS.glsl:49-108, one thread per pixel.  Neighbour normals are
// read as the shader's GL_NEAREST / GL_CLAMP lookups one texel away in a
// target of fbo_w x fbo_h: clamped at the target's edges, zero (the cleared
// buffer) beyond a reduced frame's right and top edges inside the target.
__global__ void cv_compose_kernel(const CvComposeParams C) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= C.w || y >= C.h) return;
  const size_t pix = size_t(y) * C.w + x;
  const float4 hp = C.hits[4 * pix];
  if (hp.w == 0.0f) {
    C.out[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float4 hn = C.hits[4 * pix + 1];
  const float pos[3] = {hp.x, hp.y, hp.z}, n[3] = {hn.x, hn.y, hn.z};
  float ctx[3];
  surface_lighting(pos, n, C.light_a, C.diffuse_context, C.light_s, C.light_dir, ctx);
  auto normal_at = [&](int nx, int ny) {
    nx = min(max(nx, 0), int(C.fbo_w) - 1);
    ny = min(max(ny, 0), int(C.fbo_h) - 1);
    if (nx >= int(C.w) || ny >= int(C.h)) return make_float4(0.f, 0.f, 0.f, 0.f);
    return C.hits[4 * (size_t(ny) * C.w + nx) + 1];
  };
  const float4 n_r = normal_at(int(x) + 1, int(y)), n_l = normal_at(int(x) - 1, int(y));
  const float4 n_u = normal_at(int(x), int(y) + 1), n_d = normal_at(int(x), int(y) - 1);
  const float c0 = ((fabsf(n_r.x - n[0]) + fabsf(n_l.x - n[0])) + fabsf(n_u.x - n[0])) +
                   fabsf(n_d.x - n[0]);
  const float c1 = ((fabsf(n_r.y - n[1]) + fabsf(n_l.y - n[1])) + fabsf(n_u.y - n[1])) +
                   fabsf(n_d.y - n[1]);
  const float c2 = ((fabsf(n_r.z - n[2]) + fabsf(n_l.z - n[2])) + fabsf(n_u.z - n[2])) +
                   fabsf(n_d.z - n[2]);
  const float curvature = len3(c0, c1, c2);
  const float dist_w = len3(pos[0] - C.pick[0], pos[1] - C.pick[1], pos[2] - C.pick[2]) * C.size;
  const float blend =
      fminf(fmaxf(fmaxf(curvature * C.context_scale, fminf(fmaxf(dist_w, 0.0f), 1.0f)), 0.0f),
            1.0f);
  float foc[4] = {0.f, 0.f, 0.f, 0.f};
  const float4 fp = C.hits[4 * pix + 2];
  if (fp.w != 0.0f) {
    const float4 fn = C.hits[4 * pix + 3];
    const float fpos[3] = {fp.x, fp.y, fp.z}, fnrm[3] = {fn.x, fn.y, fn.z};
    surface_lighting(fpos, fnrm, C.light_a, C.diffuse_focus, C.light_s, C.light_dir, foc);
    foc[3] = 1.0f;
  }
  const float ctx4[4] = {ctx[0], ctx[1], ctx[2], 1.0f};
  float col[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
    col[i] = fminf(fmaxf(ctx4[i] * blend + foc[i] * (1.0f - blend), 0.0f), 1.0f);
  const float dark =
      0.5f * (1.0f - fminf(fmaxf(fabsf(dist_w - 1.0f) * C.border_scale, 0.0f), 1.0f));
  C.out[pix] = make_float4(col[0] - dark, col[1] - dark, col[2] - dark, col[3]);
}

// Many frames in one persistent launch (the reference renders render regions
// and renderers one after another, GLRenderer.cpp:622-660).  Work items are
// (frame, tile) pairs numbered frame by frame (L.tile_first is the prefix sum
// of tiles per frame); each CTA takes the next item from a global counter and
// renders the tile with the same code as raycast_kernel, reading the frame's
// parameters from the launch's parameter block, so every pixel is bit-for-bit
// the single-frame result.
template <class T, bool kIso, int kRPT>
__global__ void __launch_bounds__(128, TVK_RAYCAST_MIN_BLOCKS)
raycast_batch_kernel(const __grid_constant__ BatchLaunch L, uint32_t* __restrict__ next_item) {
  __shared__ TileShared sh;
  __shared__ uint32_t item, frame_idx;
  const uint32_t n_items = L.tile_first[L.n_frames];
  for (;;) {
    __syncthreads();  // the previous item's shared state is no longer read
    if (threadIdx.x == 0) {
      const uint32_t it = atomicAdd(next_item, 1u);
      // frame whose tile range holds the item (binary search of the prefix)
      uint32_t lo = 0, hi = L.n_frames;
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (L.tile_first[mid] <= it) lo = mid; else hi = mid;
      }
      item = it;
      frame_idx = lo;
    }
    __syncthreads();
    const uint32_t it = item;
    if (it >= n_items) return;
    const uint32_t f = frame_idx;
    const RenderParams& P = L.frames[f];
    const uint32_t local = it - L.tile_first[f];
    const uint32_t tiles_x = (P.out_w + 16 * kRPT - 1) / (16 * kRPT);
    render_tile<T, kIso, kRPT>(P, local % tiles_x, local / tiles_x, sh);
  }
}

// TF entry a raw value maps to, exactly as the march computes it
__device__ __forceinline__ int tf_index(uint32_t raw, float im, float ts, float W) {
  const float v = float(raw) * im;
  const float u = v * ts;
  float fx = floorf(u * W);
  fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
  return int(fx);
}

__global__ void empty_cells_kernel(const EmptyCellParams P) {
  // one thread per 32-cell word of brick blockIdx.y
  const uint32_t b = blockIdx.y;
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t ncell = P.cell_counts[b];
  if (w * 32 >= ncell) return;
  const uint32_t* cm = P.cell_minmax + P.cell_offsets[b];
  const float W = float(P.tf_w);
  uint32_t bits = 0;
  for (uint32_t j = 0; j < 32 && w * 32 + j < ncell; ++j) {
    const uint32_t mm = cm[w * 32 + j];
    if (P.iso_mode) {
      // samples never exceed the cell maximum, so below fIsoval means no hit
      if (float(mm >> 16) * P.inv_max_raw < P.iso_norm) bits |= 1u << j;
      continue;
    }
    // trilinear results lie in [min, max] and the index is monotone in the
    // value, so the cell reaches exactly the entries lo..hi
    const int lo = tf_index(mm & 0xffffu, P.inv_max_raw, P.trans_scale, W);
    const int hi = tf_index(mm >> 16, P.inv_max_raw, P.trans_scale, W);
    if (P.nz_prefix[hi + 1] == P.nz_prefix[lo]) bits |= 1u << j;
  }
  P.bits[P.word_offsets[b] + w] = bits;
}

}  // namespace

void launch_empty_cells(const EmptyCellParams& p, uint32_t max_words_per_brick, cudaStream_t s,
                        uint64_t* launches) {
  const dim3 grid((max_words_per_brick + 127) / 128, uint32_t(p.n_bricks));
  empty_cells_kernel<<<grid, 128, 0, s>>>(p);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

namespace {

// One pass of the separable Chebyshev distance transform: one thread per line
// of cells along `axis` of brick brick_base + blockIdx.y.  Pass x measures the
// 1D distance to the nearest non-empty cell of the line (forward and backward
// sweeps); passes y and z take min over j of max(|i - j|, previous(j)) for
// |i - j| < kCellDistCap.  Cells outside the brick count as empty.
__global__ void cell_dist_kernel(const CellDistParams P, int axis, uint32_t brick_base) {
  const uint32_t b = brick_base + blockIdx.y;
  if (b >= P.n_bricks) return;
  const uint32_t dims = P.cell_dims[b];
  const uint32_t nx = dims & 1023u, ny = (dims >> 10) & 1023u, nz = dims >> 20;
  const uint32_t len = axis == 0 ? nx : (axis == 1 ? ny : nz);
  const uint32_t lines = axis == 0 ? ny * nz : (axis == 1 ? nx * nz : nx * ny);
  const uint32_t line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= lines) return;
  uint64_t base;
  uint32_t stride;
  if (axis == 0) {
    base = uint64_t(line) * nx;
    stride = 1;
  } else if (axis == 1) {
    base = uint64_t(line / nx) * nx * ny + line % nx;
    stride = nx;
  } else {
    base = line;
    stride = nx * ny;
  }
  const uint64_t co = P.cell_offsets[b];
  uint8_t* out = P.out + co;
  if (axis == 0) {
    const uint32_t* bits = P.bits + P.word_offsets[b];
    int d = kCellDistCap;
    for (uint32_t i = 0; i < len; ++i) {
      const uint64_t c = base + i;
      d = ((bits[c >> 5] >> (c & 31)) & 1u) ? min(d + 1, kCellDistCap) : 0;
      out[c] = uint8_t(d);
    }
    d = kCellDistCap;
    for (int i = int(len) - 1; i >= 0; --i) {
      const uint64_t c = base + uint64_t(i);
      d = ((bits[c >> 5] >> (c & 31)) & 1u) ? min(d + 1, kCellDistCap) : 0;
      out[c] = uint8_t(min(int(out[c]), d));
    }
    return;
  }
  const uint8_t* in = P.in + co;
  for (int i = 0; i < int(len); ++i) {
    // grow the window outward from i: a cell r away gives at least r, so the
    // search ends once r reaches the best value found
    int best = min(kCellDistCap, int(in[base + uint64_t(i) * stride]));
    for (int r = 1; r < best; ++r) {
      if (i - r >= 0) best = min(best, max(r, int(in[base + uint64_t(i - r) * stride])));
      if (i + r < int(len)) best = min(best, max(r, int(in[base + uint64_t(i + r) * stride])));
    }
    out[base + uint64_t(i) * stride] = uint8_t(best);
  }
}

}  // namespace

void launch_cell_dist(const CellDistParams& p, const uint32_t max_lines[3], uint8_t* tmp_a,
                      uint8_t* tmp_b, uint8_t* dist, cudaStream_t s, uint64_t* launches) {
  uint8_t* outs[3] = {tmp_a, tmp_b, dist};
  const uint8_t* ins[3] = {nullptr, tmp_a, tmp_b};
  for (int axis = 0; axis < 3; ++axis) {
    CellDistParams q = p;
    q.in = ins[axis];
    q.out = outs[axis];
    const uint32_t gx = std::max(1u, (max_lines[axis] + 127) / 128);
    for (uint64_t base = 0; base < p.n_bricks; base += 65535) {
      const uint32_t gy = uint32_t(std::min<uint64_t>(65535, p.n_bricks - base));
      cell_dist_kernel<<<dim3(gx, gy), 128, 0, s>>>(q, axis, uint32_t(base));
      TVK_CUDA(cudaGetLastError());
      ++*launches;
    }
  }
}

namespace {

// ================================================================= GridLeaper
//
// One GLGridLeaper pass per pixel (GLGridLeaper-blend.glsl:65-228 and
// GLGridLeaper-iso.glsl:68-200): along the ray in normalised volume
// coordinates, pick a LOD from the eye-space depth, look the brick up in the
// page table (falling back to coarser LODs and reporting the miss to the hash
// table), leap over EMPTY / CHILD_EMPTY bricks, and march resident bricks in
// steps of 0.5/srm voxel of their LOD.  Positions inside a brick are its local
// texel coordinates (the pool texture coordinates of GLVolumePool.cpp:529-545
// scaled by the pool size and shifted to the slot), so the result does not
// depend on which cache slot holds the brick.

// lighting.glsl:33-43 with a model-space eye (GLGridLeaper-Method-1D-L.glsl)
__device__ __forceinline__ void lighting_eye(const LeaperParams& L, const float pos[3],
                                             const float N[3], const float tfc[3], float out[3]) {
  const RenderParams& P = L.R;
  const float p0 = L.eye_model[0] - pos[0], p1 = L.eye_model[1] - pos[1],
              p2 = L.eye_model[2] - pos[2];
  const float lp = len3(p0, p1, p2);
  const float V0 = p0 / lp, V1 = p1 / lp, V2 = p2 / lp;
  const float d = (N[0] * V0 + N[1] * V1) + N[2] * V2;
  float R0 = V0 - (2.0f * d) * N[0];
  float R1 = V1 - (2.0f * d) * N[1];
  float R2 = V2 - (2.0f * d) * N[2];
  const float lr = len3(R0, R1, R2);
  R0 = R0 / lr; R1 = R1 / lr; R2 = R2 / lr;
  const float* Ld = L.light_dir_model;
  const float diff = fmaxf(fabsf((N[0] * Ld[0] + N[1] * Ld[1]) + N[2] * Ld[2]), 0.0f);
  const float spec = pow_int_or_real(fmaxf((R0 * Ld[0] + R1 * Ld[1]) + R2 * Ld[2], 0.0f), 8.0f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float dcol = P.light_d[i] * tfc[i];
    float c = P.light_a[i] + dcol * diff;
    c = c + P.light_s[i] * spec;
    out[i] = fminf(fmaxf(c, 0.0f), 1.0f);
  }
}

// GLHashTable.cpp:150-185: key = Serialize(brick), linear probing with
// atomicCompSwap from 0, at most `rehash` probes.  An entry only ever goes
// from 0 to a key, so two shortcuts leave the table as the plain probing
// would: one lane reports for all lanes of its warp with the same key, and a
// probe that already reads a non-zero entry needs no atomic.
__device__ __forceinline__ void report_missing(const LeaperParams& L, const uint32_t bc[3],
                                               uint32_t lod) {
  const uint32_t key = 1u + bc[0] + bc[1] * L.ser_x + bc[2] * L.ser_xy + lod * L.ser_xyz;
  const uint32_t peers = __match_any_sync(__activemask(), key);
  if (uint32_t(__ffs(peers) - 1) != (threadIdx.x & 31u)) return;
  for (uint32_t r = 0; r < L.rehash; ++r) {
    uint32_t* slot = &L.hash[(key + r) % L.hash_size];
    uint32_t old = *reinterpret_cast<volatile uint32_t*>(slot);
    if (old == 0u) old = atomicCAS(slot, 0u, key);
    if (old == 0u || old == key) return;
  }
}

// ComputeBrickCoords + GetBrickInfo
// uint(log2(x)) of ComputeLOD as the exact floor of the base-2 logarithm:
// for x >= 2 the binary exponent of x (an approximate log2 could round up to
// the next integer within an ulp of a power of two), 0 below 2 -- [1, 2) has
// level 0 and a negative logarithm is level 0 as well -- and for a NaN; an
// infinity takes the coarsest level.
__device__ __forceinline__ uint32_t lod_level(float x, uint32_t max_lod) {
  if (!(x >= 2.0f)) return 0u;
  const uint32_t e = ((__float_as_uint(x) >> 23) & 0xffu) - 127u;
  return min(max_lod, e);
}

__device__ __forceinline__ uint32_t brick_info(const LeaperParams& L, const float p[3],
                                               uint32_t lod, uint32_t bc[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) bc[a] = uint32_t(p[a] * L.layout[lod][a]);
  return __ldg(&L.page[L.lod_offset[lod] + bc[0] + bc[1] * L.lod_lx[lod] + bc[2] * L.lod_lxy[lod]]);
}

#ifndef TVK_LEAPER_MIN_BLOCKS
#define TVK_LEAPER_MIN_BLOCKS 4
#endif

// samplePool of a pool texel (raw units): the scalar, or a colour pool's red
// channel (GLVolumePool.cpp:637-639 texture(volumePool, coords).r)
template <class V>
__device__ __forceinline__ float pool_scalar(const V& v, float u0, float u1, float u2) {
  return v.sample_u(u0, u1, u2);
}
template <>
__device__ __forceinline__ float pool_scalar<ColorView>(const ColorView& v, float u0, float u1,
                                                        float u2) {
  return v.sample_u<1>(u0, u1, u2).x;
}

// One step of a colour pool at local texel position pc (raw channels * 1/255).
// Blend modes (GLGridLeaper-Method-1D-color / -1D-L-color / -2D-color /
// -2D-L-color.glsl): the filtered RGBA keeps its colour, its alpha becomes
// the TF's alpha at data.a * fTransScale (2D: at the alpha gradient's
// magnitude), opacity-corrected by the host table; lighting takes the data's
// colour as the diffuse colour, the normal from the red channel's gradient
// (1D, ComputeNormal) or domain scale * the alpha gradient / |gradient| (2D).
// Under compositing into acc; returns true when the ray is saturated.
// Iso (GLGridLeaper-Method-iso-color.glsl, GLGridLeaper-iso.glsl:160-172):
// hit at data.a >= fIsoval, 5 bisections on alpha, the normal from the red
// channel (ComputeAlphaNormal calls ComputeGradient), the colour of the
// unrefined sample packed as red + 1 and floor(green * 512) + blue, composed
// by Compose-Color-FS into hit_col; returns true on a hit.
template <bool kIso>
__device__ __forceinline__ bool leaper_color_step(const LeaperParams& L, const ColorView& vol,
                                                  const float pc[3], const float sv[3],
                                                  const float tr[3], const float sc[3], bool lit,
                                                  bool two_d, float W, float H, float4& acc,
                                                  float4& hit_col) {
  const RenderParams& P = L.R;
  const float im = P.inv_max_raw;
  auto at = [&](float l0, float l1, float l2, float& u0, float& u1, float& u2) {
    u0 = fminf(fmaxf(l0 - 0.5f, 0.0f), vol.fn0 - 1.0f);
    u1 = fminf(fmaxf(l1 - 0.5f, 0.0f), vol.fn1 - 1.0f);
    u2 = fminf(fmaxf(l2 - 0.5f, 0.0f), vol.fn2 - 1.0f);
  };
  auto red = [&](float l0, float l1, float l2) -> float {
    float u0, u1, u2;
    at(l0, l1, l2, u0, u1, u2);
    return vol.sample_u<1>(u0, u1, u2).x * im;
  };
  auto alpha = [&](float l0, float l1, float l2) -> float {
    float u0, u1, u2;
    at(l0, l1, l2, u0, u1, u2);
    return vol.sample_u<8>(u0, u1, u2).w * im;
  };
  float u0, u1, u2;
  at(pc[0], pc[1], pc[2], u0, u1, u2);
  const float4 raw = vol.sample_u<15>(u0, u1, u2);
  const float4 c = make_float4(raw.x * im, raw.y * im, raw.z * im, raw.w * im);
  if (kIso) {
    if (!(c.w >= P.iso_norm)) return false;
    float r[3] = {sv[0] / 2.0f, sv[1] / 2.0f, sv[2] / 2.0f};
    float q[3] = {pc[0] - r[0], pc[1] - r[1], pc[2] - r[2]};
    for (int k = 0; k < 5; ++k) {
#pragma unroll
      for (int a = 0; a < 3; ++a) r[a] = r[a] / 2.0f;
      const float vv = alpha(q[0], q[1], q[2]);
#pragma unroll
      for (int a = 0; a < 3; ++a) q[a] = vv >= P.iso_norm ? q[a] - r[a] : q[a] + r[a];
    }
    float g[3], hp[3];
    g[0] = ((red(q[0] - 1.0f, q[1], q[2]) - red(q[0] + 1.0f, q[1], q[2])) / 2.0f) * P.domain_scale[0];
    g[1] = ((red(q[0], q[1] - 1.0f, q[2]) - red(q[0], q[1] + 1.0f, q[2])) / 2.0f) * P.domain_scale[1];
    g[2] = ((red(q[0], q[1], q[2] - 1.0f) - red(q[0], q[1], q[2] + 1.0f)) / 2.0f) * P.domain_scale[2];
    const float gl = len3(g[0], g[1], g[2]);
    if (gl > 0.0f) { g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl; }
#pragma unroll
    for (int a = 0; a < 3; ++a) hp[a] = (q[a] - tr[a]) / sc[a];
    IsoHit h;
#pragma unroll
    for (int r2 = 0; r2 < 3; ++r2) {
      h.pos[r2] = affine_row(L.norm2eye[r2], hp[0], hp[1], hp[2]);
      h.n[r2] = fmaf(L.norm_to_eye_n[r2][2], g[2],
                     fmaf(L.norm_to_eye_n[r2][1], g[1], L.norm_to_eye_n[r2][0] * g[0]));
    }
    h.f = 1.0f;
    h.depth = 0.0f;
    h.enc_r = c.x + 1.0f;
    h.enc_gb = floorf(c.y * 512.0f) + c.z;
    hit_col = iso_compose_color(P, h);
    return true;
  } else {
    const float u = c.w * P.trans_scale;
    float fx = floorf(u * W);
    fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
    float a = 0.0f, g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, mag = 0.0f;
    if (two_d) {
      if (P.tf_col_nonzero[int(fx)] != 0) {
        // GLGridLeaper-GradientTools.glsl ComputeGradientAlpha (Yp at -delta.y)
        g0 = (alpha(pc[0] - 1.0f, pc[1], pc[2]) - alpha(pc[0] + 1.0f, pc[1], pc[2])) / 2.0f;
        g1 = (alpha(pc[0], pc[1] - 1.0f, pc[2]) - alpha(pc[0], pc[1] + 1.0f, pc[2])) / 2.0f;
        g2 = (alpha(pc[0], pc[1], pc[2] - 1.0f) - alpha(pc[0], pc[1], pc[2] + 1.0f)) / 2.0f;
        mag = len3(g0, g1, g2);
        const float w = 1.0f - mag * P.grad_scale;
        float fy = floorf(w * H);
        fy = fminf(fmaxf(fy, 0.0f), H - 1.0f);
        a = __ldg(&P.tf[int(fy) * P.tf_w + int(fx)].w);
      }
    } else {
      a = __ldg(&P.tf[int(fx)].w);
    }
    float4 src = make_float4(c.x, c.y, c.z, a);
    if (lit && a != 0.0f) {
      float N[3];
      if (two_d) {
        const float q0 = mag > 0.0f ? g0 / mag : g0, q1 = mag > 0.0f ? g1 / mag : g1,
                    q2 = mag > 0.0f ? g2 / mag : g2;
        N[0] = P.domain_scale[0] * q0; N[1] = P.domain_scale[1] * q1;
        N[2] = P.domain_scale[2] * q2;
      } else {
        N[0] = ((red(pc[0] - 1.0f, pc[1], pc[2]) - red(pc[0] + 1.0f, pc[1], pc[2])) / 2.0f) *
               P.domain_scale[0];
        N[1] = ((red(pc[0], pc[1] - 1.0f, pc[2]) - red(pc[0], pc[1] + 1.0f, pc[2])) / 2.0f) *
               P.domain_scale[1];
        N[2] = ((red(pc[0], pc[1], pc[2] - 1.0f) - red(pc[0], pc[1], pc[2] + 1.0f)) / 2.0f) *
               P.domain_scale[2];
        const float l = len3(N[0], N[1], N[2]);
        if (l > 0.0f) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
      }
      float mp[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) mp[k] = (pc[k] - tr[k]) / sc[k];
      const float tfc[3] = {c.x, c.y, c.z};
      float lc[3];
      lighting_eye(L, mp, N, tfc, lc);
      src.x = lc[0]; src.y = lc[1]; src.z = lc[2];
    }
    const float w = 1.0f - acc.w;
    acc.x = fmaf(src.x * w, src.w, acc.x);
    acc.y = fmaf(src.y * w, src.w, acc.y);
    acc.z = fmaf(src.z * w, src.w, acc.z);
    acc.w = fmaf(src.w, w, acc.w);
    return acc.w > 0.99f;
  }
}

template <class T, bool kIso>
__global__ void __launch_bounds__(128, TVK_LEAPER_MIN_BLOCKS) leaper_kernel(const LeaperParams L) {
  // RGBA8 colour pool (GLGridLeaper-Method-*-color.glsl); no macro cells
  constexpr bool kColor = std::is_same<T, uchar4>::value;
  using View = typename std::conditional<kColor, ColorView, BrickView<T>>::type;
  const RenderParams& P = L.R;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const uint32_t py = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  if (px >= P.width || py >= P.height) return;
  const size_t pix = size_t(py) * P.width + px;

  // eye-space ray through the pixel centre (z = -1) and its normalised-volume
  // counterpart; the eye point at parameter s has depth (eye z) -s
  const float nx = (float(px) + 0.5f) * P.inv_w2 - 1.0f;
  const float ny = (float(py) + 0.5f) * P.inv_h2 - 1.0f;
  const float de[3] = {nx * P.kx, ny * P.ky, -1.0f};
  float o[3], d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = L.eye2norm[a][3];
    d[a] = fmaf(L.eye2norm[a][2], de[2], fmaf(L.eye2norm[a][1], de[1], L.eye2norm[a][0] * de[0]));
  }
  // the volume box [0,1]^3: entry (front faces or the near plane), exit (back faces)
  float s0 = -INFINITY, s1 = INFINITY;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float inv = 1.0f / d[a];
    const float ta = (0.0f - o[a]) * inv, tb = (1.0f - o[a]) * inv;
    s0 = fmaxf(s0, fminf(ta, tb));
    s1 = fminf(s1, fmaxf(ta, tb));
  }
  const float s_in = fmaxf(s0, P.znear);
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(s1 > s_in) || s1 > P.zfar) {
    P.out[pix] = acc;
    L.resume_pos[pix] = make_float4(0.f, 0.f, 0.f, 1000.f);
    L.resume_col[pix] = acc;
    if (P.spp) P.spp[pix] = 0;
    return;
  }
  float ent[3], ext[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ext[a] = fmaf(s1, d[a], o[a]);
  const float exit_depth = -s1;
  float entry_depth;
  if (L.first_pass) {
#pragma unroll
    for (int a = 0; a < 3; ++a) ent[a] = fmaf(s_in, d[a], o[a]);
    entry_depth = -s_in;
  } else {
    const float4 rp = L.resume_pos[pix];
    if (rp.w == 1000.0f) {  // finished in an earlier pass
      P.out[pix] = L.resume_col[pix];
      if (P.spp) P.spp[pix] = 0;
      return;
    }
    ent[0] = rp.x; ent[1] = rp.y; ent[2] = rp.z;
    entry_depth = rp.w;
    acc = L.resume_col[pix];
  }
  float4 res_pos = make_float4(ent[0], ent[1], ent[2], entry_depth);
  float4 res_col = acc;
  const float dir[3] = {ext[0] - ent[0], ext[1] - ent[1], ext[2] - ent[2]};
  const float ray_len = len3(dir[0], dir[1], dir[2]);
  // TransformToPoolSpace: 0.5 / srm texel of the brick's LOD per step
  float sv[3] = {dir[0] * L.vol_size[0], dir[1] * L.vol_size[1], dir[2] * L.vol_size[2]};
  {
    const float l = len3(sv[0], sv[1], sv[2]);
#pragma unroll
    for (int a = 0; a < 3; ++a) sv[a] = (sv[a] / l) / (2.0f * L.srm);
  }
  const float step_len = len3(sv[0], sv[1], sv[2]);
  const float voxel_eps = 0.125f / 2000.0f;
  const float im = P.inv_max_raw;
  const float W = float(P.tf_w), H = float(P.tf_h);
  const bool lit = P.lighting != 0;
  const bool two_d = P.mode == TVK_RM_2DTRANS;
  float cur[3] = {ent[0], ent[1], ent[2]};
  float t = 0.0f;
  bool optimal = true;
  uint32_t last[4] = {0u, 0u, 0u, 9999u};
  uint32_t samples = 0;
  bool hit = false;
  float4 hit_col = make_float4(0.f, 0.f, 0.f, 0.f);

  if (ray_len > voxel_eps) {
    for (uint32_t j = 0; j < 100; ++j) {
      const float depth = entry_depth * (1.0f - t) + exit_depth * t;
      // ComputeLOD (GLVolumePool.cpp:650-656): uint(log2(x)), a negative
      // level is level 0
      uint32_t lod = lod_level(L.lod_factor * (-depth) / L.lod0_err, L.max_lod);
      // GetBrick (GLVolumePool.cpp:553-612)
      float p[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) p[a] = fminf(fmaxf(cur[a], 0.0f), 1.0f);
      bool found = true;
      uint32_t bc[3];
      uint32_t info = brick_info(L, p, lod, bc);
      if (info == kBiMissing) {
        report_missing(L, bc, lod);
        found = false;
        while (info == kBiMissing && lod < L.max_lod) {
          ++lod;
          info = brick_info(L, p, lod, bc);
        }
        if (info == kBiMissing) info = kBiEmpty;  // the coarsest brick is always resident
      }
      const bool empty = info <= kBiEmpty;
      if (empty) {
        for (uint32_t l = lod + 1; l < L.max_lod; ++l) {
          uint32_t lbc[3];
          const uint32_t linfo = brick_info(L, p, l, lbc);
          if (linfo != kBiChildEmpty) break;
          bc[0] = lbc[0]; bc[1] = lbc[1]; bc[2] = lbc[2];
          info = linfo;
          lod = l;
        }
      }
      float c0[3], c1[3], bexit[3];
      float tmin = INFINITY;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        c0[a] = float(bc[a]) / L.layout[lod][a];
        c1[a] = float(bc[a] + 1u) / L.layout[lod][a];
        const float div = 1.0f / dir[a];
        const float corner = div >= 0.0f ? c1[a] : c0[a];
        tmin = fminf(tmin, (corner - p[a]) * div);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) bexit[a] = fmaf(tmin, dir[a], p[a]);
      if (!found && optimal) {
        optimal = false;
        res_pos = make_float4(cur[0], cur[1], cur[2], depth);
        res_col = acc;
      }
      const bool same = last[0] == bc[0] && last[1] == bc[1] && last[2] == bc[2] && last[3] == lod;
      if (!empty && !same) {
        const uint32_t gid = L.lod_offset[lod] + bc[0] + bc[1] * L.lod_lx[lod] +
                             bc[2] * L.lod_lxy[lod];
        const uint32_t dims = __ldg(&L.brick_dims[gid]);
        View vol;
        vol.p = static_cast<const T*>(L.slots) + size_t(info - kBiFlagCount) * L.slot_voxels;
        vol.n0 = int(dims & 1023u); vol.n1 = int((dims >> 10) & 1023u); vol.n2 = int(dims >> 20);
        vol.fn0 = float(vol.n0); vol.fn1 = float(vol.n1); vol.fn2 = float(vol.n2);
        vol.sx = uint32_t(vol.n0); vol.sxy = uint32_t(vol.n0 * vol.n1);
        float sc[3], tr[3], pc[3], pe[3], pxx[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          sc[a] = L.max_inner[a] * L.layout[lod][a];
          tr[a] = L.ghost - c0[a] * sc[a];
          pe[a] = fmaf(p[a], sc[a], tr[a]);
          pxx[a] = fmaf(bexit[a], sc[a], tr[a]);
          pc[a] = pe[a];
        }
        int steps = int(ceilf(len3(pxx[0] - pe[0], pxx[1] - pe[1], pxx[2] - pe[2]) / step_len));
        steps = min(steps, int(ceilf(len3((ext[0] - cur[0]) * sc[0], (ext[1] - cur[1]) * sc[1],
                                          (ext[2] - cur[2]) * sc[2]) / step_len)));
        auto sample = [&](float l0, float l1, float l2) -> float {
          const float u0 = fminf(fmaxf(l0 - 0.5f, 0.0f), vol.fn0 - 1.0f);
          const float u1 = fminf(fmaxf(l1 - 0.5f, 0.0f), vol.fn1 - 1.0f);
          const float u2 = fminf(fmaxf(l2 - 0.5f, 0.0f), vol.fn2 - 1.0f);
          return pool_scalar(vol, u0, u1, u2) * im;
        };
        // macro cells of the brick (as in the brick-by-brick march): steps in
        // an empty cube add nothing and cannot hit, so they are leapt over,
        // the position keeping the chain of additions
        const uint8_t* __restrict__ dist =
            (!kColor && L.cell_dist) ? L.cell_dist + L.cell_off[gid] : nullptr;
        const int ncx = int(cells_per_axis(uint32_t(vol.n0))),
                  ncy = int(cells_per_axis(uint32_t(vol.n1))),
                  ncz = int(cells_per_axis(uint32_t(vol.n2)));
        const float idu0 = 1.0f / fabsf(sv[0]), idu1 = 1.0f / fabsf(sv[1]),
                    idu2 = 1.0f / fabsf(sv[2]);
        bool done = false;
        for (int i = 0; i < steps; ++i) {
          if (dist) {
            const float uu0 = pc[0] - 0.5f, uu1 = pc[1] - 0.5f, uu2 = pc[2] - 0.5f;
            const float u0 = fminf(fmaxf(uu0, 0.0f), vol.fn0 - 1.0f);
            const float u1 = fminf(fmaxf(uu1, 0.0f), vol.fn1 - 1.0f);
            const float u2 = fminf(fmaxf(uu2, 0.0f), vol.fn2 - 1.0f);
            const int cx = int(u0) >> kCellShift, cy = int(u1) >> kCellShift,
                      cz = int(u2) >> kCellShift;
            const int dd = __ldg(&dist[(cz * ncy + cy) * ncx + cx]);
            if (dd != 0) {
              int k = 0;
              if (uu0 == u0 && uu1 == u1 && uu2 == u2) {
                const int r = dd - 1;
                const float lo0 = float(max(cx - r, 0) << kCellShift),
                            lo1 = float(max(cy - r, 0) << kCellShift),
                            lo2 = float(max(cz - r, 0) << kCellShift);
                const float hi0 = float(min(cx + r + 1, ncx) << kCellShift),
                            hi1 = float(min(cy + r + 1, ncy) << kCellShift),
                            hi2 = float(min(cz + r + 1, ncz) << kCellShift);
                const float d0 = sv[0] > 0.0f ? hi0 - uu0 : uu0 - lo0;
                const float d1 = sv[1] > 0.0f ? hi1 - uu1 : uu1 - lo1;
                const float d2 = sv[2] > 0.0f ? hi2 - uu2 : uu2 - lo2;
                const float m = fminf(fminf((d0 - 0.015625f) * idu0, (d1 - 0.015625f) * idu1),
                                      (d2 - 0.015625f) * idu2);
                k = m > 0.0f ? int(fminf(m, float(steps - 1 - i))) : 0;
              }
              samples += uint32_t(k + 1);
#pragma unroll 4
              for (int j = 0; j <= k; ++j) {
#pragma unroll
                for (int a = 0; a < 3; ++a) pc[a] = pc[a] + sv[a];
              }
              i += k;
              continue;
            }
          }
          ++samples;
          if constexpr (kColor) {
            if (leaper_color_step<kIso>(L, vol, pc, sv, tr, sc, lit, two_d, W, H, acc, hit_col)) {
              hit = kIso;
              done = true;
              break;
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) pc[a] = pc[a] + sv[a];
            continue;
          }
          const float v = sample(pc[0], pc[1], pc[2]);
          if (kIso) {
            // GLGridLeaper-Method-iso.glsl: first sample >= fIsoval, 5 bisections
            if (v >= P.iso_norm) {
              float r[3] = {sv[0] / 2.0f, sv[1] / 2.0f, sv[2] / 2.0f};
              float q[3] = {pc[0] - r[0], pc[1] - r[1], pc[2] - r[2]};
              for (int k = 0; k < 5; ++k) {
#pragma unroll
                for (int a = 0; a < 3; ++a) r[a] = r[a] / 2.0f;
                const float vv = sample(q[0], q[1], q[2]);
#pragma unroll
                for (int a = 0; a < 3; ++a) q[a] = vv >= P.iso_norm ? q[a] - r[a] : q[a] + r[a];
              }
              // hit position (eye space) and normal (ComputeNormal, to eye space)
              float hn[3], he[3], g[3];
              const float xp = sample(q[0] + 1.0f, q[1], q[2]), xm = sample(q[0] - 1.0f, q[1], q[2]);
              const float yp = sample(q[0], q[1] - 1.0f, q[2]), ym = sample(q[0], q[1] + 1.0f, q[2]);
              const float zp = sample(q[0], q[1], q[2] + 1.0f), zm = sample(q[0], q[1], q[2] - 1.0f);
              g[0] = ((xm - xp) / 2.0f) * P.domain_scale[0];
              g[1] = ((yp - ym) / 2.0f) * P.domain_scale[1];
              g[2] = ((zm - zp) / 2.0f) * P.domain_scale[2];
              const float gl = len3(g[0], g[1], g[2]);
              if (gl > 0.0f) { g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl; }
              float hp[3];
#pragma unroll
              for (int a = 0; a < 3; ++a) hp[a] = (q[a] - tr[a]) / sc[a];
#pragma unroll
              for (int r2 = 0; r2 < 3; ++r2) {
                he[r2] = affine_row(L.norm2eye[r2], hp[0], hp[1], hp[2]);
                hn[r2] = fmaf(L.norm_to_eye_n[r2][2], g[2],
                              fmaf(L.norm_to_eye_n[r2][1], g[1], L.norm_to_eye_n[r2][0] * g[0]));
              }
              IsoHit h;
              h.pos[0] = he[0]; h.pos[1] = he[1]; h.pos[2] = he[2];
              h.n[0] = hn[0]; h.n[1] = hn[1]; h.n[2] = hn[2];
              h.f = 1.0f;
              h.depth = 0.0f;
              hit_col = iso_compose(P, h);
              hit = true;
              done = true;
              break;
            }
          } else {
            float4 src;
            const float u = v * P.trans_scale;
            float fx = floorf(u * W);
            fx = fminf(fmaxf(fx, 0.0f), W - 1.0f);
            float g0 = 0.f, g1 = 0.f, g2 = 0.f;
            bool need_grad = lit;
            if (two_d) need_grad = P.tf_col_nonzero[int(fx)] != 0;
            if (!two_d) {
              src = __ldg(&P.tf[int(fx)]);
              need_grad = lit && src.w != 0.0f;
            }
            if (need_grad) {
              // GLGridLeaper-GradientTools.glsl:6-19 (Yp sampled at -delta.y)
              const float xp = sample(pc[0] + 1.0f, pc[1], pc[2]), xm = sample(pc[0] - 1.0f, pc[1], pc[2]);
              const float yp = sample(pc[0], pc[1] - 1.0f, pc[2]), ym = sample(pc[0], pc[1] + 1.0f, pc[2]);
              const float zp = sample(pc[0], pc[1], pc[2] + 1.0f), zm = sample(pc[0], pc[1], pc[2] - 1.0f);
              g0 = (xm - xp) / 2.0f;
              g1 = (yp - ym) / 2.0f;
              g2 = (zm - zp) / 2.0f;
            }
            float mag = 0.0f;
            if (two_d) {
              if (need_grad) {
                mag = len3(g0, g1, g2);
                const float w = 1.0f - mag * P.grad_scale;
                float fy = floorf(w * H);
                fy = fminf(fmaxf(fy, 0.0f), H - 1.0f);
                src = __ldg(&P.tf[int(fy) * P.tf_w + int(fx)]);
              } else {
                src = make_float4(0.f, 0.f, 0.f, 0.f);
              }
              need_grad = need_grad && lit && src.w != 0.0f;
            }
            if (lit && need_grad) {
              float N[3];
              if (two_d) {  // GLGridLeaper-Method-2D-L.glsl: domain scale * g / |g|
                const float q0 = mag > 0.0f ? g0 / mag : g0, q1 = mag > 0.0f ? g1 / mag : g1,
                            q2 = mag > 0.0f ? g2 / mag : g2;
                N[0] = P.domain_scale[0] * q0; N[1] = P.domain_scale[1] * q1;
                N[2] = P.domain_scale[2] * q2;
              } else {      // ComputeNormal: g * domain scale, safely normalised
                N[0] = g0 * P.domain_scale[0]; N[1] = g1 * P.domain_scale[1];
                N[2] = g2 * P.domain_scale[2];
                const float l = len3(N[0], N[1], N[2]);
                if (l > 0.0f) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
              }
              float mp[3];
#pragma unroll
              for (int a = 0; a < 3; ++a) mp[a] = (pc[a] - tr[a]) / sc[a];
              const float tfc[3] = {src.x, src.y, src.z};
              float lc[3];
              lighting_eye(L, mp, N, tfc, lc);
              src.x = lc[0]; src.y = lc[1]; src.z = lc[2];
            }
            // Compositing.glsl UnderCompositing
            const float w = 1.0f - acc.w;
            acc.x = fmaf(src.x * w, src.w, acc.x);
            acc.y = fmaf(src.y * w, src.w, acc.y);
            acc.z = fmaf(src.z * w, src.w, acc.z);
            acc.w = fmaf(src.w, w, acc.w);
            if (acc.w > 0.99f) { done = true; break; }
          }
#pragma unroll
          for (int a = 0; a < 3; ++a) pc[a] = pc[a] + sv[a];
        }
        if (done) break;
#pragma unroll
        for (int a = 0; a < 3; ++a) cur[a] = (pc[a] - tr[a]) / sc[a];
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) cur[a] = fmaf(voxel_eps, dir[a] / ray_len, bexit[a]);
      }
      last[0] = bc[0]; last[1] = bc[1]; last[2] = bc[2]; last[3] = lod;
      t = len3(ent[0] - bexit[0], ent[1] - bexit[1], ent[2] - bexit[2]) / ray_len;
      if (t > 0.9999f) break;
    }
  }
  // TerminateRay: a ray that met only bricks of the wanted resolution is done
  const float4 out = kIso ? hit_col : acc;
  if (optimal) {
    res_pos.w = 1000.0f;
    res_col = out;
  }
  P.out[pix] = out;
  L.resume_pos[pix] = res_pos;
  L.resume_col[pix] = res_col;
  if (P.spp) P.spp[pix] = samples;
  const uint32_t wsum = __reduce_add_sync(__activemask(), samples);
  if ((lane == __ffs(__activemask()) - 1)) atomicAdd(&P.counters[0], (unsigned long long)wsum);
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float w) {
  return make_float4(fmaf(w, b.x - a.x, a.x), fmaf(w, b.y - a.y, a.y), fmaf(w, b.z - a.z, a.z),
                     fmaf(w, b.w - a.w, a.w));
}

__global__ void __launch_bounds__(256)
upscale_kernel(const float4* __restrict__ low, uint32_t lw, uint32_t lh, float4* __restrict__ out,
               uint32_t w, uint32_t h, float rescale) {
  // GLRenderer::FullscreenQuadRegion (GLRenderer.cpp:688-713): pixel x of the
  // viewport reads texture coordinate (x + 0.5) / w * rescale of the w-wide
  // target, i.e. texel position (x + 0.5) * rescale - 0.5, filtered with
  // GL_LINEAR and clamped to the reduced image's edge.
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y;
  if (x >= w) return;
  const float u = (float(x) + 0.5f) * rescale - 0.5f;
  const float v = (float(y) + 0.5f) * rescale - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float wx = u - fu, wy = v - fv;
  const int x0 = min(max(int(fu), 0), int(lw) - 1), x1 = min(max(int(fu) + 1, 0), int(lw) - 1);
  const int y0 = min(max(int(fv), 0), int(lh) - 1), y1 = min(max(int(fv) + 1, 0), int(lh) - 1);
  const float4 c0 = lerp4(low[size_t(y0) * lw + x0], low[size_t(y0) * lw + x1], wx);
  const float4 c1 = lerp4(low[size_t(y1) * lw + x0], low[size_t(y1) * lw + x1], wx);
  out[size_t(y) * w + x] = lerp4(c0, c1, wy);
}

}  // namespace

void launch_upscale(const float4* low, uint32_t lw, uint32_t lh, float4* out, uint32_t w,
                    uint32_t h, float rescale, cudaStream_t s, uint64_t* launches) {
  const dim3 grid((w + 255) / 256, h);
  upscale_kernel<<<grid, 256, 0, s>>>(low, lw, lh, out, w, h, rescale);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

const void* batch_kernel_function(int variant) {
  switch (variant) {
    case 0: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint8_t, false, 1>);
    case 1: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint8_t, true, 1>);
    case 2: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint16_t, false, 1>);
    case 3: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint16_t, true, 1>);
    case 4: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint8_t, false, 2>);
    case 5: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint8_t, true, 2>);
    case 6: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint16_t, false, 2>);
    default: return reinterpret_cast<const void*>(&raycast_batch_kernel<uint16_t, true, 2>);
  }
}

int batch_ctas_per_sm_max(int variant) {
  int n = 0;
  TVK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel_function(variant), 128,
                                                         0));
  return n;
}

void launch_raycast_batch(const BatchLaunch& L, int variant, uint32_t* d_next_item,
                          uint32_t ctas, cudaStream_t s, uint64_t* launches) {
  switch (variant) {
    case 0: raycast_batch_kernel<uint8_t, false, 1><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 1: raycast_batch_kernel<uint8_t, true, 1><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 2: raycast_batch_kernel<uint16_t, false, 1><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 3: raycast_batch_kernel<uint16_t, true, 1><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 4: raycast_batch_kernel<uint8_t, false, 2><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 5: raycast_batch_kernel<uint8_t, true, 2><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    case 6: raycast_batch_kernel<uint16_t, false, 2><<<ctas, 128, 0, s>>>(L, d_next_item); break;
    default: raycast_batch_kernel<uint16_t, true, 2><<<ctas, 128, 0, s>>>(L, d_next_item); break;
  }
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_leaper(const LeaperParams& p, cudaStream_t s, uint64_t* launches) {
  const dim3 grid((p.R.width + 15) / 16, (p.R.height + 7) / 8);
  const bool iso = p.R.mode == TVK_RM_ISOSURFACE;
  if (p.R.bytes == 4) {
    if (iso) leaper_kernel<uchar4, true><<<grid, 128, 0, s>>>(p);
    else leaper_kernel<uchar4, false><<<grid, 128, 0, s>>>(p);
  } else if (p.R.bytes == 1) {
    if (iso) leaper_kernel<uint8_t, true><<<grid, 128, 0, s>>>(p);
    else leaper_kernel<uint8_t, false><<<grid, 128, 0, s>>>(p);
  } else {
    if (iso) leaper_kernel<uint16_t, true><<<grid, 128, 0, s>>>(p);
    else leaper_kernel<uint16_t, false><<<grid, 128, 0, s>>>(p);
  }
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_raycast(const RenderParams& p, cudaStream_t s, uint64_t* launches) {
  const dim3 block(128);
  const uint32_t tw = 16 * TVK_RAYCAST_RPT;
  const dim3 grid((p.out_w + tw - 1) / tw, (p.out_h + 7) / 8);
  const bool iso = p.mode == TVK_RM_ISOSURFACE;
  const bool cv = iso && p.cv_on;
  if (p.bytes == 4) {
    if (iso) raycast_kernel<uchar4, true><<<grid, block, 0, s>>>(p);
    else raycast_kernel<uchar4, false><<<grid, block, 0, s>>>(p);
  } else if (p.tex) {  // hardware-filtered lookups (scalar, no ClearView)
    if (p.bytes == 1) {
      if (iso) raycast_kernel<uint8_t, true, false, true><<<grid, block, 0, s>>>(p);
      else raycast_kernel<uint8_t, false, false, true><<<grid, block, 0, s>>>(p);
    } else {
      if (iso) raycast_kernel<uint16_t, true, false, true><<<grid, block, 0, s>>>(p);
      else raycast_kernel<uint16_t, false, false, true><<<grid, block, 0, s>>>(p);
    }
  } else if (p.bytes == 1) {
    if (cv) raycast_kernel<uint8_t, true, true><<<grid, block, 0, s>>>(p);
    else if (iso) raycast_kernel<uint8_t, true><<<grid, block, 0, s>>>(p);
    else raycast_kernel<uint8_t, false><<<grid, block, 0, s>>>(p);
  } else {
    if (cv) raycast_kernel<uint16_t, true, true><<<grid, block, 0, s>>>(p);
    else if (iso) raycast_kernel<uint16_t, true><<<grid, block, 0, s>>>(p);
    else raycast_kernel<uint16_t, false><<<grid, block, 0, s>>>(p);
  }
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

void launch_cv_compose(const CvComposeParams& p, cudaStream_t s, uint64_t* launches) {
  const dim3 block(32, 4);
  const dim3 grid((p.w + 31) / 32, (p.h + 3) / 4);
  cv_compose_kernel<<<grid, block, 0, s>>>(p);
  TVK_CUDA(cudaGetLastError());
  ++*launches;
}

}  // namespace tvk
