// raycast.cpp -- scalar CPU restatement of Tuvok's brick-by-brick GLSL ray
// caster (GLRaycaster) including the OpenGL fixed-function behaviour it relies on.
//
// TEST INFRASTRUCTURE ONLY (the checker for tuvok_gb300's CUDA ray march).
// Sources restated (paths relative to the Tuvok tree):
//   Shaders/GLRaycaster-1D-FS.glsl:51-82, GLRaycaster-1D-light-FS.glsl:84-134,
//   GLRaycaster-2D-FS.glsl:53-94, GLRaycaster-2D-light-FS.glsl:61-117,
//   Volume3D.glsl:39-60, VRender1D.glsl:39-57, VRender1DLit.glsl:49-72,
//   lighting.glsl:33-50, Compositing.glsl:33-38;
//   Renderer/GL/GLRaycaster.cpp:93-99 (RGBA16F entry buffer), :239-300
//   (step size / opacity correction), :302-345 + :589-612 (eye->texture matrix),
//   :348-478 (near plane + per-brick passes);
//   Renderer/GL/GLRenderer.cpp:133-155 (blend ONE_MINUS_DST_ALPHA, ONE),
//   :1813-1819 (CalculateScaling), :2890-2913 (light colours);
//   Renderer/AbstrRenderer.cpp:860-866 (MaxValue), :953-997 (ContainsData),
//   :999-1100 (brick list); Basics/Vectors.h:1250-1276 (LookAt, Perspective);
//   IO/uvfDataset.cpp:1747-1774 (texture coordinates of a brick).
//
// Fixed-function semantics pinned here (no source states them):
//   * volume texture: texel-centre trilinear, clamp to edge, texel value =
//     raw / (2^bits - 1); lerp(a,b,f) = fma(f, b - a, a), x then y then z;
//   * transfer function: GL_NEAREST, clamp to edge;
//   * RGBA16F: IEEE binary16 round to nearest even;
//   * framebuffer blend in FP32: dst = fma(src, 1 - dst.a, dst).
// The march itself never fuses a multiply and an add unless written as fma
// (the file is built with -ffp-contract=off), so the FP32 path is an exact
// statement of the arithmetic the CUDA kernel performs.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cfenv>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" float orc_pow01(float x, float y);

extern "C" float orc_round_half(float x) {
  // IEEE 754 binary16, round to nearest, ties to even.
  if (std::isnan(x) || std::isinf(x) || x == 0.0f) return x;
  const double ax = std::fabs(double(x));
  int e = std::ilogb(ax);
  if (e < -14) e = -14;  // subnormal spacing 2^-24
  const double sp = std::ldexp(1.0, e - 10);
  double r = std::nearbyint(ax / sp) * sp;
  if (r >= 65520.0) r = INFINITY;
  return float(std::copysign(r, double(x)));
}

namespace {

struct Mat34d { double m[3][4]; };

struct View {
  double mv[3][4];     // model -> eye
  double inv[3][4];    // eye -> model
  float kx, ky;        // ray direction scale (aspect * tan(fov/2), tan(fov/2))
  float inv_w2, inv_h2;
};

View make_view(const orc_scene& s) {
  // Basics/Vectors.h:1250-1263 BuildLookAt (computed in double here).
  const double eye[3] = {s.eye[0], s.eye[1], s.eye[2]};
  double F[3] = {double(s.at[0]) - eye[0], double(s.at[1]) - eye[1], double(s.at[2]) - eye[2]};
  double U[3] = {s.up[0], s.up[1], s.up[2]};
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
  View v;
  const double* rows[3] = {S, U2, F};
  for (int r = 0; r < 3; ++r) {
    const double sg = (r == 2) ? -1.0 : 1.0;
    double d = 0;
    for (int c = 0; c < 3; ++c) {
      v.mv[r][c] = sg * rows[r][c];
      d += rows[r][c] * eye[c];
    }
    v.mv[r][3] = -sg * d;
  }
  // rigid inverse: R^T, -R^T t
  for (int r = 0; r < 3; ++r) {
    double t = 0;
    for (int c = 0; c < 3; ++c) {
      v.inv[r][c] = v.mv[c][r];
      t += v.mv[c][r] * v.mv[c][3];
    }
    v.inv[r][3] = -t;
  }
  // Vectors.h:1265-1276 Perspective; the inverse projection of pixel centres.
  const double th = std::tan(double(s.fovy_deg) * (3.14159265358979323846 / 180.0) / 2.0);
  const double aspect = double(s.width) / double(s.height);
  v.kx = float(aspect * th);
  v.ky = float(th);
  v.inv_w2 = float(2.0 / double(s.width));
  v.inv_h2 = float(2.0 / double(s.height));
  return v;
}

struct BrickR {
  float pmin[3], pmax[3];
  float tmin[3], tmax[3];  // texture coordinates of the inner region
  float tex[3][4];   // eye -> brick texture coordinates
  float step;        // fRayStepsize
  uint32_t n[3];
  std::vector<uint8_t> data;
};

// Affine map used for every matrix*point product of the march.
template <class T>
inline T affine_row(const float r[4], T x, T y, T z) {
  return std::fma(T(r[0]), x, std::fma(T(r[1]), y, std::fma(T(r[2]), z, T(r[3]))));
}

template <class T>
struct Vol {
  const BrickR* b;
  int dtype;
  T inv_max;
  int ch = 0;  // RGBA8: the channel sampled (0 = red ... 3 = alpha)
  T fetch(int x, int y, int z) const {
    const size_t i = size_t(x) + size_t(y) * b->n[0] + size_t(z) * b->n[0] * b->n[1];
    if (dtype == 2) return T(b->data[4 * i + size_t(ch)]);
    if (dtype == 0) return T(b->data[i]);
    return T(reinterpret_cast<const uint16_t*>(b->data.data())[i]);
  }
  // texel-centre trilinear with clamp-to-edge
  T sample(T tx, T ty, T tz) const {
    const T t[3] = {tx, ty, tz};
    int i0[3], i1[3];
    T f[3];
    for (int a = 0; a < 3; ++a) {
      T u = std::fma(t[a], T(b->n[a]), T(-0.5));
      u = std::fmin(std::fmax(u, T(0)), T(b->n[a] - 1));
      i0[a] = int(u);
      f[a] = u - T(i0[a]);
      i1[a] = std::min(i0[a] + 1, int(b->n[a]) - 1);
    }
    auto lerp = [](T a, T c, T w) { return std::fma(w, c - a, a); };
    const T c00 = lerp(fetch(i0[0], i0[1], i0[2]), fetch(i1[0], i0[1], i0[2]), f[0]);
    const T c10 = lerp(fetch(i0[0], i1[1], i0[2]), fetch(i1[0], i1[1], i0[2]), f[0]);
    const T c01 = lerp(fetch(i0[0], i0[1], i1[2]), fetch(i1[0], i0[1], i1[2]), f[0]);
    const T c11 = lerp(fetch(i0[0], i1[1], i1[2]), fetch(i1[0], i1[1], i1[2]), f[0]);
    const T c0 = lerp(c00, c10, f[1]);
    const T c1 = lerp(c01, c11, f[1]);
    return lerp(c0, c1, f[2]) * inv_max;
  }
};

template <class T>
inline T len3(T x, T y, T z) { return std::sqrt((x * x + y * y) + z * z); }

template <class T>
inline T dot3(const T a[3], const T b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

// GLSL pow(x, y) for x in [0, 1] (opacity correction, specular terms),
// defined by the shading language as exp2(y * log2(x)) with an
// implementation-chosen precision.  The FP32 oracle fixes one such
// implementation in double operations that round the same on every IEEE
// machine, rounded to float at the end:
//  * log2(x) = e + (2 / ln 2) * atanh(s) with x = m * 2^e, m in
//    [sqrt(1/2), sqrt(2)), s = (m - 1) / (m + 1), and the atanh series
//    s + s^3/3 + ... + s^13/13 (|s| <= 0.172: truncation below 1e-12);
//  * exp2(t) = 2^k * e^(f ln 2), k = floor(t + 1/2), |f| <= 1/2, and the
//    Taylor series of e^z to z^9 (truncation below 1e-10).
// Results below 2^-125 are 0 (callers take 1 - x^y, which that leaves
// unchanged).  The FP64 oracle keeps libm's pow.
inline float pow01f(float xf, float yf) {
  if (yf == 0.0f || xf == 1.0f) return 1.0f;
  if (!(xf > 0.0f)) return 0.0f;
  if (xf > 1.0f) return 1.0f;
  const double x = double(xf);
  uint64_t bits;
  std::memcpy(&bits, &x, sizeof bits);
  double e = double(int((bits >> 52) & 0x7ffu) - 1022);
  const uint64_t mb = (bits & 0x000fffffffffffffull) | 0x3fe0000000000000ull;
  double m;
  std::memcpy(&m, &mb, sizeof m);
  if (m < 0.70710678118654752) {
    m = m * 2.0;
    e = e - 1.0;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  const double inv_odd[7] = {1.0 / 13.0, 1.0 / 11.0, 1.0 / 9.0, 1.0 / 7.0,
                             1.0 / 5.0,  1.0 / 3.0,  1.0};
  double p = inv_odd[0];
  for (int i = 1; i < 7; ++i) p = std::fma(p, s2, inv_odd[i]);
  const double lg = std::fma(2.8853900817779268 * s, p, e);
  const double t = double(yf) * lg;
  if (!(t > -125.0)) return 0.0f;
  if (t >= 128.0) return INFINITY;
  const double k = std::floor(t + 0.5);
  const double z = (t - k) * 0.69314718055994531;
  const double inv_fact[10] = {1.0 / 362880.0, 1.0 / 40320.0, 1.0 / 5040.0, 1.0 / 720.0,
                               1.0 / 120.0,    1.0 / 24.0,    1.0 / 6.0,    0.5,
                               1.0,            1.0};
  double q = inv_fact[0];
  for (int i = 1; i < 10; ++i) q = std::fma(q, z, inv_fact[i]);
  const uint64_t kb = uint64_t(int(k) + 1023) << 52;
  double two_k;
  std::memcpy(&two_k, &kb, sizeof two_k);
  return float(q * two_k);
}

inline float glsl_pow(float x, float y) { return pow01f(x, y); }

}  // namespace

extern "C" float orc_pow01(float x, float y) { return pow01f(x, y); }

namespace {
inline double glsl_pow(double x, double y) { return std::pow(x, y); }

template <class T>
inline T pow_int_or_real(T x, float e) {
  // exponents 8 (reference) and 32 (Blinn-Phong) by repeated squaring
  if (e == 8.0f) { T a = x * x; a = a * a; return a * a; }
  if (e == 32.0f) { T a = x * x; a = a * a; a = a * a; a = a * a; return a * a; }
  return glsl_pow(x, T(e));
}

struct Setup {
  const orc_scene* s;
  View view;
  std::vector<BrickR> bricks;
  std::vector<int> visible;   // bricks that pass ContainsData
  float trans_scale, grad_scale, step_scale;
  float iso_norm;             // fIsoval (AbstrRenderer::GetNormalizedIsovalue)
  float proj_x, proj_y;       // vProjParam (CullingLOD::GetDepthScaleParams)
  float iso_diffuse[3];       // diffuse colour * m_vIsoColor (GLRenderer.cpp:2807)
  std::vector<float> tf;      // effective RGBA (after RGBA8 truncation if any)
  float light_a[3], light_d[3], light_s[3];
  float domain_scale[3];
  double norm_mat[3][3];
  // ClearView: focus isovalue, diffuse colour and the focus point in eye
  // space; per-pixel hit records (context pos + parameter, normal, focus pos +
  // parameter, normal) and the size of the target the frame is drawn into
  float cv_iso_norm = 0.0f, cv_diffuse[3] = {0, 0, 0}, cv_pick[3] = {0, 0, 0};
  double* cv_rec = nullptr;
  uint32_t fbo_w = 0, fbo_h = 0;
  // clip plane: model-space plane and its eye-space form, bricks wholly cut away
  float clip_model[4], clip_eye[4];
  std::vector<char> clipped;
};

// The clip plane in model space: the normal normalised, d kept
// (GLRaycaster.cpp:328-337 with an identity model transform).
void clip_model_plane(const float plane[4], float out[4]) {
  const float len = std::sqrt((plane[0] * plane[0] + plane[1] * plane[1]) + plane[2] * plane[2]);
  for (int a = 0; a < 3; ++a) out[a] = plane[a] / len;
  out[3] = plane[3];
}

// AbstrRenderer::Clipped (AbstrRenderer.cpp:923-948): every corner of the
// brick box on the cut side
bool brick_clipped(const float pl[4], const float pmin[3], const float pmax[3]) {
  for (int c = 0; c < 8; ++c) {
    const float x = (c & 4) ? pmax[0] : pmin[0];
    const float y = (c & 2) ? pmax[1] : pmin[1];
    const float z = (c & 1) ? pmax[2] : pmin[2];
    if (!(((pl[0] * x + pl[1] * y) + pl[2] * z) + pl[3] >= 0.0f)) return false;
  }
  return true;
}

// Ray parameters [lo, hi] kept by the clip plane along the eye-space ray
// dir * t: the cut is where the plane's eye-space form changes sign.
inline void clip_range(const float ce[4], const float dir[3], float& lo, float& hi) {
  const float s = std::fma(ce[2], dir[2], std::fma(ce[1], dir[1], ce[0] * dir[0]));
  lo = -INFINITY;
  hi = INFINITY;
  if (s > 0.0f) hi = -ce[3] / s;
  else if (s < 0.0f) lo = -ce[3] / s;
  else if (ce[3] > 0.0f) { lo = INFINITY; hi = -INFINITY; }
}

template <class T>
void lighting_ref(const Setup& st, const T pos[3], const T N[3], const T tfc[3], T out[3]) {
  // lighting.glsl:33-43 via VRender1DLit.glsl:67-68 (diffuse colour * TF colour)
  // normalize() as a multiply by the correctly rounded reciprocal length
  T p[3] = {-pos[0], -pos[1], -pos[2]};
  const T ilp = T(1) / len3(p[0], p[1], p[2]);
  T V[3] = {p[0] * ilp, p[1] * ilp, p[2] * ilp};
  const T d = dot3(N, V);
  T R[3];
  for (int i = 0; i < 3; ++i) R[i] = V[i] - (T(2) * d) * N[i];
  const T ilr = T(1) / len3(R[0], R[1], R[2]);
  for (int i = 0; i < 3; ++i) R[i] = R[i] * ilr;
  const T L[3] = {T(st.s->light_dir[0]), T(st.s->light_dir[1]), T(st.s->light_dir[2])};
  const T diff = std::fmax(std::fabs(dot3(N, L)), T(0));
  const T spec = pow_int_or_real(std::fmax(dot3(R, L), T(0)), 8.0f);
  for (int i = 0; i < 3; ++i) {
    const T dcol = T(st.light_d[i]) * tfc[i];
    T c = T(st.light_a[i]) + dcol * diff;
    c = c + T(st.light_s[i]) * spec;
    out[i] = std::fmin(std::fmax(c, T(0)), T(1));
  }
}

template <class T>
void lighting_bp(const Setup& st, const T pos[3], const T Nin[3], const T tfc[3], T out[3]) {
  // Blinn-Phong (selectable model): two-sided, half vector, ka/kd/ks/shininess.
  const orc_scene& s = *st.s;
  T p[3] = {-pos[0], -pos[1], -pos[2]};
  const T ilp = T(1) / len3(p[0], p[1], p[2]);
  T V[3] = {p[0] * ilp, p[1] * ilp, p[2] * ilp};
  T N[3] = {Nin[0], Nin[1], Nin[2]};
  if (dot3(N, V) < T(0)) { N[0] = -N[0]; N[1] = -N[1]; N[2] = -N[2]; }
  const T Lt[3] = {-T(s.light_dir[0]), -T(s.light_dir[1]), -T(s.light_dir[2])};
  T H[3] = {Lt[0] + V[0], Lt[1] + V[1], Lt[2] + V[2]};
  const T ilh = T(1) / len3(H[0], H[1], H[2]);
  for (int i = 0; i < 3; ++i) H[i] = H[i] * ilh;
  const T diff = std::fmax(dot3(N, Lt), T(0));
  const T spec = pow_int_or_real(std::fmax(dot3(N, H), T(0)), s.bp_shininess);
  for (int i = 0; i < 3; ++i) {
    T c = T(s.bp_ka) * tfc[i];
    c = c + (T(s.bp_kd) * tfc[i]) * diff;
    c = c + T(s.bp_ks) * spec;
    out[i] = std::fmin(std::fmax(c, T(0)), T(1));
  }
}

template <class T>
void brick_march(const Setup& st, const BrickR& b, const float dir[3], float t_in,
                 float t_out, T col[4], uint64_t& samples) {
  const orc_scene& s = *st.s;
  Vol<T> vol{&b, s.dtype, T(s.dtype == 1 ? 1.0f / 65535.0f : 1.0f / 255.0f)};
  // GLRaycaster.cpp:93-99: entry eye position passes through an RGBA16F target
  float en[3], ex[3];
  for (int a = 0; a < 3; ++a) {
    en[a] = orc_round_half(dir[a] * t_in);
    ex[a] = dir[a] * t_out;
  }
  // GLRaycaster-1D-FS.glsl:60-69
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = std::sqrt((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row<float>(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row<float>(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const float q = len / b.step;
  const int n = int(q) + 1;
  T inc[3], pos[3], epos[3], einc[3];
  const T iq = T(1) / T(q);  // the increment: a multiply by the step count's reciprocal
  for (int a = 0; a < 3; ++a) {
    inc[a] = T(tout[a] - tin[a]) * iq;
    pos[a] = T(tin[a]);
    epos[a] = T(en[a]);
  }
  // GLRaycaster-1D-light-FS.glsl:100-107: eye-space increment of the lit march
  {
    const T ddx = T(ex[0]) - T(en[0]), ddy = T(ex[1]) - T(en[1]), ddz = T(ex[2]) - T(en[2]);
    const T l = len3(ddx, ddy, ddz);
    const T il = T(1) / l;
    einc[0] = (ddx * il) * T(b.step);
    einc[1] = (ddy * il) * T(b.step);
    einc[2] = (ddz * il) * T(b.step);
  }
  const T vstep[3] = {T(1.0f / float(b.n[0])), T(1.0f / float(b.n[1])), T(1.0f / float(b.n[2]))};
  const bool lit = s.lighting != 0;
  const bool two_d = s.render_mode == ORC_RM_2D;
  const uint32_t W = s.tf_w, H = s.tf_h;
  T c[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    ++samples;
    const T v = vol.sample(pos[0], pos[1], pos[2]);
    T g[3] = {0, 0, 0};
    if (lit || two_d) {
      // Volume3D.glsl:43-54 (note Yp is taken at -step.y)
      const T xp = vol.sample(pos[0] + vstep[0], pos[1], pos[2]);
      const T xm = vol.sample(pos[0] + (-vstep[0]), pos[1], pos[2]);
      const T yp = vol.sample(pos[0], pos[1] + (-vstep[1]), pos[2]);
      const T ym = vol.sample(pos[0], pos[1] + vstep[1], pos[2]);
      const T zp = vol.sample(pos[0], pos[1], pos[2] + vstep[2]);
      const T zm = vol.sample(pos[0], pos[1], pos[2] + (-vstep[2]));
      g[0] = (xm - xp) / T(2);
      g[1] = (yp - ym) / T(2);
      g[2] = (zm - zp) / T(2);
    }
    size_t ti;
    if (!two_d) {
      // VRender1D.glsl:43-47, texture1D with GL_NEAREST + clamp to edge
      const T u = v * T(st.trans_scale);
      T fi = std::floor(u * T(W));
      fi = std::fmin(std::fmax(fi, T(0)), T(W - 1));
      ti = size_t(fi);
    } else {
      // GLRaycaster-2D-FS.glsl:75-80
      const T mag = len3(g[0], g[1], g[2]);
      const T u = v * T(st.trans_scale);
      const T w = T(1) - mag * T(st.grad_scale);
      T fx = std::floor(u * T(W)), fy = std::floor(w * T(H));
      fx = std::fmin(std::fmax(fx, T(0)), T(W - 1));
      fy = std::fmin(std::fmax(fy, T(0)), T(H - 1));
      ti = size_t(fy) * W + size_t(fx);
    }
    const float* e = &st.tf[4 * ti];
    T src[4] = {T(e[0]), T(e[1]), T(e[2]), T(e[3])};
    // VRender1D.glsl:53: opacity correction
    src[3] = T(1) - std::pow(T(1) - src[3], T(st.step_scale));
    if (lit) {
      // Volume3D.glsl:56-60: normal = normalize(NormalMatrix * (g * DomainScale))
      const T gs[3] = {g[0] * T(st.domain_scale[0]), g[1] * T(st.domain_scale[1]),
                       g[2] * T(st.domain_scale[2])};
      T N[3];
      for (int r = 0; r < 3; ++r)
        N[r] = std::fma(T(float(st.norm_mat[r][2])), gs[2],
                        std::fma(T(float(st.norm_mat[r][1])), gs[1],
                                 T(float(st.norm_mat[r][0])) * gs[0]));
      const T l = len3(N[0], N[1], N[2]);
      if (l > T(0)) {
        const T il = T(1) / l;
        N[0] = N[0] * il; N[1] = N[1] * il; N[2] = N[2] * il;
      }
      T lc[3];
      const T tfc[3] = {src[0], src[1], src[2]};
      if (s.light_model == ORC_LIGHT_BLINN_PHONG)
        lighting_bp<T>(st, epos, N, tfc, lc);
      else
        lighting_ref<T>(st, epos, N, tfc, lc);
      src[0] = lc[0]; src[1] = lc[1]; src[2] = lc[2];
      if (two_d) {  // GLRaycaster-2D-light-FS.glsl:107
        src[3] = std::fmin(std::fmax(src[3], T(0)), T(1));
      }
    }
    // Compositing.glsl:33-38 UnderCompositing
    const T w = T(1) - c[3];
    c[0] = std::fma(src[0] * w, src[3], c[0]);
    c[1] = std::fma(src[1] * w, src[3], c[1]);
    c[2] = std::fma(src[2] * w, src[3], c[2]);
    c[3] = std::fma(src[3], w, c[3]);
    for (int a = 0; a < 3; ++a) {
      pos[a] = pos[a] + inc[a];
      epos[a] = epos[a] + einc[a];
    }
    if (c[3] >= T(0.99f)) break;
  }
  for (int a = 0; a < 4; ++a) col[a] = c[a];
}

// GLRaycaster-ISO-FS.glsl:51-105 for one brick: first sample >= fIsoval,
// RefineIsosurface.glsl:37-52 (5 bisection steps from half a step back), the
// eye-space hit interpolated by |hit - entry| / |exit - entry| in texture
// space, its non-linear depth and the normal (Volume3D.glsl:56-60).
// kCV: GLRaycaster-ISO-CV-FS.glsl:56-115, the ClearView focus pass at
// isovalue iso_cv: the texture-space entry moves to parameter p_start
// (GLSL: entryTex * (1 - p) + exitTex * p) while the eye-space entry stays
// (the shader blends vRayEntry with itself), so the step count and the
// eye-space interpolation use the whole brick; the depth written is the ray
// exit's (gl_FragDepth from vEyePos).
template <class T, bool kCV = false>
bool iso_brick(const Setup& st, const BrickR& b, const float dir[3], float t_in, float t_out,
               T hit_eye[3], T& fpar, T nrm[3], T& depth, uint64_t& samples,
               float iso_cv = 0.0f, T p_start = T(0)) {
  const orc_scene& s = *st.s;
  Vol<T> vol{&b, s.dtype, T(s.dtype == 1 ? 1.0f / 65535.0f : 1.0f / 255.0f)};
  float en[3], ex[3];
  for (int a = 0; a < 3; ++a) {
    en[a] = orc_round_half(dir[a] * t_in);
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = std::sqrt((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row<float>(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row<float>(b.tex[a], ex[0], ex[1], ex[2]);
  }
  if (kCV)
    for (int a = 0; a < 3; ++a)
      tin[a] = float(T(tin[a]) * (T(1) - p_start) + T(tout[a]) * p_start);
  const T len_tex = len3(T(tout[0] - tin[0]), T(tout[1] - tin[1]), T(tout[2] - tin[2]));
  const float q = len / b.step;
  if (!(q < 1.0e6f)) return false;
  const int n = int(q) + 1;
  T inc[3], pos[3];
  const T iq = T(1) / T(q);  // the increment: a multiply by the step count's reciprocal
  for (int a = 0; a < 3; ++a) {
    inc[a] = T(tout[a] - tin[a]) * iq;
    pos[a] = T(tin[a]);
  }
  const T iso = T(kCV ? iso_cv : st.iso_norm);
  bool hit = false;
  for (int i = 0; i < n; ++i) {
    ++samples;
    if (vol.sample(pos[0], pos[1], pos[2]) >= iso) { hit = true; break; }
    for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
  }
  if (!hit) return false;
  T d[3], cur[3];
  for (int a = 0; a < 3; ++a) {
    d[a] = inc[a] / T(2);
    cur[a] = pos[a] - d[a];
  }
  for (int k = 0; k < 5; ++k) {
    for (int a = 0; a < 3; ++a) d[a] = d[a] / T(2);
    const bool above = vol.sample(cur[0], cur[1], cur[2]) >= iso;
    for (int a = 0; a < 3; ++a) cur[a] = above ? cur[a] - d[a] : cur[a] + d[a];
  }
  fpar = len3(cur[0] - T(tin[0]), cur[1] - T(tin[1]), cur[2] - T(tin[2])) / len_tex;
  for (int a = 0; a < 3; ++a) hit_eye[a] = T(en[a]) * (T(1) - fpar) + T(ex[a]) * fpar;
  depth = T(st.proj_x) + (T(st.proj_y) / -(kCV ? T(ex[2]) : hit_eye[2]));
  // normal at the refined position
  const T vs[3] = {T(1.0f / float(b.n[0])), T(1.0f / float(b.n[1])), T(1.0f / float(b.n[2]))};
  const T xp = vol.sample(cur[0] + vs[0], cur[1], cur[2]);
  const T xm = vol.sample(cur[0] + (-vs[0]), cur[1], cur[2]);
  const T yp = vol.sample(cur[0], cur[1] + (-vs[1]), cur[2]);
  const T ym = vol.sample(cur[0], cur[1] + vs[1], cur[2]);
  const T zp = vol.sample(cur[0], cur[1], cur[2] + vs[2]);
  const T zm = vol.sample(cur[0], cur[1], cur[2] + (-vs[2]));
  const T g[3] = {(xm - xp) / T(2), (yp - ym) / T(2), (zm - zp) / T(2)};
  const T gs[3] = {g[0] * T(st.domain_scale[0]), g[1] * T(st.domain_scale[1]),
                   g[2] * T(st.domain_scale[2])};
  for (int r = 0; r < 3; ++r)
    nrm[r] = std::fma(T(float(st.norm_mat[r][2])), gs[2],
                      std::fma(T(float(st.norm_mat[r][1])), gs[1],
                               T(float(st.norm_mat[r][0])) * gs[0]));
  const T l = len3(nrm[0], nrm[1], nrm[2]);
  if (l > T(0)) { nrm[0] = nrm[0] / l; nrm[1] = nrm[1] / l; nrm[2] = nrm[2] / l; }
  return true;
}

// Compose-FS.glsl:40-63 Lighting of the nearest hit (N.z made non-negative;
// diffuse from |N . -L|, specular exponent 8), with the diffuse colour
// `diffuse` (Compose-CV-FS.glsl:48-56 is the same function).
template <class T>
void surface_lighting(const Setup& st, const T pos[3], const T nin[3], const float diffuse[3],
                      T out[3]);

template <class T>
void iso_compose(const Setup& st, const T pos[3], const T nin[3], T out[3]) {
  surface_lighting<T>(st, pos, nin, st.iso_diffuse, out);
}

template <class T>
void surface_lighting(const Setup& st, const T pos[3], const T nin[3], const float diffuse[3],
                      T out[3]) {
  const T N[3] = {nin[0], nin[1], std::fabs(nin[2])};
  T p[3] = {T(0) - pos[0], T(0) - pos[1], T(0) - pos[2]};
  const T lp = len3(p[0], p[1], p[2]);
  const T V[3] = {p[0] / lp, p[1] / lp, p[2] / lp};
  const T d = dot3(N, V);
  T R[3];
  for (int i = 0; i < 3; ++i) R[i] = V[i] - (T(2) * d) * N[i];
  const T lr = len3(R[0], R[1], R[2]);
  for (int i = 0; i < 3; ++i) R[i] = R[i] / lr;
  const T L[3] = {T(st.s->light_dir[0]), T(st.s->light_dir[1]), T(st.s->light_dir[2])};
  const T nL[3] = {-L[0], -L[1], -L[2]};
  const T diff = std::fmax(std::fabs(dot3(N, nL)), T(0));
  const T spec = pow_int_or_real(std::fmax(dot3(R, L), T(0)), 8.0f);
  for (int i = 0; i < 3; ++i) {
    T c = T(st.light_a[i]) + T(diffuse[i]) * diff;
    c = c + T(st.light_s[i]) * spec;
    out[i] = std::fmin(std::fmax(c, T(0)), T(1));
  }
}

// Normal of a colour volume from its red channel (Volume3D.glsl:43-60 reads
// sampleVolume(...).x).
template <class T>
void color_normal(const Setup& st, Vol<T> red, const T pos[3], const T vstep[3], T N[3]) {
  red.ch = 0;
  const T xp = red.sample(pos[0] + vstep[0], pos[1], pos[2]);
  const T xm = red.sample(pos[0] + (-vstep[0]), pos[1], pos[2]);
  const T yp = red.sample(pos[0], pos[1] + (-vstep[1]), pos[2]);
  const T ym = red.sample(pos[0], pos[1] + vstep[1], pos[2]);
  const T zp = red.sample(pos[0], pos[1], pos[2] + vstep[2]);
  const T zm = red.sample(pos[0], pos[1], pos[2] + (-vstep[2]));
  const T gs[3] = {((xm - xp) / T(2)) * T(st.domain_scale[0]),
                   ((yp - ym) / T(2)) * T(st.domain_scale[1]),
                   ((zm - zp) / T(2)) * T(st.domain_scale[2])};
  for (int r = 0; r < 3; ++r)
    N[r] = std::fma(T(float(st.norm_mat[r][2])), gs[2],
                    std::fma(T(float(st.norm_mat[r][1])), gs[1], T(float(st.norm_mat[r][0])) * gs[0]));
  const T l = len3(N[0], N[1], N[2]);
  if (l > T(0)) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
}

// A brick of a colour volume in 1D mode: GLRaycaster-1D-FS.glsl /
// -1D-light-FS.glsl with VRender1D-Color.glsl:44-53 and VRender1DLit-Color.glsl:
// 44-62 -- the filtered RGBA times the TF entry at (r + g + b) / 3, opacity
// correction of the product's alpha, lit with the product's colour.
template <class T>
void brick_march_color(const Setup& st, const BrickR& b, const float dir[3], float t_in,
                       float t_out, T col[4], uint64_t& samples) {
  const orc_scene& s = *st.s;
  Vol<T> vol{&b, 2, T(1.0f / 255.0f)};
  float en[3], ex[3];
  for (int a = 0; a < 3; ++a) {
    en[a] = orc_round_half(dir[a] * t_in);
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = std::sqrt((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row<float>(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row<float>(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const float q = len / b.step;
  const int n = int(q) + 1;
  T inc[3], pos[3], epos[3], einc[3];
  const T iq = T(1) / T(q);  // the increment: a multiply by the step count's reciprocal
  for (int a = 0; a < 3; ++a) {
    inc[a] = T(tout[a] - tin[a]) * iq;
    pos[a] = T(tin[a]);
    epos[a] = T(en[a]);
  }
  {
    const T ddx = T(ex[0]) - T(en[0]), ddy = T(ex[1]) - T(en[1]), ddz = T(ex[2]) - T(en[2]);
    const T l = len3(ddx, ddy, ddz);
    const T il = T(1) / l;
    einc[0] = (ddx * il) * T(b.step);
    einc[1] = (ddy * il) * T(b.step);
    einc[2] = (ddz * il) * T(b.step);
  }
  const T vstep[3] = {T(1.0f / float(b.n[0])), T(1.0f / float(b.n[1])), T(1.0f / float(b.n[2]))};
  const uint32_t W = s.tf_w;
  T c[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    ++samples;
    T v[4];
    for (int k = 0; k < 4; ++k) {
      vol.ch = k;
      v[k] = vol.sample(pos[0], pos[1], pos[2]);
    }
    const T u = ((v[0] + v[1]) + v[2]) / T(3);
    T fi = std::floor(u * T(W));
    fi = std::fmin(std::fmax(fi, T(0)), T(W - 1));
    const float* e = &st.tf[4 * size_t(fi)];
    T src[4] = {v[0] * T(e[0]), v[1] * T(e[1]), v[2] * T(e[2]), v[3] * T(e[3])};
    src[3] = T(1) - glsl_pow(T(1) - src[3], T(st.step_scale));
    if (s.lighting && src[3] != T(0)) {
      T N[3], lc[3];
      color_normal<T>(st, vol, pos, vstep, N);
      const T tfc[3] = {src[0], src[1], src[2]};
      if (s.light_model == ORC_LIGHT_BLINN_PHONG)
        lighting_bp<T>(st, epos, N, tfc, lc);
      else
        lighting_ref<T>(st, epos, N, tfc, lc);
      src[0] = lc[0]; src[1] = lc[1]; src[2] = lc[2];
    }
    const T w = T(1) - c[3];
    c[0] = std::fma(src[0] * w, src[3], c[0]);
    c[1] = std::fma(src[1] * w, src[3], c[1]);
    c[2] = std::fma(src[2] * w, src[3], c[2]);
    c[3] = std::fma(src[3], w, c[3]);
    for (int a = 0; a < 3; ++a) {
      pos[a] = pos[a] + inc[a];
      epos[a] = epos[a] + einc[a];
    }
    if (c[3] >= T(0.99f)) break;
  }
  for (int a = 0; a < 4; ++a) col[a] = c[a];
}

// GLRaycaster-Color-FS.glsl for one brick: the first step whose alpha is >=
// fIsoval, RefineIsosurface on the red channel, the red channel's normal, and
// the colour at the unrefined step packed into the two hit buffers' alphas
// (red + 1; floor(green * 512) + blue).
template <class T>
bool iso_brick_color(const Setup& st, const BrickR& b, const float dir[3], float t_in,
                     float t_out, T hit_eye[3], T nrm[3], T& depth, T& enc_r, T& enc_gb,
                     uint64_t& samples) {
  Vol<T> vol{&b, 2, T(1.0f / 255.0f)};
  float en[3], ex[3];
  for (int a = 0; a < 3; ++a) {
    en[a] = orc_round_half(dir[a] * t_in);
    ex[a] = dir[a] * t_out;
  }
  const float dx = ex[0] - en[0], dy = ex[1] - en[1], dz = ex[2] - en[2];
  const float len = std::sqrt((dx * dx + dy * dy) + dz * dz);
  float tin[3], tout[3];
  for (int a = 0; a < 3; ++a) {
    tin[a] = affine_row<float>(b.tex[a], en[0], en[1], en[2]);
    tout[a] = affine_row<float>(b.tex[a], ex[0], ex[1], ex[2]);
  }
  const T len_tex = len3(T(tout[0] - tin[0]), T(tout[1] - tin[1]), T(tout[2] - tin[2]));
  const float q = len / b.step;
  if (!(q < 1.0e6f)) return false;
  const int n = int(q) + 1;
  T inc[3], pos[3];
  const T iq = T(1) / T(q);  // the increment: a multiply by the step count's reciprocal
  for (int a = 0; a < 3; ++a) {
    inc[a] = T(tout[a] - tin[a]) * iq;
    pos[a] = T(tin[a]);
  }
  const T iso = T(st.iso_norm);
  bool hit = false;
  vol.ch = 3;
  for (int i = 0; i < n; ++i) {
    ++samples;
    if (vol.sample(pos[0], pos[1], pos[2]) >= iso) { hit = true; break; }
    for (int a = 0; a < 3; ++a) pos[a] = pos[a] + inc[a];
  }
  if (!hit) return false;
  T d[3], cur[3];
  for (int a = 0; a < 3; ++a) {
    d[a] = inc[a] / T(2);
    cur[a] = pos[a] - d[a];
  }
  vol.ch = 0;
  for (int k = 0; k < 5; ++k) {
    for (int a = 0; a < 3; ++a) d[a] = d[a] / T(2);
    const bool above = vol.sample(cur[0], cur[1], cur[2]) >= iso;
    for (int a = 0; a < 3; ++a) cur[a] = above ? cur[a] - d[a] : cur[a] + d[a];
  }
  T rgb[3];
  for (int k = 0; k < 3; ++k) {
    vol.ch = k;
    rgb[k] = vol.sample(pos[0], pos[1], pos[2]);
  }
  const T fpar = len3(cur[0] - T(tin[0]), cur[1] - T(tin[1]), cur[2] - T(tin[2])) / len_tex;
  for (int a = 0; a < 3; ++a) hit_eye[a] = T(en[a]) * (T(1) - fpar) + T(ex[a]) * fpar;
  depth = T(st.proj_x) + (T(st.proj_y) / -hit_eye[2]);
  const T vs[3] = {T(1.0f / float(b.n[0])), T(1.0f / float(b.n[1])), T(1.0f / float(b.n[2]))};
  color_normal<T>(st, vol, cur, vs, nrm);
  enc_r = rgb[0] + T(1);
  enc_gb = std::floor(rgb[1] * T(512)) + rgb[2];
  return true;
}

template <class T>
void render_pixel(const Setup& st, uint32_t px, uint32_t py, float* out, uint32_t* spp,
                  uint64_t& samples) {
  const orc_scene& s = *st.s;
  const View& v = st.view;
  // gl_FragCoord at the pixel centre -> eye-space ray through it (z = -1)
  const float nx = (float(px) + 0.5f) * v.inv_w2 - 1.0f;
  const float ny = (float(py) + 0.5f) * v.inv_h2 - 1.0f;
  const float dir[3] = {nx * v.kx, ny * v.ky, -1.0f};
  float o[3], d[3];
  for (int a = 0; a < 3; ++a) {
    o[a] = float(v.inv[a][3]);
    d[a] = std::fma(float(v.inv[a][2]), dir[2],
                    std::fma(float(v.inv[a][1]), dir[1], float(v.inv[a][0]) * dir[0]));
  }
  float inv[3];
  for (int a = 0; a < 3; ++a) inv[a] = 1.0f / d[a];
  struct Hit { float t0, t1; int b; };
  std::vector<Hit> hits;
  float clip_lo = -INFINITY, clip_hi = INFINITY;
  if (s.clip_on) clip_range(st.clip_eye, dir, clip_lo, clip_hi);
  for (int bi : st.visible) {
    if (s.clip_on && st.clipped[bi]) continue;
    const BrickR& b = st.bricks[bi];
    float tn = -INFINITY, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
      const float t0 = (b.pmin[a] - o[a]) * inv[a];
      const float t1 = (b.pmax[a] - o[a]) * inv[a];
      tn = std::fmax(tn, std::fmin(t0, t1));
      tf = std::fmin(tf, std::fmax(t0, t1));
    }
    // near-plane quad (GLRaycaster.cpp:350-369) supplies the entry when the
    // front faces are clipped; a back face behind the far plane is clipped.
    const float ti = std::fmax(tn, s.znear);
    if (!(tf > ti) || tf > s.zfar) continue;
    // the clipped box's front faces (its cap included) and back faces
    const float ci = std::fmax(ti, clip_lo), cf = std::fmin(tf, clip_hi);
    if (!(cf > ci)) continue;
    hits.push_back({ci, cf, bi});
  }
  std::sort(hits.begin(), hits.end(), [](const Hit& a, const Hit& b) {
    return a.t0 < b.t0 || (a.t0 == b.t0 && a.b < b.b);
  });
  T frame[4] = {0, 0, 0, 0};
  const uint64_t before = samples;
  if (s.dtype == 2 && s.render_mode == ORC_RM_ISO) {
    // colour: nearest hit by the depth test, Compose-Color-FS.glsl:60-88 (the
    // hit buffer's alpha is red + 1, never 0)
    T best_depth = T(1), pos[3] = {0, 0, 0}, nrm[3] = {0, 0, 0}, er = 0, egb = 0;
    bool any = false;
    for (const Hit& h : hits) {
      T hp[3], hn[3], depth, r1, gb;
      if (!iso_brick_color<T>(st, st.bricks[h.b], dir, h.t0, h.t1, hp, hn, depth, r1, gb,
                              samples))
        continue;
      if (!(depth < best_depth)) continue;
      best_depth = depth;
      for (int a = 0; a < 3; ++a) { pos[a] = hp[a]; nrm[a] = hn[a]; }
      er = r1;
      egb = gb;
      any = true;
    }
    if (any) {
      const T rgb[3] = {er - T(1), std::floor(egb / T(2)) / T(256), egb - std::floor(egb)};
      const T n[3] = {nrm[0], nrm[1], std::fabs(nrm[2])};
      float dcol[3];  // vColor.rgb * vLightDiffuse
      T c[3];
      for (int a = 0; a < 3; ++a) dcol[a] = float(rgb[a] * T(st.light_d[a]));
      surface_lighting<T>(st, pos, n, dcol, c);
      frame[0] = c[0]; frame[1] = c[1]; frame[2] = c[2]; frame[3] = T(1);
    }
  } else if (s.render_mode == ORC_RM_ISO && s.cv_on) {
    // ClearView (GLRaycaster.cpp:421-436): per brick, in list order, the
    // context pass into m_pFBOIsoHit (depth test on the hit depth; normal.w =
    // the brick's tile ID), then the focus pass into m_pFBOCVHit, which starts
    // at the context hit when the hit buffer's tile ID is this brick's (the
    // cleared buffer reads tile 0 with parameter 0, a start at the entry).
    T best_depth = T(1), pos[3] = {0, 0, 0}, nrm[3] = {0, 0, 0}, fpar = 0;
    T cv_depth = T(1), pos2[3] = {0, 0, 0}, nrm2[3] = {0, 0, 0}, fpar2 = 0;
    bool any = false, any2 = false;
    int last_tile = 0;
    for (const Hit& h : hits) {
      T hp[3], hn[3], f, depth;
      if (iso_brick<T>(st, st.bricks[h.b], dir, h.t0, h.t1, hp, f, hn, depth, samples) &&
          depth < best_depth) {
        best_depth = depth;
        for (int a = 0; a < 3; ++a) { pos[a] = hp[a]; nrm[a] = hn[a]; }
        fpar = f;
        any = true;
        last_tile = h.b;
      }
      const T p_start = (last_tile == h.b) ? fpar : T(0);
      if (iso_brick<T, true>(st, st.bricks[h.b], dir, h.t0, h.t1, hp, f, hn, depth, samples,
                             st.cv_iso_norm, p_start) &&
          depth < cv_depth) {
        cv_depth = depth;
        for (int a = 0; a < 3; ++a) { pos2[a] = hp[a]; nrm2[a] = hn[a]; }
        fpar2 = f;
        any2 = true;
      }
    }
    double* rec = st.cv_rec + 16 * (size_t(py) * s.width + px);
    for (int k = 0; k < 16; ++k) rec[k] = 0.0;
    if (any) {
      for (int a = 0; a < 3; ++a) { rec[a] = double(pos[a]); rec[4 + a] = double(nrm[a]); }
      rec[3] = double(fpar);
    }
    if (any2) {
      for (int a = 0; a < 3; ++a) { rec[8 + a] = double(pos2[a]); rec[12 + a] = double(nrm2[a]); }
      rec[11] = double(fpar2);
    }
  } else if (s.render_mode == ORC_RM_ISO) {
    // every brick writes its refined hit through a depth test (DF_LESS on a
    // buffer cleared to 1, GLRenderer.cpp:140-141, GLRaycaster.cpp:423-433)
    T best_depth = T(1), pos[3] = {0, 0, 0}, nrm[3] = {0, 0, 0}, fpar = 0;
    bool any = false;
    for (const Hit& h : hits) {
      T hp[3], hn[3], f, depth;
      if (!iso_brick<T>(st, st.bricks[h.b], dir, h.t0, h.t1, hp, f, hn, depth, samples)) continue;
      if (!(depth < best_depth)) continue;
      best_depth = depth;
      for (int a = 0; a < 3; ++a) { pos[a] = hp[a]; nrm[a] = hn[a]; }
      fpar = f;
      any = true;
    }
    // Compose-FS.glsl:49-76: alpha (the interpolation parameter) 0 means no hit
    if (any && fpar != T(0)) {
      T c[3];
      iso_compose<T>(st, pos, nrm, c);
      frame[0] = c[0]; frame[1] = c[1]; frame[2] = c[2]; frame[3] = T(1);
    }
  } else {
    for (const Hit& h : hits) {
      if (frame[3] >= T(s.frame_ert)) break;
      T c[4];
      if (s.dtype == 2)
        brick_march_color<T>(st, st.bricks[h.b], dir, h.t0, h.t1, c, samples);
      else
        brick_march<T>(st, st.bricks[h.b], dir, h.t0, h.t1, c, samples);
      // GLRenderer.cpp:151-153 blend (ONE_MINUS_DST_ALPHA, ONE) into RGBA32F
      const T w = T(1) - frame[3];
      for (int a = 0; a < 4; ++a) frame[a] = std::fma(c[a], w, frame[a]);
    }
  }
  for (int a = 0; a < 4; ++a) out[a] = float(frame[a]);
  if (spp) *spp = uint32_t(samples - before);
}

Setup build_setup(const orc_scene& s) {
  Setup st;
  st.s = &s;
  const bool color = s.dtype == 2;  // RGBA8: LOD 0, no statistics, every brick drawn
  const int bytes = color ? 4 : (s.dtype == 0 ? 1 : 2);
  const int bits = color ? 8 : 8 * bytes;  // Dataset::GetBitWidth (per channel)
  uint64_t lod_all[3 * 64], cnt_all[3 * 64];
  const int n_lods = orc_lod_table(s.dims, s.brick_size, s.overlap, lod_all, cnt_all, 64);
  // the rendered LOD (AbstrRenderer m_iCurrentLOD); its bricks, metadata and aspect
  const uint32_t L = std::min<uint32_t>(s.lod, uint32_t(n_lods - 1));
  const uint64_t* lod = &lod_all[3 * L];
  const uint64_t* cnt = &cnt_all[3 * L];
  const uint64_t nb = cnt[0] * cnt[1] * cnt[2];
  std::vector<float> ctr(3 * nb), ext(3 * nb);
  std::vector<uint32_t> nv(3 * nb);
  double asp[3];
  orc_lod_aspect(s.dims, L, asp);
  orc_brick_metadata(lod, cnt, s.brick_size, s.overlap, asp, ctr.data(), ext.data(), nv.data());
  // LOD >= 1 bricks: the ComputeHierarchy + FillOverlap restatement
  std::vector<uint8_t> octree;
  std::vector<uint64_t> octree_off;
  uint64_t lod_first = 0;
  if (L > 0) {
    uint64_t total_vox = 0, total_bricks = 0;
    for (int l = 0; l < n_lods; ++l) {
      const uint64_t* ls = &lod_all[3 * l];
      const uint64_t* lc = &cnt_all[3 * l];
      if (uint32_t(l) == L) lod_first = total_bricks;
      for (uint64_t k = 0; k < lc[0] * lc[1] * lc[2]; ++k) {
        const uint64_t c3[3] = {k % lc[0], (k / lc[0]) % lc[1], k / (lc[0] * lc[1])};
        uint64_t bs[3];
        orc_brick_size(ls, lc, s.brick_size, s.overlap, c3, bs);
        total_vox += bs[0] * bs[1] * bs[2];
        ++total_bricks;
      }
    }
    octree.resize(total_vox * bytes);
    octree_off.resize(total_bricks);
    orc_build_octree(s.raw, s.dtype, s.dims, s.brick_size, s.overlap, s.clamp_to_edge, s.median,
                     octree.data(), total_vox, octree_off.data(), total_bricks);
  }

  // AbstrRenderer.cpp:1003-1012: scale applied to brick metadata
  const float us[3] = {float(s.user_scale[0]), float(s.user_scale[1]), float(s.user_scale[2])};
  float dcs[3];
  const float dmax = float(std::max(s.dims[0], std::max(s.dims[1], s.dims[2])));
  for (int a = 0; a < 3; ++a) dcs[a] = us[a] * float(s.dims[a]) / dmax;
  const float dcmax = std::max(dcs[0], std::max(dcs[1], dcs[2]));
  float vs[3];
  for (int a = 0; a < 3; ++a) vs[a] = us[a] / dcmax;

  // data range (dataset GetRange) and TF non-zero limits
  const uint64_t nvox = s.dims[0] * s.dims[1] * s.dims[2];
  double rmax = 0, rmin = 1e300;
  if (color) { rmin = 0; rmax = 255; }
#pragma omp parallel for reduction(max : rmax) reduction(min : rmin)
  for (int64_t ii = 0; ii < int64_t(color ? 0 : nvox); ++ii) {
    const uint64_t i = uint64_t(ii);
    const double x = bytes == 1 ? double(static_cast<const uint8_t*>(s.raw)[i])
                                : double(static_cast<const uint16_t*>(s.raw)[i]);
    rmax = std::max(rmax, x);
    rmin = std::min(rmin, x);
  }
  // GLRenderer.cpp:1813-1819 CalculateScaling: (2^bits-1)/MaxValue; with bias
  // and scale in 1D mode GLRaycaster.cpp:577-584 sets fTransScale to
  // scale_bias_and_scale's |min| + |max| (TFScaling.cpp)
  const uint32_t imax = (1u << bits) - 1;
  st.trans_scale = (s.render_mode == ORC_RM_1D && s.tf_bias_scale)
                       ? std::fabs(float(rmin)) + std::fabs(float(rmax))
                       : float(double(imax) / rmax);
  // GLRenderer.cpp:1840-1841: fGradientScale = 1 / MaxGradientMagnitude
  st.grad_scale = 1.0f;
  if (s.render_mode == ORC_RM_2D) {
    const float mg = float(orc_max_gradient(s.raw, s.dtype, s.dims, s.brick_size, s.overlap,
                                            s.clamp_to_edge));
    st.grad_scale = (mg == 0) ? 1.0f : 1.0f / mg;
  }
  // GLRaycaster.cpp:253-257: sample rate divided while decreasing it; the
  // opacity-correction exponent grows with the LOD's voxel size
  const float srm = s.sample_rate_modifier /
                    (s.decrease_sampling_rate ? s.sample_dec_factor : 1.0f);
  float dom = 0.0f;
  for (int a = 0; a < 3; ++a) dom = std::max(dom, float(lod_all[a]) / float(lod[a]));
  st.step_scale = 1.0f / srm * dom;

  // transfer function as the GPU sees it
  const size_t ntf = size_t(s.tf_w) * s.tf_h;
  st.tf.assign(s.tf, s.tf + 4 * ntf);
  if (s.tf_rgba8) {
    // TransferFunction1D.cpp:311-330 GetByteArray (clamp, x255, truncate),
    // sampled back as UNORM8
    for (float& x : st.tf) {
      const unsigned char b = (unsigned char)(std::max(0.0f, std::min(x, 1.0f)) * 255);
      x = float(b) / 255.0f;
    }
  }
  // TransferFunction1D.cpp:362-371 ComputeNonZeroLimits over alpha (1D); for 2D
  // the value range of any non-zero alpha column.
  uint64_t nz_lo = s.tf_w, nz_hi = 0;
  for (uint32_t y = 0; y < s.tf_h; ++y)
    for (uint32_t x = 0; x < s.tf_w; ++x)
      if (st.tf[4 * (size_t(y) * s.tf_w + x) + 3] != 0) {
        nz_lo = std::min<uint64_t>(nz_lo, x);
        nz_hi = std::max<uint64_t>(nz_hi, x);
      }
  // AbstrRenderer.cpp:959-974 ContainsData for RM_1DTRANS
  const double rescale = rmax / double(s.tf_w - 1);
  const double lo = double(nz_lo) * rescale, hi = double(nz_hi) * rescale;

  // lights (GLRenderer.cpp:2890-2893): colour.xyz * colour.w
  for (int a = 0; a < 3; ++a) {
    st.light_a[a] = s.ambient[a] * s.ambient[3];
    st.light_d[a] = s.diffuse[a] * s.diffuse[3];
    st.light_s[a] = s.specular[a] * s.specular[3];
    st.domain_scale[a] = 1.0f / float(s.user_scale[a]);
    st.iso_diffuse[a] = st.light_d[a] * s.iso_color[a];
  }
  // AbstrRenderer.cpp:412-424: fIsoval = isovalue / 2^bits (not 2^bits - 1)
  st.iso_norm = float(double(s.isovalue) / double(1u << bits));
  // AbstrRenderer.cpp:426-438 GetNormalizedCVIsovalue; GLRenderer.cpp:2784
  st.cv_iso_norm = float(double(s.cv_isovalue) / double(1u << bits));
  for (int a = 0; a < 3; ++a) st.cv_diffuse[a] = st.light_d[a] * s.cv_color[a];
  // CullingLOD.cpp:69-72
  st.proj_x = s.zfar / (s.zfar - s.znear);
  st.proj_y = (s.zfar * s.znear / (s.znear - s.zfar));
  const bool iso_mode = s.render_mode == ORC_RM_ISO;
  st.bricks.resize(nb);
  std::vector<char> contains_flag(nb, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t kk = 0; kk < int64_t(nb); ++kk) {
        const uint64_t k = uint64_t(kk);
        const uint64_t x = k % cnt[0], y = (k / cnt[0]) % cnt[1], z = k / (cnt[0] * cnt[1]);
        BrickR& b = st.bricks[k];
        float c[3], e[3];
        for (int a = 0; a < 3; ++a) {
          b.n[a] = nv[3 * k + a];
          e[a] = ext[3 * k + a] * vs[a];
          c[a] = ctr[3 * k + a] * vs[a];
          b.pmin[a] = c[a] - e[a] / 2.0f;
          b.pmax[a] = c[a] + e[a] / 2.0f;
        }
        // UVFDataset::GetTextCoords (uvfDataset.cpp:1747-1774): the upper
        // corner is scaled by the LOD's brick aspect
        for (int a = 0; a < 3; ++a) {
          b.tmin[a] = float(s.overlap) / float(b.n[a]);
          b.tmax[a] = (1.0f - b.tmin[a]) * float(asp[a]);
        }
        // GLRaycaster.cpp:255: step = min over axes of ext * (1/n) * 0.5 / srm
        float stp = INFINITY;
        for (int a = 0; a < 3; ++a) {
          const float vsz = 1.0f / float(b.n[a]);
          stp = std::min(stp, e[a] * vsz * 0.5f * 1.0f / srm);
        }
        b.step = stp;
        const uint64_t co[3] = {x, y, z};
        const size_t nbytes = size_t(b.n[0]) * b.n[1] * b.n[2] * bytes;
        b.data.resize(nbytes);
        if (L == 0)
          orc_lod0_brick(s.raw, s.dtype, s.dims, s.brick_size, s.overlap, s.clamp_to_edge, co,
                         b.data.data());
        else
          std::memcpy(b.data.data(), octree.data() + octree_off[lod_first + k] * bytes, nbytes);
        double mn = 0, mx = 255;
        if (!color)
          orc_brick_stats(b.data.data(), s.dtype, uint64_t(b.n[0]) * b.n[1] * b.n[2], &mn, &mx);
        // ContainsData: value range vs TF limits, or the isovalue
        // (uvfDataset.cpp:1201-1215); colour bricks always (AbstrRenderer.cpp:955-959)
        if (color)
          contains_flag[k] = 1;
        else if (iso_mode)
          contains_flag[k] = (double(s.isovalue) <= mx) ? 1 : 0;
        else
          contains_flag[k] = (hi >= mn && lo <= mx) ? 1 : 0;
  }
  for (uint64_t k = 0; k < nb; ++k)
    if (contains_flag[k]) st.visible.push_back(int(k));
  return st;
}

// Camera-dependent part: view and per-brick eye -> texture matrices
// (GLRaycaster.cpp:589-612 ComputeEyeToTextureMatrix).
void apply_view(Setup& st) {
  st.view = make_view(*st.s);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) st.norm_mat[r][c] = st.view.mv[r][c];
  // GLRenderer.cpp:2789: vCVPickPos = m_vCVPos * modelView
  for (int r = 0; r < 3; ++r) {
    double e = 0;
    for (int j = 0; j < 4; ++j) e += st.view.mv[r][j] * double(st.s->cv_pos[j]);
    st.cv_pick[r] = float(e);
  }
  st.clipped.assign(st.bricks.size(), 0);
  if (st.s->clip_on) {
    clip_model_plane(st.s->clip_plane, st.clip_model);
    double d = double(st.clip_model[3]);
    for (int j = 0; j < 3; ++j) {
      double n = 0;
      for (int i = 0; i < 3; ++i) n += double(st.clip_model[i]) * st.view.inv[i][j];
      st.clip_eye[j] = float(n);
    }
    for (int i = 0; i < 3; ++i) d += double(st.clip_model[i]) * st.view.inv[i][3];
    st.clip_eye[3] = float(d);
    for (size_t k = 0; k < st.bricks.size(); ++k)
      st.clipped[k] = brick_clipped(st.clip_model, st.bricks[k].pmin, st.bricks[k].pmax) ? 1 : 0;
  }
  for (BrickR& b : st.bricks) {
    for (int a = 0; a < 3; ++a) {
      const double sc = double((b.tmin[a] - b.tmax[a]) / (b.pmin[a] - b.pmax[a]));
      for (int j = 0; j < 3; ++j) b.tex[a][j] = float(sc * st.view.inv[a][j]);
      b.tex[a][3] = float(sc * (st.view.inv[a][3] - double(b.pmax[a])) + double(b.tmax[a]));
    }
  }
}

struct Prepared {
  orc_scene scene;  // volume/TF/mode part; the camera part is replaced per render
  Setup st;
};

// GLRenderer::SetViewPort (GLRenderer.cpp:864-889): the viewport scaled by
// 1/m_fScreenResDecFactor, rounded to the nearest pixel.
void render_size(const orc_scene& s, uint32_t* w, uint32_t* h) {
  *w = s.width;
  *h = s.height;
  if (s.decrease_screen_res) {
    const float rescale = 1.0f / s.screen_res_dec_factor;
    *w = std::max(1u, uint32_t(float(s.width) * rescale + 0.5f));
    *h = std::max(1u, uint32_t(float(s.height) * rescale + 0.5f));
  }
}

// GLRenderer::CopyOverCompletedRegion / FullscreenQuadRegion (GLRenderer.cpp:
// 688-747): viewport pixel x reads texel position (x + 0.5) * rescale - 0.5 of
// the reduced image with GL_LINEAR, clamped to its edge.
void upscale(const float* low, uint32_t lw, uint32_t lh, float* out, uint32_t w, uint32_t h,
             float rescale) {
  auto lerp = [](float a, float b, float t) { return std::fma(t, b - a, a); };
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const float u = (float(x) + 0.5f) * rescale - 0.5f;
      const float v = (float(y) + 0.5f) * rescale - 0.5f;
      const float fu = std::floor(u), fv = std::floor(v);
      const float wx = u - fu, wy = v - fv;
      const int x0 = std::min(std::max(int(fu), 0), int(lw) - 1);
      const int x1 = std::min(std::max(int(fu) + 1, 0), int(lw) - 1);
      const int y0 = std::min(std::max(int(fv), 0), int(lh) - 1);
      const int y1 = std::min(std::max(int(fv) + 1, 0), int(lh) - 1);
      for (int c = 0; c < 4; ++c) {
        const float* r0 = low + 4 * size_t(y0) * lw;
        const float* r1 = low + 4 * size_t(y1) * lw;
        const float a = lerp(r0[4 * x0 + c], r0[4 * x1 + c], wx);
        const float b = lerp(r1[4 * x0 + c], r1[4 * x1 + c], wx);
        out[4 * (size_t(y) * w + x) + c] = lerp(a, b, wy);
      }
    }
}

uint64_t march_rows(Setup& st, float* out, uint32_t* spp, double* march_s);

// Compose-CV-FS.glsl:49-108 over the hit records of a w x h frame drawn at the
// lower left of an fbo_w x fbo_h target.  The neighbour normals are GL_NEAREST
// lookups one texel away with GL_CLAMP (GLRenderer.cpp:1793): clamped at the
// target's edges; beyond a reduced frame's right or top edge the target holds
// the cleared (zero) normal.
template <class T>
void cv_compose(const Setup& st, float* out) {
  const orc_scene& s = *st.s;
  const int w = int(s.width), h = int(s.height);
  const int fw = int(st.fbo_w), fh = int(st.fbo_h);
  auto normal_at = [&](int x, int y, T n[3]) {
    x = std::min(std::max(x, 0), fw - 1);
    y = std::min(std::max(y, 0), fh - 1);
    for (int a = 0; a < 3; ++a)
      n[a] = (x >= w || y >= h) ? T(0) : T(st.cv_rec[16 * (size_t(y) * w + x) + 4 + a]);
  };
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const double* rec = st.cv_rec + 16 * (size_t(y) * w + x);
      float* o = out + 4 * (size_t(y) * w + x);
      if (T(rec[3]) == T(0)) {  // no context hit: discard (the frame stays cleared)
        for (int c = 0; c < 4; ++c) o[c] = 0.0f;
        continue;
      }
      const T pos[3] = {T(rec[0]), T(rec[1]), T(rec[2])};
      const T n[3] = {T(rec[4]), T(rec[5]), T(rec[6])};
      T ctx[4];
      surface_lighting<T>(st, pos, n, st.iso_diffuse, ctx);
      ctx[3] = T(1);
      // curvature estimate: |n(+x) - n| + |n(-x) - n| + |n(+y) - n| + |n(-y) - n|
      T nb[4][3];
      normal_at(x + 1, y, nb[0]);
      normal_at(x - 1, y, nb[1]);
      normal_at(x, y + 1, nb[2]);
      normal_at(x, y - 1, nb[3]);
      T acc[3];
      for (int a = 0; a < 3; ++a) {
        acc[a] = std::fabs(nb[0][a] - n[a]);
        for (int k = 1; k < 4; ++k) acc[a] = acc[a] + std::fabs(nb[k][a] - n[a]);
      }
      const T curvature = len3(acc[0], acc[1], acc[2]);
      const T dist_w = len3(pos[0] - T(st.cv_pick[0]), pos[1] - T(st.cv_pick[1]),
                            pos[2] - T(st.cv_pick[2])) * T(s.cv_size);
      const T blend = std::fmin(
          std::fmax(std::fmax(curvature * T(s.cv_context_scale),
                              std::fmin(std::fmax(dist_w, T(0)), T(1))),
                    T(0)),
          T(1));
      T foc[4] = {0, 0, 0, 0};
      if (T(rec[11]) != T(0)) {
        const T p2[3] = {T(rec[8]), T(rec[9]), T(rec[10])};
        const T n2[3] = {T(rec[12]), T(rec[13]), T(rec[14])};
        surface_lighting<T>(st, p2, n2, st.cv_diffuse, foc);
        foc[3] = T(1);
      }
      T col[4];
      for (int c = 0; c < 4; ++c)
        col[c] = std::fmin(std::fmax(ctx[c] * blend + foc[c] * (T(1) - blend), T(0)), T(1));
      const T dark = T(0.5) * (T(1) - std::fmin(std::fmax(std::fabs(dist_w - T(1)) *
                                                              T(s.cv_border_scale),
                                                          T(0)),
                                                T(1)));
      for (int c = 0; c < 3; ++c) o[c] = float(col[c] - dark);
      o[3] = float(col[3]);
    }
}

uint64_t march_all(Setup& st, float* out, uint32_t* spp, double* march_s) {
  uint32_t rw, rh;
  render_size(*st.s, &rw, &rh);
  st.fbo_w = st.s->width;
  st.fbo_h = st.s->height;
  if (rw == st.s->width && rh == st.s->height) return march_rows(st, out, spp, march_s);
  // reduced viewport: march the smaller image with its own projection, then stretch it
  const orc_scene* full = st.s;
  orc_scene low = *full;
  low.width = rw;
  low.height = rh;
  std::vector<float> img(size_t(rw) * rh * 4, 0.0f);
  st.s = &low;
  const uint64_t n = march_rows(st, img.data(), spp, march_s);
  st.s = full;
  upscale(img.data(), rw, rh, out, full->width, full->height, 1.0f / full->screen_res_dec_factor);
  return n;
}

uint64_t march_rows(Setup& st, float* out, uint32_t* spp, double* march_s) {
  const orc_scene& s = *st.s;
#ifdef _OPENMP
  if (s.threads > 0) omp_set_num_threads(s.threads);
#endif
  apply_view(st);
  const auto t1 = std::chrono::steady_clock::now();
  const uint32_t stride = s.row_stride ? s.row_stride : 1;
  uint64_t total = 0;
  const bool cv = s.render_mode == ORC_RM_ISO && s.cv_on;
  std::vector<double> cv_rec(cv ? size_t(s.width) * s.height * 16 : 0, 0.0);
  st.cv_rec = cv ? cv_rec.data() : nullptr;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (int64_t py = 0; py < int64_t(s.height); ++py) {
    if (uint32_t(py) % stride != s.row_phase % stride) continue;
    uint64_t local = 0;
    for (uint32_t px = 0; px < s.width; ++px) {
      const size_t i = size_t(py) * s.width + px;
      if (s.use_double)
        render_pixel<double>(st, px, uint32_t(py), out + 4 * i, spp ? spp + i : nullptr, local);
      else
        render_pixel<float>(st, px, uint32_t(py), out + 4 * i, spp ? spp + i : nullptr, local);
    }
    total += local;
  }
  if (cv) {
    if (s.use_double) cv_compose<double>(st, out);
    else cv_compose<float>(st, out);
    st.cv_rec = nullptr;
  }
  const auto t2 = std::chrono::steady_clock::now();
  if (march_s) *march_s = std::chrono::duration<double>(t2 - t1).count();
  return total;
}

}  // namespace

extern "C" uint64_t orc_render_timed(const orc_scene* sc, float* out, uint32_t* spp,
                                     double* setup_s, double* march_s) {
#ifdef _OPENMP
  if (sc->threads > 0) omp_set_num_threads(sc->threads);
#endif
  const auto t0 = std::chrono::steady_clock::now();
  Setup st = build_setup(*sc);
  const auto t1 = std::chrono::steady_clock::now();
  if (setup_s) *setup_s = std::chrono::duration<double>(t1 - t0).count();
  return march_all(st, out, spp, march_s);
}

extern "C" uint64_t orc_render(const orc_scene* sc, float* out, uint32_t* spp) {
  return orc_render_timed(sc, out, spp, nullptr, nullptr);
}

extern "C" void* orc_prepare(const orc_scene* sc) {
#ifdef _OPENMP
  if (sc->threads > 0) omp_set_num_threads(sc->threads);
#endif
  Prepared* p = new Prepared();
  p->scene = *sc;
  p->st = build_setup(p->scene);
  p->st.s = &p->scene;
  return p;
}

extern "C" uint64_t orc_render_prepared(void* h, const orc_scene* cam, float* out,
                                        uint32_t* spp, double* march_s) {
  Prepared* p = static_cast<Prepared*>(h);
  orc_scene& s = p->scene;
  for (int a = 0; a < 3; ++a) {
    s.eye[a] = cam->eye[a];
    s.at[a] = cam->at[a];
    s.up[a] = cam->up[a];
  }
  s.fovy_deg = cam->fovy_deg;
  s.znear = cam->znear;
  s.zfar = cam->zfar;
  s.width = cam->width;
  s.height = cam->height;
  s.row_stride = cam->row_stride;
  s.row_phase = cam->row_phase;
  s.threads = cam->threads;
  s.use_double = cam->use_double;
  return march_all(p->st, out, spp, march_s);
}

extern "C" void orc_release(void* h) { delete static_cast<Prepared*>(h); }

// ---------------------------------------------------------------- GridLeaper
//
// One pass of GLGridLeaper-blend.glsl:65-228 / GLGridLeaper-iso.glsl:68-200 over
// a page table (GetBrick and friends, GLVolumePool.cpp:484-656), restated per
// pixel.  Bricks are addressed in their local texel coordinates (the pool
// texture coordinates of a slot, scaled by the pool size), so only the page
// table's states matter, not which slot holds a brick.

namespace {

struct LeaperBrick {
  const uint8_t* data;
  uint32_t n[3];
};

// texel-centre trilinear at local texel coordinates, clamp to the brick's edge;
// RGBA8 bricks (dtype 2): channel ch
float leaper_sample(const LeaperBrick& b, int dtype, float l0, float l1, float l2, float im,
                    int ch = 0) {
  const float u[3] = {std::fmin(std::fmax(l0 - 0.5f, 0.0f), float(b.n[0]) - 1.0f),
                      std::fmin(std::fmax(l1 - 0.5f, 0.0f), float(b.n[1]) - 1.0f),
                      std::fmin(std::fmax(l2 - 0.5f, 0.0f), float(b.n[2]) - 1.0f)};
  int i0[3], i1[3];
  float f[3];
  for (int a = 0; a < 3; ++a) {
    i0[a] = int(u[a]);
    f[a] = u[a] - float(i0[a]);
    i1[a] = std::min(i0[a] + 1, int(b.n[a]) - 1);
  }
  auto fetch = [&](int x, int y, int z) -> float {
    const size_t i = size_t(x) + size_t(y) * b.n[0] + size_t(z) * b.n[0] * b.n[1];
    if (dtype == 2) return float(b.data[4 * i + size_t(ch)]);
    return dtype == 0 ? float(b.data[i]) : float(reinterpret_cast<const uint16_t*>(b.data)[i]);
  };
  auto lerp = [](float a, float c, float w) { return std::fma(w, c - a, a); };
  const float c00 = lerp(fetch(i0[0], i0[1], i0[2]), fetch(i1[0], i0[1], i0[2]), f[0]);
  const float c10 = lerp(fetch(i0[0], i1[1], i0[2]), fetch(i1[0], i1[1], i0[2]), f[0]);
  const float c01 = lerp(fetch(i0[0], i0[1], i1[2]), fetch(i1[0], i0[1], i1[2]), f[0]);
  const float c11 = lerp(fetch(i0[0], i1[1], i1[2]), fetch(i1[0], i1[1], i1[2]), f[0]);
  const float c0 = lerp(c00, c10, f[1]);
  const float c1 = lerp(c01, c11, f[1]);
  return lerp(c0, c1, f[2]) * im;
}

inline float len3f(float x, float y, float z) { return std::sqrt((x * x + y * y) + z * z); }

// ComputeLOD's uint(log2(x)) (GLVolumePool.cpp:650-656) as the exact floor of
// the base-2 logarithm: the binary exponent of x for x >= 2, level 0 below 2
// and for a NaN, the coarsest level for an infinity.
inline uint32_t lod_level(float x, uint32_t max_lod) {
  if (!(x >= 2.0f)) return 0u;
  uint32_t bits;
  std::memcpy(&bits, &x, sizeof bits);
  return std::min(max_lod, ((bits >> 23) & 0xffu) - 127u);
}

}  // namespace

extern "C" uint64_t orc_leaper_render(const orc_scene* sc, const uint32_t* page, uint64_t n_page,
                                      float* out, uint32_t* spp, uint64_t* missing,
                                      uint64_t max_missing, uint64_t* n_missing) {
  const orc_scene& s = *sc;
  // RGBA8 colour volumes (dtype 2): 8 bits per channel, range [0, 255], no
  // gradient statistics (fGradientScale 1)
  const bool color = s.dtype == 2;
  const int bytes = color ? 4 : (s.dtype == 0 ? 1 : 2);
  const int cbits = color ? 8 : 8 * bytes;
  uint64_t lsz[3 * 64], lcnt[3 * 64];
  const int n_lods = orc_lod_table(s.dims, s.brick_size, s.overlap, lsz, lcnt, 64);
  std::vector<uint64_t> first(n_lods + 1, 0), shapes;
  uint64_t total_vox = 0;
  std::vector<std::array<uint32_t, 3>> nv;
  for (int l = 0; l < n_lods; ++l) {
    first[l + 1] = first[l] + lcnt[3 * l] * lcnt[3 * l + 1] * lcnt[3 * l + 2];
    for (uint64_t k = 0; k < first[l + 1] - first[l]; ++k) {
      const uint64_t c3[3] = {k % lcnt[3 * l], (k / lcnt[3 * l]) % lcnt[3 * l + 1],
                              k / (lcnt[3 * l] * lcnt[3 * l + 1])};
      uint64_t bs[3];
      orc_brick_size(&lsz[3 * l], &lcnt[3 * l], s.brick_size, s.overlap, c3, bs);
      nv.push_back({uint32_t(bs[0]), uint32_t(bs[1]), uint32_t(bs[2])});
      total_vox += bs[0] * bs[1] * bs[2];
    }
  }
  if (n_page < first[n_lods]) return 0;
  std::vector<uint8_t> pool(total_vox * bytes);
  std::vector<uint64_t> off(first[n_lods]);
  orc_build_octree(s.raw, s.dtype, s.dims, s.brick_size, s.overlap, s.clamp_to_edge, s.median,
                   pool.data(), total_vox, off.data(), first[n_lods]);
  // TF with the opacity correction of ocFactor = 1 / srm (host table, as the GPU)
  const size_t ntf = size_t(s.tf_w) * s.tf_h;
  std::vector<float> tf(4 * ntf, 0.0f);
  const float oc = 1.0f / s.sample_rate_modifier;
  for (size_t i = 0; i < ntf && s.render_mode != ORC_RM_ISO; ++i) {
    float e[4];
    for (int c = 0; c < 4; ++c) {
      e[c] = s.tf[4 * i + c];
      if (s.tf_rgba8) {
        const unsigned char b = (unsigned char)(std::max(0.0f, std::min(e[c], 1.0f)) * 255);
        e[c] = float(b) / 255.0f;
      }
    }
    tf[4 * i] = e[0];
    tf[4 * i + 1] = e[1];
    tf[4 * i + 2] = e[2];
    tf[4 * i + 3] = 1.0f - std::pow(1.0f - e[3], oc);
  }
  double rmax = color ? 255.0 : 0.0;
  for (uint64_t i = 0; !color && i < s.dims[0] * s.dims[1] * s.dims[2]; ++i)
    rmax = std::max(rmax, bytes == 1 ? double(static_cast<const uint8_t*>(s.raw)[i])
                                     : double(static_cast<const uint16_t*>(s.raw)[i]));
  const uint32_t imax = (1u << cbits) - 1;
  const float trans_scale = float(double(imax) / rmax);
  float grad_scale = 1.0f;
  if (s.render_mode == ORC_RM_2D && !color) {
    const float mg = float(orc_max_gradient(s.raw, s.dtype, s.dims, s.brick_size, s.overlap,
                                            s.clamp_to_edge));
    grad_scale = (mg == 0) ? 1.0f : 1.0f / mg;
  }
  const float im = bytes == 2 ? 1.0f / 65535.0f : 1.0f / 255.0f;
  const float iso_norm = float(double(s.isovalue) / double(1u << cbits));
  Setup st;  // the fields iso_compose reads
  st.s = &s;
  for (int a = 0; a < 3; ++a) {
    st.light_a[a] = s.ambient[a] * s.ambient[3];
    st.light_d[a] = s.diffuse[a] * s.diffuse[3];
    st.light_s[a] = s.specular[a] * s.specular[3];
    st.iso_diffuse[a] = st.light_d[a] * s.iso_color[a];
  }
  const View v = make_view(s);
  // layouts (GetFloatBrickLayout) and geometry
  float layout[64][3];
  for (int l = 0; l < n_lods; ++l)
    for (int a = 0; a < 3; ++a) {
      float c = float(s.dims[a]) / float(s.brick_size[a] - 2 * s.overlap);
      c /= float(uint64_t(1) << l);
      if (float(uint32_t(c)) == c) c -= c * std::numeric_limits<float>::epsilon();
      layout[l][a] = c;
    }
  const uint32_t max_lod = uint32_t(n_lods - 1);
  float ext[3], vol_size[3], max_inner[3];
  const float dmax = float(std::max(s.dims[0], std::max(s.dims[1], s.dims[2])));
  for (int a = 0; a < 3; ++a) {
    ext[a] = float(s.dims[a]) / dmax;
    vol_size[a] = float(s.dims[a]);
    max_inner[a] = float(s.brick_size[a] - 2 * s.overlap);
  }
  const float ghost = float(s.overlap);
  const float lod_factor =
      2.0f * std::tan(s.fovy_deg * ((3.1416f / 180.0f) / 2.0f)) * 1.0f / float(s.height);
  const float lod0_err = std::max(ext[0] / vol_size[0], std::max(ext[1] / vol_size[1], ext[2] / vol_size[2]));
  double e2n[3][4];
  float eye2norm[3][4], norm2eye[3][4], nte[3][3];
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) e2n[r][c] = v.inv[r][c] / double(ext[r]);
    e2n[r][3] += 0.5;
  }
  for (int r = 0; r < 3; ++r) {
    double acc = v.mv[r][3];
    for (int c = 0; c < 4; ++c) eye2norm[r][c] = float(e2n[r][c]);
    for (int c = 0; c < 3; ++c) {
      norm2eye[r][c] = float(v.mv[r][c] * double(ext[c]));
      acc -= v.mv[r][c] * double(ext[c]) * 0.5;
      nte[r][c] = float(v.mv[r][c]);
    }
    norm2eye[r][3] = float(acc);
  }
  double ld[3], em[3];
  for (int r = 0; r < 3; ++r) {
    ld[r] = e2n[r][0] * s.light_dir[0] + e2n[r][1] * s.light_dir[1] + e2n[r][2] * s.light_dir[2];
    em[r] = e2n[r][0] * s.eye[0] + e2n[r][1] * s.eye[1] + e2n[r][2] * s.eye[2] + e2n[r][3];
  }
  const double ll = std::sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2]);
  float Lm[3], Em[3];
  for (int a = 0; a < 3; ++a) {
    Lm[a] = float(ld[a] / ll);
    Em[a] = float(em[a]);
  }
  const float srm = s.sample_rate_modifier;
  const float W = float(s.tf_w), H = float(s.tf_h);
  const bool lit = s.lighting != 0, two_d = s.render_mode == ORC_RM_2D,
             iso = s.render_mode == ORC_RM_ISO;
  std::vector<char> wanted(first[n_lods], 0);
  uint64_t total = 0;
  // rows are independent (each writes its own pixels); the request set is the
  // union over all rows.  row_stride / row_phase restrict the pass to a sample
  // of rows, the rest are left untouched.
  const uint32_t stride = s.row_stride ? s.row_stride : 1;
#ifdef _OPENMP
  if (s.threads > 0) omp_set_num_threads(s.threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (int64_t py_ = 0; py_ < int64_t(s.height); ++py_) {
    const uint32_t py = uint32_t(py_);
    if (py % stride != s.row_phase % stride) continue;
    for (uint32_t px = 0; px < s.width; ++px) {
      const size_t pix = size_t(py) * s.width + px;
      float* o4 = out + 4 * pix;
      o4[0] = o4[1] = o4[2] = o4[3] = 0.0f;
      if (spp) spp[pix] = 0;
      const float nx = (float(px) + 0.5f) * v.inv_w2 - 1.0f;
      const float ny = (float(py) + 0.5f) * v.inv_h2 - 1.0f;
      const float de[3] = {nx * v.kx, ny * v.ky, -1.0f};
      float o[3], d[3];
      for (int a = 0; a < 3; ++a) {
        o[a] = eye2norm[a][3];
        d[a] = std::fma(eye2norm[a][2], de[2], std::fma(eye2norm[a][1], de[1], eye2norm[a][0] * de[0]));
      }
      float s0 = -INFINITY, s1 = INFINITY;
      for (int a = 0; a < 3; ++a) {
        const float inv = 1.0f / d[a];
        const float ta = (0.0f - o[a]) * inv, tb = (1.0f - o[a]) * inv;
        s0 = std::fmax(s0, std::fmin(ta, tb));
        s1 = std::fmin(s1, std::fmax(ta, tb));
      }
      const float s_in = std::fmax(s0, s.znear);
      if (!(s1 > s_in) || s1 > s.zfar) continue;
      float ent[3], exi[3];
      for (int a = 0; a < 3; ++a) {
        exi[a] = std::fma(s1, d[a], o[a]);
        ent[a] = std::fma(s_in, d[a], o[a]);
      }
      const float exit_depth = -s1, entry_depth = -s_in;
      const float dir[3] = {exi[0] - ent[0], exi[1] - ent[1], exi[2] - ent[2]};
      const float ray_len = len3f(dir[0], dir[1], dir[2]);
      float sv[3] = {dir[0] * vol_size[0], dir[1] * vol_size[1], dir[2] * vol_size[2]};
      {
        const float l = len3f(sv[0], sv[1], sv[2]);
        for (int a = 0; a < 3; ++a) sv[a] = (sv[a] / l) / (2.0f * srm);
      }
      const float step_len = len3f(sv[0], sv[1], sv[2]);
      const float voxel_eps = 0.125f / 2000.0f;
      float acc[4] = {0, 0, 0, 0};
      float cur[3] = {ent[0], ent[1], ent[2]};
      float t = 0.0f;
      uint32_t last[4] = {0, 0, 0, 9999};
      uint32_t samples = 0;
      float hitc[4] = {0, 0, 0, 0};
      auto info_at = [&](const float p[3], uint32_t lod, uint32_t bc[3]) {
        for (int a = 0; a < 3; ++a) bc[a] = uint32_t(p[a] * layout[lod][a]);
        const uint64_t id = first[lod] + bc[0] + bc[1] * lcnt[3 * lod] +
                            bc[2] * lcnt[3 * lod] * lcnt[3 * lod + 1];
        return std::make_pair(page[id], id);
      };
      if (ray_len > voxel_eps) {
        for (uint32_t j = 0; j < 100; ++j) {
          const float depth = entry_depth * (1.0f - t) + exit_depth * t;
          uint32_t lod = lod_level(lod_factor * (-depth) / lod0_err, max_lod);
          float p[3];
          for (int a = 0; a < 3; ++a) p[a] = std::fmin(std::fmax(cur[a], 0.0f), 1.0f);
          uint32_t bc[3];
          auto r = info_at(p, lod, bc);
          uint32_t info = r.first;
          uint64_t id = r.second;
          if (info == 0) {
#pragma omp atomic write
            wanted[id] = 1;
            while (info == 0 && lod < max_lod) {
              ++lod;
              r = info_at(p, lod, bc);
              info = r.first;
              id = r.second;
            }
            if (info == 0) info = 2;
          }
          const bool empty = info <= 2;
          if (empty) {
            for (uint32_t l = lod + 1; l < max_lod; ++l) {
              uint32_t lbc[3];
              const auto rr = info_at(p, l, lbc);
              if (rr.first != 1) break;
              bc[0] = lbc[0]; bc[1] = lbc[1]; bc[2] = lbc[2];
              info = rr.first;
              id = rr.second;
              lod = l;
            }
          }
          float c0[3], c1[3], bexit[3];
          float tmin = INFINITY;
          for (int a = 0; a < 3; ++a) {
            c0[a] = float(bc[a]) / layout[lod][a];
            c1[a] = float(bc[a] + 1u) / layout[lod][a];
            const float div = 1.0f / dir[a];
            const float corner = div >= 0.0f ? c1[a] : c0[a];
            tmin = std::fmin(tmin, (corner - p[a]) * div);
          }
          for (int a = 0; a < 3; ++a) bexit[a] = std::fma(tmin, dir[a], p[a]);
          const bool same = last[0] == bc[0] && last[1] == bc[1] && last[2] == bc[2] && last[3] == lod;
          bool done = false;
          if (!empty && !same) {
            LeaperBrick b;
            b.data = pool.data() + off[id] * bytes;
            b.n[0] = nv[id][0]; b.n[1] = nv[id][1]; b.n[2] = nv[id][2];
            float sc[3], tr[3], pc[3], pe[3], pxx[3];
            for (int a = 0; a < 3; ++a) {
              sc[a] = max_inner[a] * layout[lod][a];
              tr[a] = ghost - c0[a] * sc[a];
              pe[a] = std::fma(p[a], sc[a], tr[a]);
              pxx[a] = std::fma(bexit[a], sc[a], tr[a]);
              pc[a] = pe[a];
            }
            int steps = int(std::ceil(len3f(pxx[0] - pe[0], pxx[1] - pe[1], pxx[2] - pe[2]) / step_len));
            steps = std::min(steps, int(std::ceil(len3f((exi[0] - cur[0]) * sc[0], (exi[1] - cur[1]) * sc[1],
                                                        (exi[2] - cur[2]) * sc[2]) / step_len)));
            auto smp = [&](float a0, float a1, float a2) { return leaper_sample(b, s.dtype, a0, a1, a2, im); };
            auto chan = [&](int ch, float a0, float a1, float a2) {
              return leaper_sample(b, s.dtype, a0, a1, a2, im, ch);
            };
            // lighting.glsl:33-43 with the model-space eye; tfc = diffuse colour
            auto light = [&](const float N[3], const float mp[3], float src[4]) {
              const float q0 = Em[0] - mp[0], q1 = Em[1] - mp[1], q2 = Em[2] - mp[2];
              const float lq = len3f(q0, q1, q2);
              const float V0 = q0 / lq, V1 = q1 / lq, V2 = q2 / lq;
              const float dd = (N[0] * V0 + N[1] * V1) + N[2] * V2;
              float R0 = V0 - (2.0f * dd) * N[0], R1 = V1 - (2.0f * dd) * N[1],
                    R2 = V2 - (2.0f * dd) * N[2];
              const float lr = len3f(R0, R1, R2);
              R0 = R0 / lr; R1 = R1 / lr; R2 = R2 / lr;
              const float diff = std::fmax(std::fabs((N[0] * Lm[0] + N[1] * Lm[1]) + N[2] * Lm[2]), 0.0f);
              const float spec = pow_int_or_real(std::fmax((R0 * Lm[0] + R1 * Lm[1]) + R2 * Lm[2], 0.0f), 8.0f);
              for (int c = 0; c < 3; ++c) {
                const float dcol = st.light_d[c] * src[c];
                float x = st.light_a[c] + dcol * diff;
                x = x + st.light_s[c] * spec;
                src[c] = std::fmin(std::fmax(x, 0.0f), 1.0f);
              }
            };
            for (int i = 0; i < steps; ++i) {
              ++samples;
              if (color) {
                // GLGridLeaper-Method-*-color.glsl: the filtered RGBA
                const float cd[4] = {chan(0, pc[0], pc[1], pc[2]), chan(1, pc[0], pc[1], pc[2]),
                                     chan(2, pc[0], pc[1], pc[2]), chan(3, pc[0], pc[1], pc[2])};
                if (iso) {
                  // GLGridLeaper-Method-iso-color.glsl: alpha >= fIsoval, bisection on
                  // alpha, ComputeAlphaNormal = the red channel's gradient
                  if (cd[3] >= iso_norm) {
                    float rr2[3] = {sv[0] / 2.0f, sv[1] / 2.0f, sv[2] / 2.0f};
                    float q[3] = {pc[0] - rr2[0], pc[1] - rr2[1], pc[2] - rr2[2]};
                    for (int k = 0; k < 5; ++k) {
                      for (int a = 0; a < 3; ++a) rr2[a] = rr2[a] / 2.0f;
                      const float vv = chan(3, q[0], q[1], q[2]);
                      for (int a = 0; a < 3; ++a) q[a] = vv >= iso_norm ? q[a] - rr2[a] : q[a] + rr2[a];
                    }
                    float g[3] = {(chan(0, q[0] - 1.0f, q[1], q[2]) - chan(0, q[0] + 1.0f, q[1], q[2])) / 2.0f,
                                  (chan(0, q[0], q[1] - 1.0f, q[2]) - chan(0, q[0], q[1] + 1.0f, q[2])) / 2.0f,
                                  (chan(0, q[0], q[1], q[2] - 1.0f) - chan(0, q[0], q[1], q[2] + 1.0f)) / 2.0f};
                    const float gl = len3f(g[0], g[1], g[2]);
                    if (gl > 0.0f) { g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl; }
                    float hp[3], he[3], hn[3];
                    for (int a = 0; a < 3; ++a) hp[a] = (q[a] - tr[a]) / sc[a];
                    for (int r2 = 0; r2 < 3; ++r2) {
                      he[r2] = std::fma(norm2eye[r2][0], hp[0],
                                        std::fma(norm2eye[r2][1], hp[1],
                                                 std::fma(norm2eye[r2][2], hp[2], norm2eye[r2][3])));
                      hn[r2] = std::fma(nte[r2][2], g[2], std::fma(nte[r2][1], g[1], nte[r2][0] * g[0]));
                    }
                    // GLGridLeaper-iso.glsl:169-171 packing, Compose-Color-FS unpacking
                    const float enc_r = cd[0] + 1.0f;
                    const float enc_gb = std::floor(cd[1] * 512.0f) + cd[2];
                    const float rgb[3] = {enc_r - 1.0f, std::floor(enc_gb / 2.0f) / 256.0f,
                                          enc_gb - std::floor(enc_gb)};
                    float dcol[3], c3[3];
                    for (int a = 0; a < 3; ++a) dcol[a] = rgb[a] * st.light_d[a];
                    surface_lighting<float>(st, he, hn, dcol, c3);
                    hitc[0] = c3[0]; hitc[1] = c3[1]; hitc[2] = c3[2]; hitc[3] = 1.0f;
                    done = true;
                    break;
                  }
                } else {
                  const float u = cd[3] * trans_scale;
                  float fx = std::floor(u * W);
                  fx = std::fmin(std::fmax(fx, 0.0f), W - 1.0f);
                  float al = 0.0f, g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, mag = 0.0f;
                  if (two_d) {
                    bool col_any = false;
                    for (uint32_t y = 0; y < s.tf_h; ++y)
                      if (tf[4 * (size_t(y) * s.tf_w + size_t(fx)) + 3] != 0.0f) col_any = true;
                    if (col_any) {
                      // ComputeGradientAlpha
                      g0 = (chan(3, pc[0] - 1.0f, pc[1], pc[2]) - chan(3, pc[0] + 1.0f, pc[1], pc[2])) / 2.0f;
                      g1 = (chan(3, pc[0], pc[1] - 1.0f, pc[2]) - chan(3, pc[0], pc[1] + 1.0f, pc[2])) / 2.0f;
                      g2 = (chan(3, pc[0], pc[1], pc[2] - 1.0f) - chan(3, pc[0], pc[1], pc[2] + 1.0f)) / 2.0f;
                      mag = len3f(g0, g1, g2);
                      const float w = 1.0f - mag * grad_scale;
                      float fy = std::floor(w * H);
                      fy = std::fmin(std::fmax(fy, 0.0f), H - 1.0f);
                      al = tf[4 * (size_t(fy) * s.tf_w + size_t(fx)) + 3];
                    }
                  } else {
                    al = tf[4 * size_t(fx) + 3];
                  }
                  float src[4] = {cd[0], cd[1], cd[2], al};
                  if (lit && al != 0.0f) {
                    float N[3];
                    if (two_d) {
                      N[0] = mag > 0.0f ? g0 / mag : g0;
                      N[1] = mag > 0.0f ? g1 / mag : g1;
                      N[2] = mag > 0.0f ? g2 / mag : g2;
                    } else {  // ComputeNormal on the red channel
                      N[0] = (chan(0, pc[0] - 1.0f, pc[1], pc[2]) - chan(0, pc[0] + 1.0f, pc[1], pc[2])) / 2.0f;
                      N[1] = (chan(0, pc[0], pc[1] - 1.0f, pc[2]) - chan(0, pc[0], pc[1] + 1.0f, pc[2])) / 2.0f;
                      N[2] = (chan(0, pc[0], pc[1], pc[2] - 1.0f) - chan(0, pc[0], pc[1], pc[2] + 1.0f)) / 2.0f;
                      const float l = len3f(N[0], N[1], N[2]);
                      if (l > 0.0f) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
                    }
                    float mp[3];
                    for (int a = 0; a < 3; ++a) mp[a] = (pc[a] - tr[a]) / sc[a];
                    light(N, mp, src);
                  }
                  const float w = 1.0f - acc[3];
                  acc[0] = std::fma(src[0] * w, src[3], acc[0]);
                  acc[1] = std::fma(src[1] * w, src[3], acc[1]);
                  acc[2] = std::fma(src[2] * w, src[3], acc[2]);
                  acc[3] = std::fma(src[3], w, acc[3]);
                  if (acc[3] > 0.99f) { done = true; break; }
                }
                for (int a = 0; a < 3; ++a) pc[a] = pc[a] + sv[a];
                continue;
              }
              const float val = smp(pc[0], pc[1], pc[2]);
              if (iso) {
                if (val >= iso_norm) {
                  float rr2[3] = {sv[0] / 2.0f, sv[1] / 2.0f, sv[2] / 2.0f};
                  float q[3] = {pc[0] - rr2[0], pc[1] - rr2[1], pc[2] - rr2[2]};
                  for (int k = 0; k < 5; ++k) {
                    for (int a = 0; a < 3; ++a) rr2[a] = rr2[a] / 2.0f;
                    const float vv = smp(q[0], q[1], q[2]);
                    for (int a = 0; a < 3; ++a) q[a] = vv >= iso_norm ? q[a] - rr2[a] : q[a] + rr2[a];
                  }
                  const float xp = smp(q[0] + 1.0f, q[1], q[2]), xm = smp(q[0] - 1.0f, q[1], q[2]);
                  const float yp = smp(q[0], q[1] - 1.0f, q[2]), ym = smp(q[0], q[1] + 1.0f, q[2]);
                  const float zp = smp(q[0], q[1], q[2] + 1.0f), zm = smp(q[0], q[1], q[2] - 1.0f);
                  float g[3] = {(xm - xp) / 2.0f, (yp - ym) / 2.0f, (zm - zp) / 2.0f};
                  const float gl = len3f(g[0], g[1], g[2]);
                  if (gl > 0.0f) { g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl; }
                  float hp[3], he[3], hn[3];
                  for (int a = 0; a < 3; ++a) hp[a] = (q[a] - tr[a]) / sc[a];
                  for (int r2 = 0; r2 < 3; ++r2) {
                    he[r2] = std::fma(norm2eye[r2][0], hp[0],
                                      std::fma(norm2eye[r2][1], hp[1],
                                               std::fma(norm2eye[r2][2], hp[2], norm2eye[r2][3])));
                    hn[r2] = std::fma(nte[r2][2], g[2], std::fma(nte[r2][1], g[1], nte[r2][0] * g[0]));
                  }
                  float c3[3];
                  iso_compose<float>(st, he, hn, c3);
                  hitc[0] = c3[0]; hitc[1] = c3[1]; hitc[2] = c3[2]; hitc[3] = 1.0f;
                  done = true;
                  break;
                }
              } else {
                float src[4];
                const float u = val * trans_scale;
                float fx = std::floor(u * W);
                fx = std::fmin(std::fmax(fx, 0.0f), W - 1.0f);
                float g0 = 0, g1 = 0, g2 = 0;
                bool need = lit;
                bool col_any = true;
                if (two_d) {
                  col_any = false;
                  for (uint32_t y = 0; y < s.tf_h; ++y)
                    if (tf[4 * (size_t(y) * s.tf_w + size_t(fx)) + 3] != 0.0f) col_any = true;
                  need = col_any;
                } else {
                  for (int c = 0; c < 4; ++c) src[c] = tf[4 * size_t(fx) + c];
                  need = lit && src[3] != 0.0f;
                }
                if (need) {
                  const float xp = smp(pc[0] + 1.0f, pc[1], pc[2]), xm = smp(pc[0] - 1.0f, pc[1], pc[2]);
                  const float yp = smp(pc[0], pc[1] - 1.0f, pc[2]), ym = smp(pc[0], pc[1] + 1.0f, pc[2]);
                  const float zp = smp(pc[0], pc[1], pc[2] + 1.0f), zm = smp(pc[0], pc[1], pc[2] - 1.0f);
                  g0 = (xm - xp) / 2.0f;
                  g1 = (yp - ym) / 2.0f;
                  g2 = (zm - zp) / 2.0f;
                }
                float mag = 0.0f;
                if (two_d) {
                  if (need) {
                    mag = len3f(g0, g1, g2);
                    const float w = 1.0f - mag * grad_scale;
                    float fy = std::floor(w * H);
                    fy = std::fmin(std::fmax(fy, 0.0f), H - 1.0f);
                    for (int c = 0; c < 4; ++c) src[c] = tf[4 * (size_t(fy) * s.tf_w + size_t(fx)) + c];
                  } else {
                    src[0] = src[1] = src[2] = src[3] = 0.0f;
                  }
                  need = need && lit && src[3] != 0.0f;
                }
                if (lit && need) {
                  float N[3];
                  if (two_d) {
                    N[0] = mag > 0.0f ? g0 / mag : g0;
                    N[1] = mag > 0.0f ? g1 / mag : g1;
                    N[2] = mag > 0.0f ? g2 / mag : g2;
                  } else {
                    N[0] = g0; N[1] = g1; N[2] = g2;
                    const float l = len3f(N[0], N[1], N[2]);
                    if (l > 0.0f) { N[0] = N[0] / l; N[1] = N[1] / l; N[2] = N[2] / l; }
                  }
                  float mp[3];
                  for (int a = 0; a < 3; ++a) mp[a] = (pc[a] - tr[a]) / sc[a];
                  // lighting.glsl:33-43 with the model-space eye
                  const float q0 = Em[0] - mp[0], q1 = Em[1] - mp[1], q2 = Em[2] - mp[2];
                  const float lq = len3f(q0, q1, q2);
                  const float V0 = q0 / lq, V1 = q1 / lq, V2 = q2 / lq;
                  const float dd = (N[0] * V0 + N[1] * V1) + N[2] * V2;
                  float R0 = V0 - (2.0f * dd) * N[0], R1 = V1 - (2.0f * dd) * N[1],
                        R2 = V2 - (2.0f * dd) * N[2];
                  const float lr = len3f(R0, R1, R2);
                  R0 = R0 / lr; R1 = R1 / lr; R2 = R2 / lr;
                  const float diff = std::fmax(std::fabs((N[0] * Lm[0] + N[1] * Lm[1]) + N[2] * Lm[2]), 0.0f);
                  const float spec = pow_int_or_real(std::fmax((R0 * Lm[0] + R1 * Lm[1]) + R2 * Lm[2], 0.0f), 8.0f);
                  for (int c = 0; c < 3; ++c) {
                    const float dcol = st.light_d[c] * src[c];
                    float x = st.light_a[c] + dcol * diff;
                    x = x + st.light_s[c] * spec;
                    src[c] = std::fmin(std::fmax(x, 0.0f), 1.0f);
                  }
                }
                const float w = 1.0f - acc[3];
                acc[0] = std::fma(src[0] * w, src[3], acc[0]);
                acc[1] = std::fma(src[1] * w, src[3], acc[1]);
                acc[2] = std::fma(src[2] * w, src[3], acc[2]);
                acc[3] = std::fma(src[3], w, acc[3]);
                if (acc[3] > 0.99f) { done = true; break; }
              }
              for (int a = 0; a < 3; ++a) pc[a] = pc[a] + sv[a];
            }
            if (done) break;
            for (int a = 0; a < 3; ++a) cur[a] = (pc[a] - tr[a]) / sc[a];
          } else {
            for (int a = 0; a < 3; ++a) cur[a] = std::fma(voxel_eps, dir[a] / ray_len, bexit[a]);
          }
          last[0] = bc[0]; last[1] = bc[1]; last[2] = bc[2]; last[3] = lod;
          t = len3f(ent[0] - bexit[0], ent[1] - bexit[1], ent[2] - bexit[2]) / ray_len;
          if (t > 0.9999f) break;
        }
      }
      const float* res = iso ? hitc : acc;
      for (int c = 0; c < 4; ++c) o4[c] = res[c];
      if (spp) spp[pix] = samples;
      total += samples;
    }
  }
  uint64_t nm = 0;
  for (uint64_t i = 0; i < first[n_lods]; ++i)
    if (wanted[i]) {
      if (nm < max_missing && missing) missing[nm] = i;
      ++nm;
    }
  if (n_missing) *n_missing = nm;
  return total;
}

extern "C" void orc_render_size(const orc_scene* sc, uint32_t* w, uint32_t* h) {
  render_size(*sc, w, h);
}
