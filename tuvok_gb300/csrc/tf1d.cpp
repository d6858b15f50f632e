// tf1d.cpp -- TransferFunction1D (IO/TransferFunction1D.h:53-101) as a caller-held
// table of n RGBA float entries: SetStdFunction, Set (bytes), Resample,
// FillOrTruncate, Clear, ComputeNonZeroLimits, GetByteArray / GetShortArray,
// Load / Save of the text format.  Host code only; the renderer takes the
// table through tvk_set_tf1d_float (or the bytes through tvk_set_tf1d_rgba8).
//
// Every expression keeps the reference's float evaluation order and this file
// is built with -ffp-contract=off, so tables are the reference's bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tvk_internal.h"

namespace tvk {

namespace {

// TransferFunction1D::Smoothstep (TransferFunction1D.cpp:70-72): 3x^2 - 2x^3
// evaluated left to right, unfused.
inline float smoothstep_ref(float x) {
  const float a = (3.0f * x) * x;
  const float b = ((2.0f * x) * x) * x;
  return a - b;
}

}  // namespace

// TransferFunction1D::SetStdFunction (TransferFunction1D.cpp:81-113) on one
// component: zero (one, inverted) up to the ramp, a smoothstep ramp of width
// inv_gradient * (n - 1) entries centred on center * (n - 1), one (zero) after.
void tf1d_std_function(float* rgba, uint64_t n, float center, float inv_gradient, int comp,
                       bool inverted) {
  const float cc = std::min(std::max(0.0f, center), 1.0f);
  const float cg = std::min(std::max(0.0f, inv_gradient), 1.0f);
  const uint64_t ic = uint64_t(float(n - 1) * cc);
  const uint64_t ig = uint64_t(float(n - 1) * cg);
  const uint64_t half = ig / 2;
  const uint64_t start = half > ic ? 0 : ic - half;
  const uint64_t end = half + ic > n ? n : ic + half;
  for (uint64_t i = 0; i < start && i < n; ++i) rgba[4 * i + comp] = inverted ? 1.0f : 0.0f;
  for (uint64_t i = start; i < end; ++i) {
    // i - ic + half in unsigned (wrapping) arithmetic, as size_t in the reference
    const float v = smoothstep_ref(float(i - ic + half) / float(ig));
    rgba[4 * i + comp] = inverted ? 1.0f - v : v;
  }
  for (uint64_t i = end; i < n; ++i) rgba[4 * i + comp] = inverted ? 0.0f : 1.0f;
}

// TransferFunction1D::Set (TransferFunction1D.cpp:146-177) with the
// minmax_component4 helper (:115-144): every channel's minimum and maximum
// start from the first byte of the table (entry 0's red), then take each
// entry's own channel; colour channels are lerped from [min, max] onto [0, 1]
// by MathTools::lerp (Basics/MathTools.h:81-84, in double), alpha from
// [0, 255].  A constant channel divides by zero (NaN, or +-inf where the
// byte differs from the start value).
void tf1d_from_bytes(const uint8_t* bytes, uint64_t n, float* rgba) {
  uint8_t mn[4], mx[4];
  for (int c = 0; c < 4; ++c) mn[c] = mx[c] = bytes[0];
  for (uint64_t i = 0; i < n; ++i)
    for (int c = 0; c < 4; ++c) {
      const uint8_t v = bytes[4 * i + c];
      if (v < mn[c]) mn[c] = v;
      if (v > mx[c]) mx[c] = v;
    }
  auto lerp = [](int value, int imin, int imax) {
    const double q = double(1.0f - 0.0f) / double(imax - imin);
    return float(0.0f + double(value - imin) * q);
  };
  for (uint64_t i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) rgba[4 * i + c] = lerp(bytes[4 * i + c], mn[c], mx[c]);
    rgba[4 * i + 3] = lerp(bytes[4 * i + 3], 0, 255);
  }
}

// TransferFunction1D::Resample (TransferFunction1D.cpp:198-238).  Down: entry
// i averages the next floor(remaining source / remaining target) source
// entries (float sums in order, divided by the count).  Up: linear
// interpolation at position i * (n_src - 1) / n_dst.
void tf1d_resample(const float* src, uint64_t n_src, float* dst, uint64_t n_dst) {
  if (n_dst == n_src) {
    std::memmove(dst, src, sizeof(float) * 4 * n_src);
    return;
  }
  std::vector<float> out(4 * n_dst);
  if (n_dst < n_src) {
    uint64_t from = 0, tgt = n_dst, srcn = n_src;
    for (uint64_t i = 0; i < n_dst; ++i) {
      const uint64_t to = from + srcn / tgt;
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (uint64_t j = from; j < to; ++j)
        for (int c = 0; c < 4; ++c) acc[c] += src[4 * j + c];
      const float cnt = float(to - from);
      for (int c = 0; c < 4; ++c) out[4 * i + c] = acc[c] / cnt;
      tgt -= 1;
      srcn -= to - from;
      from = to;
    }
  } else {
    for (uint64_t i = 0; i < n_dst; ++i) {
      const float pos = (float(i) * float(n_src - 1)) / float(n_dst);
      const uint64_t lo = uint64_t(std::floor(pos));
      const uint64_t hi = std::min(lo + 1, n_src - 1);
      const float w = pos - float(lo);
      for (int c = 0; c < 4; ++c) {
        const float a = src[4 * lo + c] * (1.0f - w);
        const float b = src[4 * hi + c] * w;
        out[4 * i + c] = a + b;
      }
    }
  }
  std::memcpy(dst, out.data(), sizeof(float) * out.size());
}

// TransferFunction1D::ComputeNonZeroLimits (TransferFunction1D.cpp:362-371):
// [first, last] entry with a non-zero alpha; (n, 0) when there is none.
void tf1d_nonzero_limits(const float* rgba, uint64_t n, uint64_t lim[2]) {
  lim[0] = n;
  lim[1] = 0;
  for (uint64_t i = 0; i < n; ++i)
    if (rgba[4 * i + 3] != 0.0f) {
      lim[0] = std::min(lim[0], i);
      lim[1] = i;
    }
}

}  // namespace tvk

namespace {

template <class F>
tvk_status tf_guarded(F&& f) {
  try {
    f();
    tvk::set_last_error("");
    return TVK_OK;
  } catch (const tvk::Error& e) {
    tvk::set_last_error(e.msg);
    return e.status;
  } catch (const std::bad_alloc&) {
    tvk::set_last_error("host allocation failed");
    return TVK_ERR_OUT_OF_MEMORY;
  } catch (...) {
    tvk::set_last_error("unknown failure");
    return TVK_ERR_INTERNAL;
  }
}

void require(bool ok, const char* msg) {
  if (!ok) tvk::fail(TVK_ERR_INVALID_ARG, msg);
}

}  // namespace

extern "C" {

tvk_status tvk_tf1d_set_std_function(float* rgba, uint64_t n, float center, float inv_gradient,
                                     int component, int inverted) {
  return tf_guarded([&] {
    require(rgba && n >= 1, "need a table of at least one entry");
    require(component >= -1 && component <= 3, "component must be 0..3, or -1 for all four");
    if (component < 0) {
      for (int c = 0; c < 4; ++c) tvk::tf1d_std_function(rgba, n, center, inv_gradient, c, false);
    } else {
      tvk::tf1d_std_function(rgba, n, center, inv_gradient, component, inverted != 0);
    }
  });
}

tvk_status tvk_tf1d_from_bytes(const uint8_t* rgba8, uint64_t n, float* rgba) {
  return tf_guarded([&] {
    require(rgba8 && rgba && n >= 1, "need byte and float tables of at least one entry");
    tvk::tf1d_from_bytes(rgba8, n, rgba);
  });
}

tvk_status tvk_tf1d_resample(const float* src, uint64_t n_src, float* dst, uint64_t n_dst) {
  return tf_guarded([&] {
    require(src && dst && n_src >= 1 && n_dst >= 1, "need two tables of at least one entry");
    tvk::tf1d_resample(src, n_src, dst, n_dst);
  });
}

tvk_status tvk_tf1d_fill_or_truncate(const float* src, uint64_t n_src, float* dst,
                                     uint64_t n_dst) {
  return tf_guarded([&] {
    require((src || n_src == 0) && (dst || n_dst == 0), "null table");
    // FillOrTruncate (TransferFunction1D.cpp:188-197): keep the first entries,
    // zero the rest
    std::vector<float> out(4 * n_dst, 0.0f);
    if (std::min(n_src, n_dst) > 0)
      std::memcpy(out.data(), src, sizeof(float) * 4 * std::min(n_src, n_dst));
    if (n_dst) std::memcpy(dst, out.data(), sizeof(float) * out.size());
  });
}

tvk_status tvk_tf1d_nonzero_limits(const float* rgba, uint64_t n, uint64_t limits[2]) {
  return tf_guarded([&] {
    require((rgba || n == 0) && limits, "null table or output");
    tvk::tf1d_nonzero_limits(rgba, n, limits);
  });
}

tvk_status tvk_tf1d_byte_array(const float* rgba, uint64_t n, uint8_t used_range, uint8_t* out) {
  return tf_guarded([&] {
    require((rgba && out) || n == 0, "null table or output");
    // GetByteArray (TransferFunction1D.cpp:311-330): clamp to [0, 1], scale, truncate
    for (uint64_t i = 0; i < 4 * n; ++i)
      out[i] = static_cast<uint8_t>(std::max(0.0f, std::min(rgba[i], 1.0f)) * float(used_range));
  });
}

tvk_status tvk_tf1d_short_array(const float* rgba, uint64_t n, uint16_t used_range,
                                uint16_t* out) {
  return tf_guarded([&] {
    require((rgba && out) || n == 0, "null table or output");
    // GetShortArray (TransferFunction1D.cpp:332-351)
    for (uint64_t i = 0; i < 4 * n; ++i)
      out[i] = static_cast<uint16_t>(std::max(0.0f, std::min(rgba[i], 1.0f)) * float(used_range));
  });
}

tvk_status tvk_tf1d_load(const char* path, float* rgba, uint64_t capacity, uint64_t* n_out) {
  return tf_guarded([&] {
    require(path && n_out, "need a path and an entry count output");
    // Load(istream) (TransferFunction1D.cpp:274-292): the entry count, then 4
    // floats per entry; the stream must still be good after the last one
    std::ifstream f(path);
    if (!f) tvk::fail(TVK_ERR_INVALID_ARG, std::string("cannot open ") + path);
    uint32_t size = 0;
    f >> size;
    if (!f) tvk::fail(TVK_ERR_INVALID_ARG, "transfer function size information invalid");
    *n_out = size;
    if (!rgba) return;  // size query
    require(capacity >= size, "table capacity below the file's entry count");
    std::vector<float> t(size_t(4) * size, 0.0f);
    for (size_t i = 0; i < t.size(); ++i) f >> t[i];
    if (!f.good()) tvk::fail(TVK_ERR_INVALID_ARG, "transfer function entries invalid or truncated");
    std::memcpy(rgba, t.data(), sizeof(float) * t.size());
  });
}

tvk_status tvk_tf1d_save(const char* path, const float* rgba, uint64_t n) {
  return tf_guarded([&] {
    require(path && (rgba || n == 0), "need a path and a table");
    // Save(ostream) (TransferFunction1D.cpp:294-306)
    std::ofstream f(path);
    if (!f) tvk::fail(TVK_ERR_INVALID_ARG, std::string("cannot write ") + path);
    f << n << std::endl;
    for (uint64_t i = 0; i < n; ++i) {
      for (int c = 0; c < 4; ++c) f << rgba[4 * i + c] << " ";
      f << std::endl;
    }
    if (!f) tvk::fail(TVK_ERR_INVALID_ARG, std::string("write failed: ") + path);
  });
}

}  // extern "C"
