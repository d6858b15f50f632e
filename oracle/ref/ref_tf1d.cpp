// ref_tf1d.cpp -- C entry points around the reference's own TransferFunction1D
// (IO/TransferFunction1D.cpp), compiled from the reference sources by
// oracle/ref/Makefile into oracle/_ref/libtuvok_ref.so.
//
// TEST INFRASTRUCTURE ONLY: pins tuvok_gb300's tvk_tf1d_* table functions
// (and the golden vectors tests/golden/tf1d/make_tf1d_golden.py writes) to the
// reference's methods on the same inputs.
#include <cstdint>
#include <cstring>
#include <vector>

#include "IO/TransferFunction1D.h"

namespace {

void put(TransferFunction1D& tf, const float* rgba, uint64_t n) {
  tf.Resize(n);
  for (uint64_t i = 0; i < n; ++i)
    tf.SetColor(i, FLOATVECTOR4(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]));
}

void get(const TransferFunction1D& tf, float* out) {
  for (size_t i = 0; i < tf.GetSize(); ++i) {
    const FLOATVECTOR4 c = tf.GetColor(i);
    out[4 * i] = c.x;
    out[4 * i + 1] = c.y;
    out[4 * i + 2] = c.z;
    out[4 * i + 3] = c.w;
  }
}

void limits(TransferFunction1D& tf, uint64_t lim[2]) {
  const UINT64VECTOR2& l = tf.GetNonZeroLimits();
  lim[0] = l.x;
  lim[1] = l.y;
}

}  // namespace

extern "C" {

// SetStdFunction on the table `in` (component -1: the 2-argument overload)
void ref_tf1d_std(const float* in, uint64_t n, float center, float inv_gradient, int component,
                  int inverted, float* out, uint64_t lim[2]) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  if (component < 0)
    tf.SetStdFunction(center, inv_gradient);
  else
    tf.SetStdFunction(center, inv_gradient, component, inverted != 0);
  get(tf, out);
  limits(tf, lim);
}

void ref_tf1d_set(const uint8_t* bytes, uint64_t n, float* out, uint64_t lim[2]) {
  TransferFunction1D tf(0);
  tf.Set(std::vector<unsigned char>(bytes, bytes + 4 * n));
  get(tf, out);
  limits(tf, lim);
}

void ref_tf1d_resample(const float* in, uint64_t n, uint64_t target, float* out,
                       uint64_t lim[2]) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  tf.Resample(target);
  get(tf, out);
  limits(tf, lim);
}

void ref_tf1d_fill_or_truncate(const float* in, uint64_t n, uint64_t target, float* out) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  tf.FillOrTruncate(target);
  get(tf, out);
}

void ref_tf1d_limits(const float* in, uint64_t n, uint64_t lim[2]) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  tf.ComputeNonZeroLimits();
  limits(tf, lim);
}

void ref_tf1d_bytes(const float* in, uint64_t n, uint8_t used_range, uint8_t* out) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  std::vector<unsigned char> v;
  tf.GetByteArray(v, used_range);
  std::memcpy(out, v.data(), v.size());
}

int ref_tf1d_save(const float* in, uint64_t n, const char* path) {
  TransferFunction1D tf(0);
  put(tf, in, n);
  return tf.Save(std::string(path)) ? 1 : 0;
}

// returns 1 and the table (up to cap entries) when Load succeeds
int ref_tf1d_load(const char* path, float* out, uint64_t cap, uint64_t* n) {
  TransferFunction1D tf(0);
  if (!tf.Load(std::string(path))) return 0;
  *n = tf.GetSize();
  if (tf.GetSize() <= cap) get(tf, out);
  return 1;
}

}  // extern "C"
