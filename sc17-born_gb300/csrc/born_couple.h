// The Born coupling of cpuProp::imageAdd (base/cpu_prop.cc:216-223),
//   recField[i] += .000001 * srcField[i] * img[i];
// with float fields and a double literal: the reference forms
// W = (double)r + ((1e-6 * (double)s) * (double)m) in double, each operation
// rounded to nearest, and stores (float)W.  couple_exact returns that float
// bit for bit, computing in float arithmetic with a double fallback for the
// few cells where float arithmetic cannot decide the rounding.
//
// Method (error-free transformations, Dekker's product and Knuth's sum):
// 1e-6 as a double is exactly kCHi + kCLo (two floats).  With
//   u = kCHi s = uh + ue exactly (fma), ul = kCLo s + ue (rounded),
//   v = uh m  = vh + ve exactly,     vl = ul m + ve (rounded),
//   r + vh = t + e exactly (TwoSum),  yl = e + vl (rounded),
// y = t + yl approximates W with |y - W| < delta = 2^-44 (|vh| + |t|) when
// |uh|, |vh| >= 2^-100 (no underflow in the exact products).  R = fl(y) and
// d = (t - R) + yl = y - R (t - R exact by Sterbenz while |yl| <= |t|/4).
// If |d| + delta stays inside half the float spacing around R, W lies
// strictly inside R's rounding interval, so (float)W = R.  An exact zero s
// or m makes the product a signed zero, and r + (+-0) rounds alike in
// float and double; a product far below half an ulp of r gives r itself;
// every other cell takes the reference's expression in double.  The host
// instance is compiled without
// fused multiply-adds (-ffp-contract=off) and checked against the double
// expression on random and near-tie inputs; the device instance uses the
// same operations with explicit rounding intrinsics, which are never
// contracted.
#pragma once

#include <cstring>

#if defined(__CUDACC__)
#define BORN_HD __host__ __device__ __forceinline__
#else
#define BORN_HD inline
#endif

namespace born {
namespace couple {

BORN_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
BORN_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
BORN_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
BORN_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}
BORN_HD float fabs_(float a) {
#ifdef __CUDA_ARCH__
  return fabsf(a);
#else
  return __builtin_fabsf(a);
#endif
}
BORN_HD unsigned int bits(float a) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(a);
#else
  unsigned int u;
  std::memcpy(&u, &a, 4);
  return u;
#endif
}
BORN_HD float from_bits(unsigned int u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float a;
  std::memcpy(&a, &u, 4);
  return a;
#endif
}

// the reference's expression, operation by operation in double
BORN_HD float reference_double(float r, float s, float m) {
#ifdef __CUDA_ARCH__
  return __double2float_rn(
      __dadd_rn((double)r, __dmul_rn(__dmul_rn(1e-6, (double)s), (double)m)));
#else
  return (float)((double)r + 1e-6 * (double)s * (double)m);
#endif
}

// 1e-6 (double) = kCHi + kCLo exactly
constexpr float kCHi = 0x1.0c6f7ap-20f;
constexpr float kCLo = 0x1.6bdb1ap-49f;

// (float)((double)r + 1e-6 * (double)s * (double)m); *fell_back (when not
// null) reports whether the double expression was needed
BORN_HD float couple_exact(float r, float s, float m, bool *fell_back) {
  if (fell_back) *fell_back = false;
  if (s == 0.f || m == 0.f)  // the product is a signed zero in both forms
    return fadd(r, fmul(fmul(kCHi, s), m));
  const float uh = fmul(kCHi, s);
  const float ue = ffma(kCHi, s, -uh);
  const float ul = ffma(kCLo, s, ue);
  const float vh = fmul(uh, m);
  const float ve = ffma(uh, m, -vh);
  const float vl = ffma(ul, m, ve);
  const float t = fadd(r, vh);
  const float z = fsub(t, r);
  const float e = fadd(fsub(r, fsub(t, z)), fsub(vh, z));
  const float yl = fadd(e, vl);
  const float R = fadd(t, yl);
  const float d = fadd(fsub(t, R), yl);
  const float avh = fabs_(vh), at = fabs_(t);
  const unsigned int rb = bits(R) & 0x7fffffffu;
  const unsigned int ex = rb & 0x7f800000u;
  // R in [2^-97, 2^127]: half the spacing around R is a normal float (the
  // spacing below a power of two is half the one above: take the smaller)
  if (fabs_(uh) >= 0x1p-100f && avh >= 0x1p-100f &&
      fabs_(yl) <= fmul(0.25f, at) && ex >= (30u << 23) && ex < (255u << 23)) {
    const float half =
        from_bits(ex - ((rb & 0x7fffffu) == 0u ? (25u << 23) : (24u << 23)));
    const float delta = fmul(0x1p-44f, fadd(avh, at));
    if (fabs_(d) < fsub(fsub(half, fmul(half, 0x1p-20f)), delta)) return R;
  }
  // a product far below half an ulp of r: |vh| < 2^-100 and |m| <= 2^20
  // bound |V| below 2^-99 (|uh| normal: relative error 2^-24; |uh| below
  // 2^-126: |1e-6 s| < 2^-125), and |r| >= 2^-60 has half an ulp >= 2^-85
  if (avh < 0x1p-100f && fabs_(m) <= 0x1p20f && fabs_(r) >= 0x1p-60f &&
      fabs_(r) <= 0x1p127f)
    return r;
  if (fell_back) *fell_back = true;
  return reference_double(r, s, m);
}

}  // namespace couple
}  // namespace born
