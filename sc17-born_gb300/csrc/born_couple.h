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
// |uh|, |vh| >= 2^-100 (no underflow in the exact products).  R = fl(t + yl)
// is the answer when fl(t + fl(yl - 2 delta)) and fl(t + fl(yl + 2 delta))
// both equal R: those sums bracket W (the inner roundings move them by less
// than delta / 2), and rounding to nearest is monotonic, so W rounds to R
// too.  An exact zero s or m makes the product a signed zero, and r + (+-0)
// rounds alike in float and double; a product far below half an ulp of r
// gives r itself; small fields are evaluated scaled by 2^64 (exact); every
// other cell (a bracket that straddles a rounding boundary, results in or
// near float's subnormal range) takes the reference's expression in double.
// Measured on the oracle's own fields (a 160^3 grid of the benchmark's
// model family, 400 steps): 3.8e-4 of the cell updates take the double
// fallback, all of them in the first steps' faint tails.  The host instance is compiled without fused multiply-adds
// (-ffp-contract=off) and checked against the double expression on random
// and near-tie inputs; the device instance uses the same operations with
// explicit rounding intrinsics, which are never contracted.
#pragma once

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

// (float)((double)r + 1e-6 * (double)s * (double)m) in float arithmetic,
// or *fell_back = true when only the double expression decides it.  One
// float evaluation per cell, the cases chosen by selects, so that the lanes
// of a warp stay together.
BORN_HD float couple_fast(float r, float s, float m, bool *fell_back) {
  // small fields (the faint tails ahead of a wavefront) are evaluated as
  // 2^64 s and 2^64 r: exact scalings that make the double expression
  // exactly 2^64 W, so the float evaluation scaled back is (float)W while
  // that is a normal float (|result| >= 2^-125 keeps clear of the
  // subnormals, whose rounding does not scale)
  const bool small = fabs_(s) < 0x1p-40f && fabs_(r) < 0x1p60f;
  const float sc = small ? 0x1p64f : 1.f;
  const float s2 = fmul(s, sc), r2 = fmul(r, sc);
  const float uh = fmul(kCHi, s2);
  const float vh = fmul(uh, m);
  const float ue = ffma(kCHi, s2, -uh);
  const float ul = ffma(kCLo, s2, ue);
  const float ve = ffma(uh, m, -vh);
  const float vl = ffma(ul, m, ve);
  const float t = fadd(r2, vh);
  const float z = fsub(t, r2);
  const float e = fadd(fsub(r2, fsub(t, z)), fsub(vh, z));
  const float yl = fadd(e, vl);
  const float R = fadd(t, yl);
  const float avh = fabs_(vh);
  const float d2 = fmul(0x1p-43f, fadd(avh, fabs_(t)));  // 2 delta
  const bool ok = fabs_(uh) >= 0x1p-100f && avh >= 0x1p-100f &&
                  fadd(t, fsub(yl, d2)) == R && fadd(t, fadd(yl, d2)) == R &&
                  (!small || fabs_(R) >= 0x1p-61f);
  // the product is a signed zero in both forms: r + (+-0) rounds alike
  const bool zero = s == 0.f || m == 0.f;
  // a product far below half an ulp of r: |vh| < 2^-100 (unscaled) and
  // |m| <= 2^20 bound |V| below 2^-99 (|uh| normal: relative error 2^-24;
  // |uh| below 2^-126: |1e-6 s| < 2^-125), and |r| >= 2^-60 has half an ulp
  // >= 2^-85
  const float inv = small ? 0x1p-64f : 1.f;
  const bool keep_r = fmul(avh, inv) < 0x1p-100f && fabs_(m) <= 0x1p20f &&
                      fabs_(r) >= 0x1p-60f && fabs_(r) <= 0x1p127f;
  const float res = zero ? fadd(r, fmul(fmul(kCHi, s), m))
                  : keep_r ? r
                  : fmul(R, inv);
  *fell_back = !zero && !keep_r && !ok;
  return res;
}

#ifdef __CUDACC__
// couple_fast on two cells at once (lanes lo, hi of a 64-bit pair), with
// the sums and multiply-adds in packed FP32 pairs (each lane rounds as the
// scalar operation).  The products whose results feed an add (vh, and the
// scalings of r) stay scalar: the compiler contracts a packed multiply
// feeding a packed add into a fused multiply-add, and vh must be rounded
// before r + vh for the exact sum.  Bit 0 / 1 of the result flag: lane lo /
// hi needs the double fallback.
__device__ __forceinline__ unsigned long long cp_pk(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 cp_upk(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ unsigned long long cp_add(unsigned long long a,
                                                     unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long cp_sub(unsigned long long a,
                                                     unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long cp_mul(unsigned long long a,
                                                     unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long cp_fma(unsigned long long a,
                                                     unsigned long long b,
                                                     unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

__device__ __forceinline__ float2 couple_fast2(float2 r, float2 s, float2 m,
                                               unsigned int *fell_back) {
  const bool sml0 = fabsf(s.x) < 0x1p-40f && fabsf(r.x) < 0x1p60f;
  const bool sml1 = fabsf(s.y) < 0x1p-40f && fabsf(r.y) < 0x1p60f;
  const float sc0 = sml0 ? 0x1p64f : 1.f, sc1 = sml1 ? 0x1p64f : 1.f;
  // scalings by powers of two are exact
  const unsigned long long S = cp_mul(cp_pk(s.x, s.y), cp_pk(sc0, sc1));
  const float rs0 = __fmul_rn(r.x, sc0), rs1 = __fmul_rn(r.y, sc1);
  const unsigned long long Rr = cp_pk(rs0, rs1), M = cp_pk(m.x, m.y);
  const unsigned long long CH = cp_pk(kCHi, kCHi), CL = cp_pk(kCLo, kCLo);
  const unsigned long long UH = cp_mul(CH, S);
  const float2 uh = cp_upk(UH);
  const float vh0 = __fmul_rn(uh.x, m.x), vh1 = __fmul_rn(uh.y, m.y);
  const unsigned long long VH = cp_pk(vh0, vh1);
  const unsigned long long NUH = cp_pk(-uh.x, -uh.y);
  const unsigned long long UE = cp_fma(CH, S, NUH);
  const unsigned long long UL = cp_fma(CL, S, UE);
  const unsigned long long VE = cp_fma(UH, M, cp_pk(-vh0, -vh1));
  const unsigned long long VL = cp_fma(UL, M, VE);
  const unsigned long long T = cp_add(Rr, VH);
  const unsigned long long Z = cp_sub(T, Rr);
  const unsigned long long E =
      cp_add(cp_sub(Rr, cp_sub(T, Z)), cp_sub(VH, Z));
  const unsigned long long YL = cp_add(E, VL);
  const unsigned long long RR = cp_add(T, YL);
  const float2 t = cp_upk(T);
  const unsigned long long D2 = cp_mul(
      cp_pk(0x1p-43f, 0x1p-43f),
      cp_add(cp_pk(fabsf(vh0), fabsf(vh1)), cp_pk(fabsf(t.x), fabsf(t.y))));
  const float2 lo = cp_upk(cp_add(T, cp_sub(YL, D2)));
  const float2 hi = cp_upk(cp_add(T, cp_add(YL, D2)));
  const float2 R = cp_upk(RR);
  const float inv0 = sml0 ? 0x1p-64f : 1.f, inv1 = sml1 ? 0x1p-64f : 1.f;
  const bool ok0 = fabsf(uh.x) >= 0x1p-100f && fabsf(vh0) >= 0x1p-100f &&
                   lo.x == R.x && hi.x == R.x &&
                   (!sml0 || fabsf(R.x) >= 0x1p-61f);
  const bool ok1 = fabsf(uh.y) >= 0x1p-100f && fabsf(vh1) >= 0x1p-100f &&
                   lo.y == R.y && hi.y == R.y &&
                   (!sml1 || fabsf(R.y) >= 0x1p-61f);
  const bool zero0 = s.x == 0.f || m.x == 0.f;
  const bool zero1 = s.y == 0.f || m.y == 0.f;
  const bool keep0 = __fmul_rn(fabsf(vh0), inv0) < 0x1p-100f &&
                     fabsf(m.x) <= 0x1p20f && fabsf(r.x) >= 0x1p-60f &&
                     fabsf(r.x) <= 0x1p127f;
  const bool keep1 = __fmul_rn(fabsf(vh1), inv1) < 0x1p-100f &&
                     fabsf(m.y) <= 0x1p20f && fabsf(r.y) >= 0x1p-60f &&
                     fabsf(r.y) <= 0x1p127f;
  // an exact zero s or m: vh is that signed zero (scaled by a positive
  // power of two), and r + (+-0) rounds alike in float and double
  float2 out;
  out.x = zero0 ? __fadd_rn(r.x, vh0) : keep0 ? r.x : __fmul_rn(R.x, inv0);
  out.y = zero1 ? __fadd_rn(r.y, vh1) : keep1 ? r.y : __fmul_rn(R.y, inv1);
  *fell_back = (!zero0 && !keep0 && !ok0 ? 1u : 0u) |
               (!zero1 && !keep1 && !ok1 ? 2u : 0u);
  return out;
}

// the double fallback out of line, so that the compiler cannot turn the
// rare branch into double arithmetic on every cell (FP64 runs at a small
// fraction of the FP32 rate on this GPU)
static __device__ __noinline__ float couple_slow(float r, float s, float m) {
  return reference_double(r, s, m);
}
#endif

// the reference's coupling: the float evaluation, else the double one;
// *fell_back (when not null) reports the fallback
BORN_HD float couple_exact(float r, float s, float m, bool *fell_back) {
  bool fb = false;
  float v = couple_fast(r, s, m, &fb);
  if (fell_back) *fell_back = fb;
#ifdef __CUDA_ARCH__
  if (fb) v = couple_slow(r, s, m);
#else
  if (fb) v = reference_double(r, s, m);
#endif
  return v;
}

}  // namespace couple
}  // namespace born
