// Templated body of the fused time-step kernels (design in born_step.cuh).
// Included by born_step.cu (FP32 storage, reference order),
// born_step_bf16.cu, born_step_f16.cu, born_step_f32fused.cu and
// born_step_f32exact.cu so that the storage families compile in parallel; each includer instantiates its
// storage type with BORN_DEFINE_STORAGE_ENTRY.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "born_couple.h"
#include "born_step.cuh"

namespace born {
namespace {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + TMA (sm_90+ forms, valid on sm_103a)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: gives up after ~2 s of wall time so that a lost transfer
// turns into an error status instead of a hung GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar,
                                                  uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63u) == 63u && global_ns() - t0 > 2000000000ull) return false;
  }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm,
                                            int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::"
      "bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ float comp(const float4 &v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp(float4 &v, int j, float x) {
  if (j == 0) v.x = x;
  else if (j == 1) v.y = x;
  else if (j == 2) v.z = x;
  else v.w = x;
}
__device__ __forceinline__ float4 scale4(const float4 &v, float s) {
  return make_float4(v.x * s, v.y * s, v.z * s, v.w * s);
}
__device__ __forceinline__ float absmax4(const float4 &v, float m) {
  return fmaxf(fmaxf(fmaxf(m, fabsf(v.x)), fmaxf(fabsf(v.y), fabsf(v.z))),
               fabsf(v.w));
}

// ---------------------------------------------------------------------------
// Storage of the wavefield levels

template <int ST>
struct Store {
  static constexpr bool kLow = ST == kStoreBF16 || ST == kStoreF16;
  static constexpr int kBytes = kLow ? 2 : 4;
  // fused multiply-add arithmetic (every storage but the reference order)
  static constexpr bool kFused = ST != kStoreF32 && ST != kStoreF32Exact;
  // the Born coupling formed as the reference's double expression
  static constexpr bool kExact = ST == kStoreF32Exact;
};

// Four consecutive values starting at element `e` of a shared tile.
template <int ST>
__device__ __forceinline__ float4 ld4(const unsigned char *base, int e) {
  if constexpr (!Store<ST>::kLow) {
    return *reinterpret_cast<const float4 *>(base + 4 * e);
  } else {
    const uint2 u = *reinterpret_cast<const uint2 *>(base + 2 * e);
    if constexpr (ST == kStoreBF16) {
      // a bf16 is the upper half of the float with the same bits
      return make_float4(__uint_as_float(u.x << 16),
                         __uint_as_float(u.x & 0xffff0000u),
                         __uint_as_float(u.y << 16),
                         __uint_as_float(u.y & 0xffff0000u));
    } else {
      const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
      const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
      return make_float4(a.x, a.y, b.x, b.y);
    }
  }
}

__device__ __forceinline__ float clamp_f16(float x) {
  // largest finite FP16; NaN passes through
  return x > 65504.f ? 65504.f : (x < -65504.f ? -65504.f : x);
}

// Stores four consecutive values at element idx of a level (raw units).
template <int ST>
__device__ __forceinline__ void st4_level(void *base, long long idx,
                                          const float4 &v) {
  if constexpr (!Store<ST>::kLow) {
    *reinterpret_cast<float4 *>(static_cast<float *>(base) + idx) = v;
  } else {
    uint2 u;
    if constexpr (ST == kStoreBF16) {
      __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
      __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
      u.x = *reinterpret_cast<unsigned int *>(&a);
      u.y = *reinterpret_cast<unsigned int *>(&b);
    } else {
      __half2 a = __floats2half2_rn(clamp_f16(v.x), clamp_f16(v.y));
      __half2 b = __floats2half2_rn(clamp_f16(v.z), clamp_f16(v.w));
      u.x = *reinterpret_cast<unsigned int *>(&a);
      u.y = *reinterpret_cast<unsigned int *>(&b);
    }
    *reinterpret_cast<uint2 *>(static_cast<unsigned short *>(base) + idx) = u;
  }
}

template <int ST>
__device__ __forceinline__ float ld1_level(const void *base, long long i) {
  if constexpr (!Store<ST>::kLow) {
    return static_cast<const float *>(base)[i];
  } else if constexpr (ST == kStoreBF16) {
    const unsigned short b = static_cast<const unsigned short *>(base)[i];
    return __uint_as_float((unsigned int)b << 16);
  } else {
    return __half2float(static_cast<const __half *>(base)[i]);
  }
}

template <int ST>
__device__ __forceinline__ void st1_level(void *base, long long i, float v) {
  if constexpr (!Store<ST>::kLow) {
    static_cast<float *>(base)[i] = v;
  } else if constexpr (ST == kStoreBF16) {
    static_cast<__nv_bfloat16 *>(base)[i] = __float2bfloat16_rn(v);
  } else {
    static_cast<__half *>(base)[i] = __float2half_rn(clamp_f16(v));
  }
}

// Stored values are kept at or below 2^15 in magnitude (FP16 overflows
// above 65504): the scale of a new level is the power of two
// 2^(ceil(log2 bound) - 15) for a bound on its magnitude.
constexpr int kScaleHeadroomLog2 = 15;

__device__ __forceinline__ float pow2_scale_for(float bound) {
  if (!(bound > 0.f) || bound > 3.0e38f) return 1.f;
  const unsigned int b = __float_as_uint(bound);
  int e = (int)((b >> 23) & 0xffu) - 127;       // floor(log2) (normal floats)
  if ((b & 0x7fffffu) != 0u || e < -126) e += 1;  // round up to a power of two
  e -= kScaleHeadroomLog2;
  e = e < -120 ? -120 : (e > 120 ? 120 : e);
  return __uint_as_float((unsigned int)(e + 127) << 23);
}

__device__ __forceinline__ float rec_max(const unsigned long long *lv, int r) {
  return r < 0 ? 0.f
               : __uint_as_float((unsigned int)(lv[2 * r] & 0xffffffffull));
}
__device__ __forceinline__ float rec_scale(const unsigned long long *lv,
                                           int r) {
  return r < 0 ? 1.f
               : __uint_as_float((unsigned int)(lv[2 * r + 1] & 0xffffffffull));
}

// Bound of one step's injection: |trace| * |dir/jt| * sum |tab| per point,
// times the most points sharing a cell.
__device__ __forceinline__ float inject_bound(const PointSet &ps) {
  if (!ps.active || !ps.absmax) return 0.f;
  float t = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += fabsf(ps.tab[k]);
  return __uint_as_float(*ps.absmax) * fabsf(ps.scale) * t * (float)ps.mult;
}

// ---------------------------------------------------------------------------
// Reference arithmetic (FP32 storage)

// Leapfrog update of cpuProp::prop (cpu_prop.cc:233-248): v*S + p + p - old,
// every operation separately rounded (no FMA contraction).
__device__ __forceinline__ float leapfrog(float vel, float s, float p,
                                          float old) {
  return __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(vel, s), p), p), old);
}

// dir/jt * (t0 v0 + ... + t7 v7), cpu_prop.cc:169-177 / 186-194
__device__ __forceinline__ float point_value(const PointSet &ps, int idx) {
  const float *v = ps.traces + (long long)idx * ps.nt_trace + ps.id;
  float s = __fmul_rn(ps.tab[0], v[0]);
#pragma unroll
  for (int k = 1; k < 8; ++k) s = __fadd_rn(s, __fmul_rn(ps.tab[k], v[k]));
  return __fmul_rn(ps.scale, s);
}

// Adds the injection of every point lying on this thread's 4 cells of row
// gy, plane z, in point order.  Uniform early-out when the plane is empty.
__device__ __forceinline__ void inject_row(const PointSet &ps, int n1, int n2,
                                           int z, int gy, int gx, float4 &v) {
  if (z < ps.zlo || z > ps.zhi) return;
  const int off = ps.plane_off[z];
  if (off < 0) return;
  const int4 h = *reinterpret_cast<const int4 *>(ps.cell_head + off +
                                                 (long long)gy * n1 + gx);
  const int hh[4] = {h.x, h.y, h.z, h.w};
  const long long cell0 = ((long long)z * n2 + gy) * n1 + gx;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (hh[j] < 0) continue;
    float a = comp(v, j);
    for (int s = hh[j]; s < ps.npts && ps.slot_cell[s] == (int)(cell0 + j);
         ++s)
      a = __fadd_rn(a, point_value(ps, ps.slot_index[s]));
    set_comp(v, j, a);
  }
}

// rec[idx][id+k] += v * t[k] at every point on this thread's cells
// (cpu_prop.cc:205-212).
__device__ __forceinline__ void extract_row(const PointSet &ps, int n1, int n2,
                                            int z, int gy, int gx,
                                            const float4 &v) {
  if (z < ps.zlo || z > ps.zhi) return;
  const int off = ps.plane_off[z];
  if (off < 0) return;
  const int4 h = *reinterpret_cast<const int4 *>(ps.cell_head + off +
                                                 (long long)gy * n1 + gx);
  const int hh[4] = {h.x, h.y, h.z, h.w};
  const long long cell0 = ((long long)z * n2 + gy) * n1 + gx;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (hh[j] < 0) continue;
    const float a = comp(v, j);
    for (int s = hh[j]; s < ps.npts && ps.slot_cell[s] == (int)(cell0 + j);
         ++s) {
      float *r = ps.traces + (long long)ps.slot_index[s] * ps.nt_trace + ps.id;
#pragma unroll
      for (int k = 0; k < 8; ++k) r[k] = __fadd_rn(r[k], __fmul_rn(a, ps.tab[k]));
    }
  }
}

__device__ __forceinline__ void st4(float *p, const float4 &v) {
  *reinterpret_cast<float4 *>(p) = v;
}

// Packed FP32 pairs (add/sub/mul/fma.rn.f32x2, sm_100 family): one
// instruction rounds each lane exactly as the scalar form does (IEEE
// round-to-nearest, subnormals kept; checked lane by lane on sm_103a).  A
// pair is two adjacent 32-bit registers: the (x, y) and (z, w) halves of a
// float4 are pairs as loaded.  One caveat decides where they may be used in
// the reference-order arithmetic: the compiler contracts a packed multiply
// whose result feeds a packed add or subtract into a packed fused
// multiply-add, whatever the rounding modifier or -fmad setting (measured on
// sm_103a, also for fma(a, b, -0)), while a scalar mul.rn feeding a packed
// add is left alone.  So the reference-order sums multiply with scalar
// __fmul_rn (mulc2s, mul2s) and add in pairs; the fused-arithmetic paths
// use packed multiplies and multiply-adds throughout.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 upk2(f32x2 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
// c * v and a * b lane by lane with scalar, never-contracted multiplies
__device__ __forceinline__ f32x2 mulc2s(float c, f32x2 v) {
  const float2 t = upk2(v);
  return pk2(__fmul_rn(c, t.x), __fmul_rn(c, t.y));
}
__device__ __forceinline__ f32x2 mul2s(f32x2 a, f32x2 b) {
  const float2 x = upk2(a), y = upk2(b);
  return pk2(__fmul_rn(x.x, y.x), __fmul_rn(x.y, y.y));
}
// cells (x, x+1) (h = 0) or (x+2, x+3) (h = 1) of a float4
__device__ __forceinline__ f32x2 cells2(const float4 &v, int h) {
  return h == 0 ? pk2(v.x, v.y) : pk2(v.z, v.w);
}
__device__ __forceinline__ void set_cells2(float4 &v, int h, f32x2 x) {
  const float2 t = upk2(x);
  if (h == 0) {
    v.x = t.x;
    v.y = t.y;
  } else {
    v.z = t.x;
    v.w = t.y;
  }
}
// leapfrog() on a pair of cells
__device__ __forceinline__ f32x2 leapfrog2(f32x2 vel, f32x2 s, f32x2 p,
                                           f32x2 old) {
  return sub2(add2(add2(mul2s(vel, s), p), p), old);
}

// Stencil sums of this thread's 4 consecutive cells (x .. x+3) of one row,
// from a TMA box (x/y neighbours) and the register z window.  Each cell's
// sum is formed in the reference order of cpuProp::prop (cpu_prop.cc:235-247):
// C0 p, then the x pairs, the y pairs and the z pairs, every product and sum
// separately rounded.  The four cells advance together so that every shared
// load is a float4 (3 for the x window, 2 per y offset), as two packed pairs
// (cells x, x+1 and x+2, x+3) whose neighbour sums and running sums are
// packed adds; the products are scalar (see f32x2).  The x offsets of odd
// distance need pairs that straddle the loaded float4s, built once
// (w1..w10).
template <int BX>
__device__ __forceinline__ float4 stencil4(const float *box, int brow,
                                           int bcol, const float4 (&q)[9],
                                           const float *c, float4 &center) {
  const float *r = box + brow * BX + bcol;
  const float4 L = *reinterpret_cast<const float4 *>(r - 4);
  const float4 M = *reinterpret_cast<const float4 *>(r);
  const float4 R = *reinterpret_cast<const float4 *>(r + 4);
  center = M;
  // x window w0..w11 = L, M, R: pairs starting at even w (as loaded) and at
  // odd w
  const f32x2 e0 = pk2(L.x, L.y), e2 = pk2(L.z, L.w), e4 = pk2(M.x, M.y),
              e6 = pk2(M.z, M.w), e8 = pk2(R.x, R.y), e10 = pk2(R.z, R.w);
  const f32x2 o1 = pk2(L.y, L.z), o3 = pk2(L.w, M.x), o5 = pk2(M.y, M.z),
              o7 = pk2(M.w, R.x), o9 = pk2(R.y, R.z);
  // cells (x, x+1): centre e4; cells (x+2, x+3): centre e6
  f32x2 s0 = mulc2s(c[0], e4), s1 = mulc2s(c[0], e6);
  s0 = add2(s0, mulc2s(c[2], add2(o3, o5)));
  s1 = add2(s1, mulc2s(c[2], add2(o5, o7)));
  s0 = add2(s0, mulc2s(c[5], add2(e2, e6)));
  s1 = add2(s1, mulc2s(c[5], add2(e4, e8)));
  s0 = add2(s0, mulc2s(c[8], add2(o1, o7)));
  s1 = add2(s1, mulc2s(c[8], add2(o3, o9)));
  s0 = add2(s0, mulc2s(c[11], add2(e0, e8)));
  s1 = add2(s1, mulc2s(c[11], add2(e2, e10)));
  const int cy[4] = {3, 6, 9, 12}, cz[4] = {1, 4, 7, 10};
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    const float4 u = *reinterpret_cast<const float4 *>(r - m * BX);
    const float4 d = *reinterpret_cast<const float4 *>(r + m * BX);
    const float k = c[cy[m - 1]];
    s0 = add2(s0, mulc2s(k, add2(pk2(u.x, u.y), pk2(d.x, d.y))));
    s1 = add2(s1, mulc2s(k, add2(pk2(u.z, u.w), pk2(d.z, d.w))));
  }
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    const float4 &u = q[4 - m], &d = q[4 + m];
    const float k = c[cz[m - 1]];
    s0 = add2(s0, mulc2s(k, add2(pk2(u.x, u.y), pk2(d.x, d.y))));
    s1 = add2(s1, mulc2s(k, add2(pk2(u.z, u.w), pk2(d.z, d.w))));
  }
  const float2 a = upk2(s0), b = upk2(s1);
  return make_float4(a.x, a.y, b.x, b.y);
}

// The same sums with fused multiply-adds, over the stored values of any
// storage (16-bit values in raw units: the caller applies the level's
// scale).  Used by every storage but the reference-order FP32 one: these
// paths are judged by their error, not by bit equality.  Packed pairs as in
// stencil4 (fma.rn.f32x2 rounds each lane once, as fmaf does).
template <int BX, int ST>
__device__ __forceinline__ float4 stencil4_lp(const unsigned char *box,
                                              int brow, int bcol,
                                              const float4 (&q)[9],
                                              const float *c, float4 &center) {
  const int e = brow * BX + bcol;
  const float4 L = ld4<ST>(box, e - 4);
  const float4 M = ld4<ST>(box, e);
  const float4 R = ld4<ST>(box, e + 4);
  center = M;
  const f32x2 e0 = pk2(L.x, L.y), e2 = pk2(L.z, L.w), e4 = pk2(M.x, M.y),
              e6 = pk2(M.z, M.w), e8 = pk2(R.x, R.y), e10 = pk2(R.z, R.w);
  const f32x2 o1 = pk2(L.y, L.z), o3 = pk2(L.w, M.x), o5 = pk2(M.y, M.z),
              o7 = pk2(M.w, R.x), o9 = pk2(R.y, R.z);
  auto cc = [&](int k) { return pk2(c[k], c[k]); };
  f32x2 s0 = mul2(cc(0), e4), s1 = mul2(cc(0), e6);
  s0 = fma2(cc(2), add2(o3, o5), s0);
  s1 = fma2(cc(2), add2(o5, o7), s1);
  s0 = fma2(cc(5), add2(e2, e6), s0);
  s1 = fma2(cc(5), add2(e4, e8), s1);
  s0 = fma2(cc(8), add2(o1, o7), s0);
  s1 = fma2(cc(8), add2(o3, o9), s1);
  s0 = fma2(cc(11), add2(e0, e8), s0);
  s1 = fma2(cc(11), add2(e2, e10), s1);
  const int cy[4] = {3, 6, 9, 12}, cz[4] = {1, 4, 7, 10};
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    const float4 u = ld4<ST>(box, e - m * BX);
    const float4 d = ld4<ST>(box, e + m * BX);
    const f32x2 k = cc(cy[m - 1]);
    s0 = fma2(k, add2(pk2(u.x, u.y), pk2(d.x, d.y)), s0);
    s1 = fma2(k, add2(pk2(u.z, u.w), pk2(d.z, d.w)), s1);
  }
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    const float4 &u = q[4 - m], &d = q[4 + m];
    const f32x2 k = cc(cz[m - 1]);
    s0 = fma2(k, add2(pk2(u.x, u.y), pk2(d.x, d.y)), s0);
    s1 = fma2(k, add2(pk2(u.z, u.w), pk2(d.z, d.w)), s1);
  }
  const float2 a = upk2(s0), b = upk2(s1);
  return make_float4(a.x, a.y, b.x, b.y);
}

// ---------------------------------------------------------------------------
// Compile-time description of a mode

template <int MODE, bool PA, bool PB>
struct ModeTraits {
  static constexpr bool kTwoField = (MODE == kModeForward ||
                                     MODE == kModeBornLin ||
                                     MODE == kModeAdjoint);
  static constexpr bool kBoxA = PA;
  static constexpr bool kBoxB = kTwoField && PB;
  static constexpr int kNF = (kBoxA ? 1 : 0) + (kBoxB ? 1 : 0);
  static constexpr unsigned kMask =
      MODE == kModeSource || MODE == kModeModel
          ? (1u << kOldA) | (1u << kVelA)
      : MODE == kModeForward || MODE == kModeBornLin
          ? (1u << kOldA) | (1u << kOldB) | (1u << kVelA) | (1u << kImg)
      : MODE == kModeAdjoint
          ? (1u << kOldA) | (1u << kOldB) | (1u << kImg) |
                (PA ? (1u << kVelA) : 0u) | (PB ? (1u << kVelB) : 0u)
          : /* kModeBornAdj: OldB slot carries g = A s */
          (1u << kOldA) | (1u << kOldB) | (1u << kVelA) | (1u << kImg);
  static constexpr bool kDampA = MODE != kModeSource;
  static constexpr bool kDampB = MODE == kModeForward || MODE == kModeBornLin;
};

// Shared-memory geometry of one tile shape for field elements of EB bytes.
// TMA copies of 16-bit rows must start at an x that is a multiple of 8
// elements; the interior starts at x = 4, so 16-bit centre tiles are copied
// from x0 - 4 with 8 extra columns (the halo boxes already start there).
template <int TX, int TY, int EB>
struct Tile {
  static constexpr int kBX = TX + 2 * kRadius, kBY = TY + 2 * kRadius;
  static constexpr int kThreads = (TX / 4) * TY;
  static constexpr int kZCols = EB == 4 ? TX : TX + 2 * kRadius;
  static constexpr int kZOff = EB == 4 ? 0 : kRadius;
  static constexpr int kZRaw = kZCols * TY * EB;  // bytes one copy delivers
  static constexpr int kZBytes = (kZRaw + 127) / 128 * 128;
  static constexpr int kBoxRaw = kBX * kBY * EB;
  static constexpr int kBoxBytes = (kBoxRaw + 127) / 128 * 128;
  static constexpr int kCRaw = TX * TY * 4;       // FP32 centre tile
  static constexpr int kCBytes = (kCRaw + 127) / 128 * 128;
  // whole warps (the level maxima reduce over full warps); TMA boxes of
  // whole 16-byte rows starting on 16-byte boundaries for both element
  // sizes (tile origins are multiples of TX after the 4-cell halo)
  static_assert(kThreads % 32 == 0, "tile threads must fill whole warps");
  static_assert(TX % 8 == 0 && TX + 2 * kRadius <= 256 && TY + 2 * kRadius <= 256,
                "tile width must keep TMA rows 16-byte aligned");
};

// centre slots that hold levels of the propagated fields (field storage)
template <int MODE>
__host__ __device__ constexpr bool fslot(int slot) {
  return slot == kOldA || (slot == kOldB && MODE != kModeBornAdj);
}
template <int MODE, class T>
__host__ __device__ constexpr int slot_raw(int slot) {
  return fslot<MODE>(slot) ? T::kZRaw : T::kCRaw;
}
template <int MODE, class T>
__host__ __device__ constexpr int slot_bytes(int slot) {
  return fslot<MODE>(slot) ? T::kZBytes : T::kCBytes;
}
// byte offset of a centre slot inside the centre part of an output stage
template <int MODE, unsigned MASK, class T>
__host__ __device__ constexpr int slot_off(int slot) {
  int off = 0;
  for (int s = 0; s < slot; ++s)
    if (MASK & (1u << s)) off += slot_bytes<MODE, T>(s);
  return off;
}
template <int MODE, unsigned MASK, class T>
__host__ __device__ constexpr int centre_bytes(bool raw) {
  int b = 0;
  for (int s = 0; s < kNumCentre; ++s)
    if (MASK & (1u << s))
      b += raw ? slot_raw<MODE, T>(s) : slot_bytes<MODE, T>(s);
  return b;
}

template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
struct Layout {
  using M = ModeTraits<MODE, PA, PB>;
  using T = Tile<TX, TY, Store<ST>::kBytes>;
  static constexpr int kZStage = M::kNF * T::kZBytes;
  static constexpr int kOStage =
      M::kNF * T::kBoxBytes + centre_bytes<MODE, M::kMask, T>(false);
  static constexpr uint32_t kZTx = M::kNF * T::kZRaw;
  static constexpr uint32_t kOTx =
      M::kNF * T::kBoxRaw + centre_bytes<MODE, M::kMask, T>(true);
  static constexpr int kOSt = out_stages(MODE);  // output ring depth
  static constexpr int kZSt = z_stages(MODE);     // z ring depth
  static constexpr size_t kSmem =
      (size_t)kZSt * kZStage + (size_t)kOSt * kOStage + 128;
};

// Scales of one step's levels (16-bit storage), shared by the CTA.
struct StepScales {
  float cur_a, old_a, inv_new_a, cur_b, old_b, inv_new_b;
};

// One CTA's work: xy tile `tile`, z segment `seg`, with the TMA descriptors
// `mp` (kernel parameter space, or global memory in the batched launch) and
// the step parameters `p`.
template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
__device__ __forceinline__ void step_body(const StepMaps *mp,
                                          const StepParams &p, int tile,
                                          int seg) {
  const StepMaps &maps = *mp;
  // programmatic dependent launch: the next step's grid may be scheduled
  // from now on, and this grid touches global memory only once the previous
  // one has completed and its writes are visible (levels, image, traces,
  // error word); both are no-ops for a plain launch
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  using M = ModeTraits<MODE, PA, PB>;
  using T = Tile<TX, TY, Store<ST>::kBytes>;
  using LY = Layout<ST, MODE, PA, PB, TX, TY>;
  constexpr bool LP = Store<ST>::kLow;
  constexpr bool FUSED = Store<ST>::kFused;
  constexpr int NF = M::kNF;
  constexpr int BX = T::kBX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t zbars[kZStages];
  __shared__ __align__(8) uint64_t obars[kOStages];  // the first LY::kOSt
  // copies issued per ring stage (the abort path waits for the last one)
  __shared__ unsigned int s_nz[kZStages], s_no[kOStages];
  __shared__ int abort_flag;
  __shared__ float s_bound[kNBound];
  __shared__ StepScales s_sc;
  __shared__ unsigned int s_mx[2];
  // TMA destinations need 128-byte alignment: align the dynamic base here
  // (the launch reserves 128 spare bytes for this)
  unsigned char *smem =
      smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  // z ring: centre tiles of the current levels, one per new plane
  unsigned char *zring = smem;
  // output ring: halo boxes and per-cell inputs of the output plane
  unsigned char *oring = smem + LY::kZSt * LY::kZStage;

  const int tid = threadIdx.x;
  const int lx = tid % (TX / 4), ly = tid / (TX / 4);
  const int tx = tile % p.tiles_x, ty = tile / p.tiles_x;
  const int x0 = kRadius + tx * TX, y0 = kRadius + ty * TY;
  const int z0 = kRadius + seg * p.zseg;
  const int z1 = min(z0 + p.zseg, p.n3 - kRadius);
  if (z0 >= z1) return;  // uniform over the CTA
  const int n1 = p.n1, n2 = p.n2, n3 = p.n3;
  const long long n12 = (long long)n1 * n2;
  const int gx = x0 + 4 * lx, gy = y0 + ly;
  const bool valid = (gx < n1 - kRadius) && (gy < n2 - kRadius);
  // x of the field centre copies (16-bit rows start 4 columns early)
  const int xz = x0 - T::kZOff;

  // taper: distance to the interior faces in x/y per cell (cpu_prop.cc:146-151)
  int exy[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int x = gx + j;
    exy[j] = min(min(x - 4, n1 - 4 - x), min(gy - 4, n2 - 4 - gy));
  }

  if (tid == 0) {
    for (int s = 0; s < LY::kZSt; ++s) mbar_init(&zbars[s], 1);
    for (int s = 0; s < LY::kOSt; ++s) mbar_init(&obars[s], 1);
    for (int s = 0; s < kZStages; ++s) s_nz[s] = 0u;
    for (int s = 0; s < kOStages; ++s) s_no[s] = 0u;
    // a wait elsewhere already gave up: the whole CTA leaves untouched
    abort_flag = *reinterpret_cast<volatile unsigned int *>(p.err) != 0u;
    mbar_fence_init();
    if constexpr (LP) {
      // scales of the levels read, and of the levels written from a bound
      // on their magnitude: |v S| <= vmax csum max|cur|, plus 2 max|cur|,
      // max|old| and the injections (every CTA computes the same values)
      const float ga = __uint_as_float(*p.vmax_a) * p.csum + 2.f;
      const float ma = rec_max(p.lv, p.la.cur), mo = rec_max(p.lv, p.la.old);
      const float ba = ga * ma + mo + inject_bound(p.pa);
      s_sc.cur_a = rec_scale(p.lv, p.la.cur);
      s_sc.old_a = rec_scale(p.lv, p.la.old);
      const float na = pow2_scale_for(ba);
      s_sc.inv_new_a = 1.f / na;  // exact: a power of two
      s_sc.cur_b = s_sc.old_b = s_sc.inv_new_b = 1.f;
      float nb = 1.f;
      if (M::kTwoField) {
        const float gb = __uint_as_float(*p.vmax_b) * p.csum + 2.f;
        float bb = gb * rec_max(p.lv, p.lb.cur) + rec_max(p.lv, p.lb.old);
        if (MODE == kModeAdjoint) bb += inject_bound(p.pb);  // pending, old
        if (MODE == kModeForward)  // Born coupling 1e-6 s_new img
          bb += 1e-6f * ba * __uint_as_float(*p.imgmax);
        s_sc.cur_b = rec_scale(p.lv, p.lb.cur);
        s_sc.old_b = rec_scale(p.lv, p.lb.old);
        nb = pow2_scale_for(bb);
        s_sc.inv_new_b = 1.f / nb;
      }
      if (tile == 0 && seg == 0) {  // one CTA records the new scales
        if (p.la.out >= 0) p.lv[2 * p.la.out + 1] = __float_as_uint(na);
        if (M::kTwoField && p.lb.out >= 0)
          p.lv[2 * p.lb.out + 1] = __float_as_uint(nb);
      }
      s_mx[0] = 0u;
      s_mx[1] = 0u;
    }
  }
  if (tid < kNBound) s_bound[tid] = p.bound[tid];
  __syncthreads();
  if (abort_flag) return;  // uniform: read after the barrier
  // The taper factor of a cell is B(min(ex, ey, ez)) with B(e) = bound[e]
  // for e < 40 and 1 beyond: B does not decrease over the interior (e >= 0),
  // so the factor is min(B(min(ex, ey)), B(ez)) exactly -- one value per
  // x/y position here, one per plane below
  float bxy[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    bxy[j] = (exy[j] >= 0 && exy[j] < kNBound) ? s_bound[exy[j]] : 1.0f;

  const int K = (z1 - z0) + 2 * kRadius;  // z-window planes z0-4 .. z1+3
  const int J = z1 - z0;                  // output planes
  auto issue_z = [&](int k) {
    const int plane = z0 - kRadius + k;
    const int st = k % LY::kZSt;
    ++s_nz[st];
    mbar_expect_tx(&zbars[st], LY::kZTx);
    unsigned char *dst = zring + st * LY::kZStage;
    if (M::kBoxA) tma_load_3d(dst, &maps.zc_a, xz, y0, plane, &zbars[st]);
    if (M::kBoxB)
      tma_load_3d(dst + (M::kBoxA ? T::kZBytes : 0), &maps.zc_b, xz, y0,
                  plane, &zbars[st]);
  };
  auto issue_out = [&](int j) {
    const int plane = z0 + j;
    const int st = j % LY::kOSt;
    ++s_no[st];
    mbar_expect_tx(&obars[st], LY::kOTx);
    unsigned char *dst = oring + st * LY::kOStage;
    if (M::kBoxA)
      tma_load_3d(dst, &maps.box_a, x0 - kRadius, y0 - kRadius, plane,
                  &obars[st]);
    if (M::kBoxB)
      tma_load_3d(dst + (M::kBoxA ? T::kBoxBytes : 0), &maps.box_b,
                  x0 - kRadius, y0 - kRadius, plane, &obars[st]);
    unsigned char *cdst = dst + NF * T::kBoxBytes;
#pragma unroll
    for (int s = 0; s < kNumCentre; ++s)
      if (M::kMask & (1u << s)) {
        tma_load_3d(cdst + slot_off<MODE, M::kMask, T>(s), &maps.cm[s],
                    fslot<MODE>(s) ? xz : x0, y0, plane, &obars[st]);
      }
  };
  if (tid == 0) {
    if (NF > 0)
      for (int k = 0; k < min(K, LY::kZSt); ++k) issue_z(k);
    for (int j = 0; j < min(J, LY::kOSt); ++j) issue_out(j);
  }

  float4 qa[9], qb[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    qa[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    qb[i] = qa[i];
  }
  const int brow = ly + kRadius, bcol = 4 * lx + kRadius;
  const int fe = ly * T::kZCols + T::kZOff + 4 * lx;  // field centre element
  const int ce = ly * TX + 4 * lx;                     // FP32 centre element
  float mx_a = 0.f, mx_b = 0.f;  // max |stored value| (16-bit storage)

  // unrolling by 3 realigns the z window's registers every third plane
  // instead of shifting it every plane (measured: source and forward steps
  // 2-4 % faster, the two-field adjoint step 6 % slower)
  constexpr int kUnroll = MODE == kModeAdjoint ? 1 : 3;
#pragma unroll kUnroll
  for (int k = 0; k < K; ++k) {
    const int st = k % LY::kZSt;
    const int j = k - 2 * kRadius;       // output index once k >= 8
    const int zo = z0 + j;
    const long long idx = (long long)zo * n12 + (long long)gy * n1 + gx;

    bool ok = true;
    if (NF > 0) {
      ok = mbar_wait_bounded(&zbars[st], (uint32_t)((k / LY::kZSt) & 1));
      // newest plane's centre enters the z window
      const unsigned char *sa = zring + st * LY::kZStage;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        qa[i] = qa[i + 1];
        qb[i] = qb[i + 1];
      }
      if (M::kBoxA) qa[8] = ld4<ST>(sa, fe);
      if (M::kBoxB) qb[8] = ld4<ST>(sa + (M::kBoxA ? T::kZBytes : 0), fe);
    }

    if (j >= 0 && ok) {
      const int os = j % LY::kOSt;
      ok = mbar_wait_bounded(&obars[os], (uint32_t)((j / LY::kOSt) & 1));
      const unsigned char *ost = oring + os * LY::kOStage;
      const unsigned char *cst = ost + NF * T::kBoxBytes;
      auto centre = [&](int slot) {
        const unsigned char *b = cst + slot_off<MODE, M::kMask, T>(slot);
        return fslot<MODE>(slot) ? ld4<ST>(b, fe) : ld4<kStoreF32>(b, ce);
      };
      const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 oa = (M::kMask & (1u << kOldA)) ? centre(kOldA) : zero4;
      float4 ob = (M::kMask & (1u << kOldB)) ? centre(kOldB) : zero4;
      if constexpr (LP) {  // true values of the previous levels
        oa = scale4(oa, s_sc.old_a);
        ob = scale4(ob, s_sc.old_b);
      }
      const float4 va = (M::kMask & (1u << kVelA)) ? centre(kVelA) : zero4;
      const float4 vb = (M::kMask & (1u << kVelB)) ? centre(kVelB)
                        : (MODE == kModeForward || MODE == kModeBornLin) ? va
                                                                        : zero4;
      const float4 im = (M::kMask & (1u << kImg)) ? centre(kImg) : zero4;

      const unsigned char *box_a = ost;
      const unsigned char *box_b = box_a + (M::kBoxA ? T::kBoxBytes : 0);
      const int ez = min(zo - 4, n3 - 4 - zo);

      // pending source injection owed to the previous level of s (adjoint)
      if (MODE == kModeAdjoint && PB && p.pb.active && valid && ok)
        inject_row(p.pb, n1, n2, zo, gy, gx, ob);

      float4 na = oa, nb = ob, ga = zero4, sb = zero4, ca = zero4, cb = zero4;
      if constexpr (FUSED) {
        if (M::kBoxA) {
          ga = stencil4_lp<BX, ST>(box_a, brow, bcol, qa, p.c, ca);
          if constexpr (LP) {
            ga = scale4(ga, s_sc.cur_a);
            ca = scale4(ca, s_sc.cur_a);
          }
        }
        if (M::kBoxB) {
          sb = stencil4_lp<BX, ST>(box_b, brow, bcol, qb, p.c, cb);
          if constexpr (LP) {
            sb = scale4(sb, s_sc.cur_b);
            cb = scale4(cb, s_sc.cur_b);
          }
        }
      } else {
        if (M::kBoxA)
          ga = stencil4<BX>(reinterpret_cast<const float *>(box_a), brow,
                            bcol, qa, p.c, ca);
        if (M::kBoxB)
          sb = stencil4<BX>(reinterpret_cast<const float *>(box_b), brow,
                            bcol, qb, p.c, cb);
      }
      const float bz = ez < kNBound ? s_bound[ez] : 1.0f;  // ez >= 0 here
      float bj[4];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) bj[jj] = fminf(bxy[jj], bz);
      // leapfrog and taper per pair of cells (x, x+1), (x+2, x+3); each lane
      // rounds as the scalar operation of cpu_prop.cc:233-248 and
      // cpu_prop.cc:150-160 does.  Products are scalar in the reference
      // order (a packed product feeding a packed add would be contracted).
      auto mulx = [](f32x2 a, f32x2 b) {
        if constexpr (FUSED) return mul2(a, b);
        else return mul2s(a, b);
      };
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const f32x2 b = pk2(bj[2 * h], bj[2 * h + 1]);
        if (M::kBoxA) {
          f32x2 old = cells2(oa, h);
          if (M::kDampA) old = mulx(old, b);
          const f32x2 c = cells2(ca, h);
          f32x2 v = FUSED ? fma2(cells2(va, h), cells2(ga, h),
                                 sub2(add2(c, c), old))
                          : leapfrog2(cells2(va, h), cells2(ga, h), c, old);
          // the adjoint of the linearised step injects its data before the
          // taper (see below); every other tapered mode tapers here
          if (MODE != kModeBornAdj && M::kDampA) v = mulx(v, b);
          set_cells2(na, h, v);
        } else if (MODE == kModeAdjoint) {
          // receiver level not propagated (it == 0): both damping passes
          set_cells2(na, h, mulx(mulx(cells2(oa, h), b), b));
        }
        if (M::kBoxB) {
          f32x2 old = cells2(ob, h);
          if (M::kDampB) old = mulx(old, b);
          const f32x2 c = cells2(cb, h);
          f32x2 v = FUSED ? fma2(cells2(vb, h), cells2(sb, h),
                                 sub2(add2(c, c), old))
                          : leapfrog2(cells2(vb, h), cells2(sb, h), c, old);
          // linearised Born: scattering source m (A s) inside the taper
          if (MODE == kModeBornLin)
            v = add2(v, mulx(cells2(im, h), cells2(ga, h)));
          if (M::kDampB) v = mulx(v, b);
          set_cells2(nb, h, v);
        }
      }

      // stores a level of field A or B (scaled and tracked with 16-bit
      // storage)
      auto store_a = [&](const float4 &v) {
        if constexpr (LP) {
          mx_a = absmax4(v, mx_a);
          st4_level<ST>(p.a_out, idx, scale4(v, s_sc.inv_new_a));
        } else {
          st4_level<ST>(p.a_out, idx, v);
        }
      };
      auto store_b = [&](const float4 &v) {
        if constexpr (LP) {
          mx_b = absmax4(v, mx_b);
          st4_level<ST>(p.b_out, idx, scale4(v, s_sc.inv_new_b));
        } else {
          st4_level<ST>(p.b_out, idx, v);
        }
      };

      if (valid && ok) {
        if (MODE == kModeBornAdj) {
          // w = b (v A w + 2w - b w_old + v E^T d); image += (A s) w
          float4 inj = zero4;
          if (p.pa.active) inject_row(p.pa, n1, n2, zo, gy, gx, inj);
          float4 ni;
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const float w = __fmul_rn(
                __fadd_rn(comp(na, jj), __fmul_rn(comp(va, jj), comp(inj, jj))),
                bj[jj]);
            set_comp(na, jj, w);
            set_comp(ni, jj, __fadd_rn(comp(im, jj), __fmul_rn(comp(ob, jj), w)));
          }
          st4(p.img_out + idx, ni);
          store_a(na);
        } else {
          if (p.pa.active) inject_row(p.pa, n1, n2, zo, gy, gx, na);
          if (MODE == kModeForward) {
            // Born coupling r += 1e-6 s img, then extraction from r
            if constexpr (Store<ST>::kExact) {
              // float evaluation of every cell (two packed pairs), the
              // double expression out of line for the few the rounding
              // test cannot decide
              unsigned int f0, f1;
              const float2 c0 = couple::couple_fast2(
                  make_float2(nb.x, nb.y), make_float2(na.x, na.y),
                  make_float2(im.x, im.y), &f0);
              const float2 c1 = couple::couple_fast2(
                  make_float2(nb.z, nb.w), make_float2(na.z, na.w),
                  make_float2(im.z, im.w), &f1);
              float4 nr = make_float4(c0.x, c0.y, c1.x, c1.y);
              const unsigned int slow = f0 | (f1 << 2);
              if (slow) {
                for (int jj = 0; jj < 4; ++jj)
                  if (slow & (1u << jj))
                    set_comp(nr, jj, couple::couple_slow(comp(nb, jj),
                                                         comp(na, jj),
                                                         comp(im, jj)));
              }
              nb = nr;
            } else {
#pragma unroll
              for (int h = 0; h < 2; ++h)
                set_cells2(nb, h,
                          add2(cells2(nb, h),
                               mulx(mulx(pk2(1e-6f, 1e-6f), cells2(na, h)),
                                    cells2(im, h))));
            }
          }
          if (MODE == kModeForward || MODE == kModeBornLin) {
            if (p.pb.active) extract_row(p.pb, n1, n2, zo, gy, gx, nb);
            store_a(na);
            store_b(nb);
          } else if (MODE == kModeAdjoint) {
            // s is the new level when propagated, else the stored one
            float4 ni;
#pragma unroll
            for (int h = 0; h < 2; ++h)
              set_cells2(ni, h, add2(cells2(im, h),
                                    mulx(cells2(nb, h), cells2(na, h))));
            st4(p.img_out + idx, ni);
            store_a(na);
            if (PB) store_b(nb);
          } else {  // source, model
            if (MODE == kModeModel) {
              if (p.pb.active) extract_row(p.pb, n1, n2, zo, gy, gx, na);
              if (p.g_out) st4(p.g_out + idx, ga);
            }
            store_a(na);
          }
        }
      }
    }
    if (!ok) {
      abort_flag = 1;
      atomicOr(p.err, kErrWaitTimeout);
    }

    __syncthreads();
    if (abort_flag) break;
    if (tid == 0) {
      fence_proxy_async();
      if (NF > 0 && k + LY::kZSt < K) issue_z(k + LY::kZSt);
      if (j >= 0 && j + LY::kOSt < J) issue_out(j + LY::kOSt);
    }
  }

  if (abort_flag && tid == 0) {
    // wait (bounded) for the last copy issued into each ring stage before
    // the CTA retires; thread 0 is the only issuer, so the counts are final
    for (int s = 0; s < LY::kZSt + LY::kOSt; ++s) {
      uint64_t *b = s < LY::kZSt ? &zbars[s] : &obars[s - LY::kZSt];
      const unsigned int n = s < LY::kZSt ? s_nz[s] : s_no[s - LY::kZSt];
      if (n == 0u) continue;
      const uint64_t t0 = global_ns();
      while (!mbar_try_wait(b, (n - 1u) & 1u) &&
             global_ns() - t0 < 100000000ull) {
      }
    }
  }

  if constexpr (LP) {
    // the level maxima: warp, then CTA, then one tagged atomic per CTA
    const unsigned int wa = __reduce_max_sync(0xffffffffu, __float_as_uint(mx_a));
    const unsigned int wb = __reduce_max_sync(0xffffffffu, __float_as_uint(mx_b));
    if ((tid & 31) == 0) {
      atomicMax(&s_mx[0], wa);
      atomicMax(&s_mx[1], wb);
    }
    __syncthreads();
    if (tid == 0 && !abort_flag) {
      if (p.la.out >= 0)
        atomicMax(&p.lv[2 * p.la.out],
                  ((unsigned long long)p.la.tag << 32) | s_mx[0]);
      if (M::kTwoField && PB && p.lb.out >= 0)
        atomicMax(&p.lv[2 * p.lb.out],
                  ((unsigned long long)p.lb.tag << 32) | s_mx[1]);
    }
  }
}

template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
__global__ void __launch_bounds__(Tile<TX, TY, 4>::kThreads)
    step_kernel(const __grid_constant__ StepMaps maps, const StepParams p) {
  step_body<ST, MODE, PA, PB, TX, TY>(&maps, p, blockIdx.x, blockIdx.y);
}

// Batched launch: blockIdx.x enumerates the CTAs of every shot in turn
// (block_start[s] .. block_start[s+1]-1 belong to shot s); each shot brings
// its own grid, buffers, point sets and TMA descriptors (one set per level
// parity), the step-varying scalars come in `var`.
template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
__global__ void __launch_bounds__(Tile<TX, TY, 4>::kThreads)
    step_kernel_batched(const BatchShot *shots, const int *block_start,
                        int nshots, const StepVar var) {
  __shared__ __align__(16) StepParams sp;
  static_assert(sizeof(StepParams) % 4 == 0, "word-wise copy");
  // every thread finds the shot (same addresses: broadcast loads) and the
  // CTA copies the shot's parameters word by word
  int lo = 0, hi = nshots - 1;  // last shot whose start <= blockIdx.x
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (block_start[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const int shot = lo, local = (int)blockIdx.x - block_start[lo];
  {
    const unsigned int *src =
        reinterpret_cast<const unsigned int *>(&shots[shot].params);
    unsigned int *dst = reinterpret_cast<unsigned int *>(&sp);
    for (int i = threadIdx.x; i < (int)(sizeof(StepParams) / 4);
         i += blockDim.x)
      dst[i] = src[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const BatchShot &b = shots[shot];
    sp.a_out = b.a_out[var.parity];
    sp.b_out = b.b_out[var.parity];
    sp.pa.id = var.pa_id;
    sp.pa.active = var.pa_active && sp.pa.npts > 0;
    sp.pa.scale = var.pa_scale;
    sp.pb.id = var.pb_id;
    sp.pb.active = var.pb_active && sp.pb.npts > 0;
    sp.pb.scale = var.pb_scale;
    for (int k = 0; k < 8; ++k) {
      sp.pa.tab[k] = var.pa_tab[k];
      sp.pb.tab[k] = var.pb_tab[k];
    }
    sp.la = var.la;
    sp.lb = var.lb;
  }
  __syncthreads();
  const BatchShot &b = shots[shot];
  const int ntiles = sp.tiles_x * sp.tiles_y;
  step_body<ST, MODE, PA, PB, TX, TY>(&b.maps[var.parity], sp, local % ntiles,
                                      local / ntiles);
}

// ---------------------------------------------------------------------------
// Host side: launches and dispatch for one storage type

struct TileCfg {
  int tx, ty;
};
// (24x16 and 40x16 tiles, which divide a 360-cell interior exactly, ran
// slower than 64x8 in every loop on a 368^3 grid: forward 0.339 and 0.314
// ms per launch against 0.266, adjoint 0.380 and 0.371 against 0.314)
constexpr TileCfg kTileCfgs[] = {{64, 16}, {32, 16}, {32, 32}, {64, 8},
                                 {32, 8}};
constexpr int kNumTileCfgs = sizeof(kTileCfgs) / sizeof(kTileCfgs[0]);

// The dynamic shared-memory limit of a kernel is an attribute of the
// current device: set it once per device (bit d of `done`; devices beyond
// 63 set it on every launch).
template <class K>
cudaError_t configure_smem(K kern, size_t smem,
                           std::atomic<unsigned long long> &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_relaxed) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_relaxed);
  return e;
}

template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
cudaError_t launch_t(const StepMaps &maps, const StepParams &p,
                     cudaStream_t stream) {
  using T = Tile<TX, TY, 4>;
  const size_t smem = Layout<ST, MODE, PA, PB, TX, TY>::kSmem;
  auto kern = step_kernel<ST, MODE, PA, PB, TX, TY>;
  static std::atomic<unsigned long long> configured{0};
  cudaError_t e = configure_smem(kern, smem, configured);
  if (e != cudaSuccess) return e;
  const int nseg = (p.n3 - 2 * kRadius + p.zseg - 1) / p.zseg;
  dim3 grid(p.tiles_x * p.tiles_y, nseg);
  if (p.overlap) {
    // the grid's CTAs may become resident while the previous step's last
    // CTAs finish; the kernel waits for that grid before reading anything
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(T::kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, maps, p);
  }
  kern<<<grid, T::kThreads, smem, stream>>>(maps, p);
  return cudaGetLastError();
}

template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
cudaError_t launch_t_batched(const BatchShot *shots, const int *block_start,
                             int nshots, int total, const StepVar &var,
                             cudaStream_t stream) {
  using T = Tile<TX, TY, 4>;
  const size_t smem = Layout<ST, MODE, PA, PB, TX, TY>::kSmem;
  auto kern = step_kernel_batched<ST, MODE, PA, PB, TX, TY>;
  static std::atomic<unsigned long long> configured{0};
  cudaError_t e = configure_smem(kern, smem, configured);
  if (e != cudaSuccess) return e;
  if (total == 0) return cudaSuccess;  // configuration only
  kern<<<total, T::kThreads, smem, stream>>>(shots, block_start, nshots, var);
  return cudaGetLastError();
}

// Dispatch over (mode, pa, pb) for one tile shape; F::go is instantiated
// for every variant (FP32 storage: every mode; 16-bit and fused FP32:
// source, forward and adjoint; exact coupling: the forward step).
template <int ST, int TX, int TY, class F>
auto dispatch(int mode, bool pa, bool pb, F f) {
  if constexpr (ST == kStoreF32Exact) {
    // the only step with a Born coupling; the other steps of this storage
    // are the FP32 ones
    (void)mode;
    (void)pa;
    (void)pb;
    return f.template go<ST, kModeForward, true, true, TX, TY>();
  } else {
    if constexpr (ST == kStoreF32) {
      switch (mode) {
        case kModeModel:
          return f.template go<ST, kModeModel, true, false, TX, TY>();
        case kModeBornLin:
          return f.template go<ST, kModeBornLin, true, true, TX, TY>();
        case kModeBornAdj:
          return f.template go<ST, kModeBornAdj, true, false, TX, TY>();
        default: break;
      }
    }
    switch (mode) {
      case kModeSource:
        return f.template go<ST, kModeSource, true, false, TX, TY>();
      case kModeForward:
        return f.template go<ST, kModeForward, true, true, TX, TY>();
      default:
        if (pa && pb)
          return f.template go<ST, kModeAdjoint, true, true, TX, TY>();
        if (pa) return f.template go<ST, kModeAdjoint, true, false, TX, TY>();
        if (pb) return f.template go<ST, kModeAdjoint, false, true, TX, TY>();
        return f.template go<ST, kModeAdjoint, false, false, TX, TY>();
    }
  }
}

template <int ST, class F>
auto dispatch_cfg(int cfg, int mode, bool pa, bool pb, F f) {
  switch (cfg) {
    case 1: return dispatch<ST, 32, 16>(mode, pa, pb, f);
    case 2: return dispatch<ST, 32, 32>(mode, pa, pb, f);
    case 3: return dispatch<ST, 64, 8>(mode, pa, pb, f);
    case 4: return dispatch<ST, 32, 8>(mode, pa, pb, f);
    default: return dispatch<ST, 64, 16>(mode, pa, pb, f);
  }
}

struct LaunchF {
  const StepMaps &maps;
  const StepParams &p;
  cudaStream_t s;
  template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
  cudaError_t go() const {
    return launch_t<ST, MODE, PA, PB, TX, TY>(maps, p, s);
  }
};

struct LaunchBatchedF {
  const BatchShot *shots;
  const int *block_start;
  int nshots, total;
  const StepVar &var;
  cudaStream_t s;
  template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
  cudaError_t go() const {
    return launch_t_batched<ST, MODE, PA, PB, TX, TY>(shots, block_start,
                                                      nshots, total, var, s);
  }
};

struct SmemF {
  template <int ST, int MODE, bool PA, bool PB, int TX, int TY>
  size_t go() const {
    return Layout<ST, MODE, PA, PB, TX, TY>::kSmem;
  }
};

}  // namespace

// Per-storage entry points, defined by the translation unit that owns the
// storage type (born_step.cu, born_step_bf16.cu, born_step_f16.cu,
// born_step_f32fused.cu).
#define BORN_DECLARE_STORAGE_ENTRY(NAME)                                     \
  cudaError_t launch_step_##NAME(int mode, bool pa, bool pb, int cfg,        \
                                 const StepMaps &maps, const StepParams &p,  \
                                 cudaStream_t s);                            \
  cudaError_t launch_step_batched_##NAME(                                    \
      int mode, bool pa, bool pb, int cfg, const BatchShot *shots,           \
      const int *block_start, int nshots, int total, const StepVar &var,     \
      cudaStream_t s);                                                       \
  size_t step_smem_##NAME(int cfg, int mode, bool pa, bool pb);

BORN_DECLARE_STORAGE_ENTRY(f32)
BORN_DECLARE_STORAGE_ENTRY(bf16)
BORN_DECLARE_STORAGE_ENTRY(f16)
BORN_DECLARE_STORAGE_ENTRY(f32fused)
BORN_DECLARE_STORAGE_ENTRY(f32exact)

#define BORN_DEFINE_STORAGE_ENTRY(ST, NAME)                                  \
  cudaError_t launch_step_##NAME(int mode, bool pa, bool pb, int cfg,        \
                                 const StepMaps &maps, const StepParams &p,  \
                                 cudaStream_t s) {                           \
    return dispatch_cfg<ST>(cfg, mode, pa, pb, LaunchF{maps, p, s});         \
  }                                                                          \
  cudaError_t launch_step_batched_##NAME(                                    \
      int mode, bool pa, bool pb, int cfg, const BatchShot *shots,           \
      const int *block_start, int nshots, int total, const StepVar &var,     \
      cudaStream_t s) {                                                      \
    return dispatch_cfg<ST>(                                                 \
        cfg, mode, pa, pb,                                                   \
        LaunchBatchedF{shots, block_start, nshots, total, var, s});          \
  }                                                                          \
  size_t step_smem_##NAME(int cfg, int mode, bool pa, bool pb) {             \
    return dispatch_cfg<ST>(cfg, mode, pa, pb, SmemF{});                     \
  }

}  // namespace born
