// Fused 2.5D time-step kernels (see born_step.cuh for the design).
#include <algorithm>

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

__device__ __forceinline__ void tma_load_3d(float *dst, const CUtensorMap *tm,
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

// Stencil sums of this thread's 4 consecutive cells (x .. x+3) of one row,
// from a TMA box (x/y neighbours) and the register z window.  Each cell's
// sum is formed in the reference order of cpuProp::prop (cpu_prop.cc:235-247):
// C0 p, then the x pairs, the y pairs and the z pairs, every product and sum
// separately rounded; the four cells advance together so that every shared
// load is a float4 (3 for the x window, 2 per y offset).
template <int BX>
__device__ __forceinline__ float4 stencil4(const float *box, int brow,
                                           int bcol, const float4 (&q)[9],
                                           const float *c, float4 &center) {
  const float *r = box + brow * BX + bcol;
  float w[12];
  {
    const float4 L = *reinterpret_cast<const float4 *>(r - 4);
    const float4 M = *reinterpret_cast<const float4 *>(r);
    const float4 R = *reinterpret_cast<const float4 *>(r + 4);
    w[0] = L.x; w[1] = L.y; w[2] = L.z; w[3] = L.w;
    w[4] = M.x; w[5] = M.y; w[6] = M.z; w[7] = M.w;
    w[8] = R.x; w[9] = R.y; w[10] = R.z; w[11] = R.w;
    center = M;
  }
  float s[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    s[j] = __fmul_rn(c[0], w[4 + j]);
    s[j] = __fadd_rn(s[j], __fmul_rn(c[2], __fadd_rn(w[3 + j], w[5 + j])));
    s[j] = __fadd_rn(s[j], __fmul_rn(c[5], __fadd_rn(w[2 + j], w[6 + j])));
    s[j] = __fadd_rn(s[j], __fmul_rn(c[8], __fadd_rn(w[1 + j], w[7 + j])));
    s[j] = __fadd_rn(s[j], __fmul_rn(c[11], __fadd_rn(w[0 + j], w[8 + j])));
  }
  const int cy[4] = {3, 6, 9, 12}, cz[4] = {1, 4, 7, 10};
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    const float4 u = *reinterpret_cast<const float4 *>(r - m * BX);
    const float4 d = *reinterpret_cast<const float4 *>(r + m * BX);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      s[j] = __fadd_rn(s[j], __fmul_rn(c[cy[m - 1]],
                                       __fadd_rn(comp(u, j), comp(d, j))));
  }
#pragma unroll
  for (int m = 1; m <= 4; ++m)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      s[j] = __fadd_rn(
          s[j], __fmul_rn(c[cz[m - 1]],
                          __fadd_rn(comp(q[4 - m], j), comp(q[4 + m], j))));
  return make_float4(s[0], s[1], s[2], s[3]);
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
  static constexpr int kNC = __builtin_popcount(kMask);
  // tile index of a slot inside a centre stage
  __host__ __device__ static constexpr int pos(int slot) {
    return __builtin_popcount(kMask & ((1u << slot) - 1u));
  }
  static constexpr bool kDampA = MODE != kModeSource;
  static constexpr bool kDampB = MODE == kModeForward || MODE == kModeBornLin;
};

template <int TX, int TY>
struct Tile {
  static constexpr int kBX = TX + 2 * kRadius, kBY = TY + 2 * kRadius;
  static constexpr int kBoxFloats = kBX * kBY;
  static constexpr int kBoxPitch = ((kBoxFloats * 4 + 127) / 128) * 32;
  static constexpr int kCFloats = TX * TY;
  static constexpr int kThreads = (TX / 4) * TY;
};

template <int MODE, bool PA, bool PB, int TX, int TY>
__global__ void __launch_bounds__(Tile<TX, TY>::kThreads)
    step_kernel(const __grid_constant__ StepMaps maps, const StepParams p) {
  using M = ModeTraits<MODE, PA, PB>;
  using T = Tile<TX, TY>;
  constexpr int NF = M::kNF, NC = M::kNC;
  constexpr int BX = T::kBX, PITCH = T::kBoxPitch, CF = T::kCFloats;
  constexpr uint32_t kBoxBytes = T::kBoxFloats * 4u;
  constexpr uint32_t kCBytes = T::kCFloats * 4u;
  extern __shared__ __align__(128) float smem_raw[];
  __shared__ __align__(8) uint64_t zbars[kZStages];
  __shared__ __align__(8) uint64_t obars[kOStages];
  __shared__ int abort_flag;
  __shared__ float s_bound[kNBound];
  // TMA destinations need 128-byte alignment: align the dynamic base here
  // (the launch reserves 128 spare bytes for this)
  float *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u) / 4u;
  // z ring: centre tiles of the current levels, one per new plane
  float *zring = smem;
  // output ring: halo boxes and per-cell inputs of the output plane
  constexpr int OSTRIDE = NF * PITCH + NC * CF;
  float *oring = smem + kZStages * NF * CF;

  const int tid = threadIdx.x;
  const int lx = tid % (TX / 4), ly = tid / (TX / 4);
  const int tile = blockIdx.x;
  const int tx = tile % p.tiles_x, ty = tile / p.tiles_x;
  const int x0 = kRadius + tx * TX, y0 = kRadius + ty * TY;
  const int z0 = kRadius + blockIdx.y * p.zseg;
  const int z1 = min(z0 + p.zseg, p.n3 - kRadius);
  if (z0 >= z1) return;  // uniform over the CTA
  const int n1 = p.n1, n2 = p.n2, n3 = p.n3;
  const long long n12 = (long long)n1 * n2;
  const int gx = x0 + 4 * lx, gy = y0 + ly;
  const bool valid = (gx < n1 - kRadius) && (gy < n2 - kRadius);

  // taper: distance to the interior faces in x/y per cell (cpu_prop.cc:146-151)
  int exy[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int x = gx + j;
    exy[j] = min(min(x - 4, n1 - 4 - x), min(gy - 4, n2 - 4 - gy));
  }

  if (tid == 0) {
    for (int s = 0; s < kZStages; ++s) mbar_init(&zbars[s], 1);
    for (int s = 0; s < kOStages; ++s) mbar_init(&obars[s], 1);
    // a wait elsewhere already gave up: the whole CTA leaves untouched
    abort_flag = *reinterpret_cast<volatile unsigned int *>(p.err) != 0u;
    mbar_fence_init();
  }
  if (tid < kNBound) s_bound[tid] = p.bound[tid];
  __syncthreads();
  if (abort_flag) return;  // uniform: read after the barrier

  const int K = (z1 - z0) + 2 * kRadius;  // z-window planes z0-4 .. z1+3
  const int J = z1 - z0;                  // output planes
  auto issue_z = [&](int k) {
    const int plane = z0 - kRadius + k;
    const int st = k % kZStages;
    mbar_expect_tx(&zbars[st], NF * kCBytes);
    float *dst = zring + st * NF * CF;
    if (M::kBoxA) tma_load_3d(dst, &maps.zc_a, x0, y0, plane, &zbars[st]);
    if (M::kBoxB)
      tma_load_3d(dst + (M::kBoxA ? CF : 0), &maps.zc_b, x0, y0, plane,
                  &zbars[st]);
  };
  auto issue_out = [&](int j) {
    const int plane = z0 + j;
    const int st = j % kOStages;
    mbar_expect_tx(&obars[st], NF * kBoxBytes + NC * kCBytes);
    float *dst = oring + st * OSTRIDE;
    if (M::kBoxA)
      tma_load_3d(dst, &maps.box_a, x0 - kRadius, y0 - kRadius, plane,
                  &obars[st]);
    if (M::kBoxB)
      tma_load_3d(dst + (M::kBoxA ? PITCH : 0), &maps.box_b, x0 - kRadius,
                  y0 - kRadius, plane, &obars[st]);
    float *cdst = dst + NF * PITCH;
#pragma unroll
    for (int s = 0; s < kNumCentre; ++s)
      if (M::kMask & (1u << s))
        tma_load_3d(cdst + M::pos(s) * CF, &maps.cm[s], x0, y0, plane,
                    &obars[st]);
  };
  if (tid == 0) {
    if (NF > 0)
      for (int k = 0; k < min(K, kZStages); ++k) issue_z(k);
    for (int j = 0; j < min(J, kOStages); ++j) issue_out(j);
  }

  float4 qa[9], qb[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    qa[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    qb[i] = qa[i];
  }
  const int brow = ly + kRadius, bcol = 4 * lx + kRadius;
  const int coff = ly * TX + 4 * lx;  // this thread's float4 in a centre tile

  for (int k = 0; k < K; ++k) {
    const int st = k % kZStages;
    const int j = k - 2 * kRadius;       // output index once k >= 8
    const int zo = z0 + j;
    const long long idx = (long long)zo * n12 + (long long)gy * n1 + gx;

    bool ok = true;
    if (NF > 0) {
      ok = mbar_wait_bounded(&zbars[st], (uint32_t)((k / kZStages) & 1));
      // newest plane's centre enters the z window
      const float *sa = zring + st * NF * CF + coff;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        qa[i] = qa[i + 1];
        qb[i] = qb[i + 1];
      }
      if (M::kBoxA) qa[8] = *reinterpret_cast<const float4 *>(sa);
      if (M::kBoxB)
        qb[8] = *reinterpret_cast<const float4 *>(sa + (M::kBoxA ? CF : 0));
    }

    if (j >= 0 && ok) {
      const int os = j % kOStages;
      ok = mbar_wait_bounded(&obars[os], (uint32_t)((j / kOStages) & 1));
      const float *ost = oring + os * OSTRIDE;
      const float *cst = ost + NF * PITCH + coff;
      auto centre = [&](int slot) {
        return *reinterpret_cast<const float4 *>(cst + M::pos(slot) * CF);
      };
      const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 oa = (M::kMask & (1u << kOldA)) ? centre(kOldA) : zero4;
      float4 ob = (M::kMask & (1u << kOldB)) ? centre(kOldB) : zero4;
      const float4 va = (M::kMask & (1u << kVelA)) ? centre(kVelA) : zero4;
      const float4 vb = (M::kMask & (1u << kVelB)) ? centre(kVelB)
                        : (MODE == kModeForward || MODE == kModeBornLin) ? va
                                                                        : zero4;
      const float4 im = (M::kMask & (1u << kImg)) ? centre(kImg) : zero4;

      const float *box_a = ost;
      const float *box_b = box_a + (M::kBoxA ? PITCH : 0);
      const int ez = min(zo - 4, n3 - 4 - zo);

      // pending source injection owed to the previous level of s (adjoint)
      if (MODE == kModeAdjoint && PB && p.pb.active && valid && ok)
        inject_row(p.pb, n1, n2, zo, gy, gx, ob);

      float4 na = oa, nb = ob, ga = zero4, sb = zero4, ca = zero4, cb = zero4;
      if (M::kBoxA) ga = stencil4<BX>(box_a, brow, bcol, qa, p.c, ca);
      if (M::kBoxB) sb = stencil4<BX>(box_b, brow, bcol, qb, p.c, cb);
      float bj[4];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int e = min(exy[jj], ez);
        const float b = (e >= 0 && e < kNBound) ? s_bound[e] : 1.0f;
        bj[jj] = b;
        if (M::kBoxA) {
          float old = comp(oa, jj);
          if (M::kDampA) old = __fmul_rn(old, b);
          float v = leapfrog(comp(va, jj), comp(ga, jj), comp(ca, jj), old);
          // the adjoint of the linearised step injects its data before the
          // taper (see below); every other tapered mode tapers here
          if (MODE != kModeBornAdj && M::kDampA) v = __fmul_rn(v, b);
          set_comp(na, jj, v);
        } else if (MODE == kModeAdjoint) {
          // receiver level not propagated (it == 0): both damping passes
          set_comp(na, jj, __fmul_rn(__fmul_rn(comp(oa, jj), b), b));
        }
        if (M::kBoxB) {
          float old = comp(ob, jj);
          if (M::kDampB) old = __fmul_rn(old, b);
          float v = leapfrog(comp(vb, jj), comp(sb, jj), comp(cb, jj), old);
          // linearised Born: scattering source m (A s) inside the taper
          if (MODE == kModeBornLin)
            v = __fadd_rn(v, __fmul_rn(comp(im, jj), comp(ga, jj)));
          if (M::kDampB) v = __fmul_rn(v, b);
          set_comp(nb, jj, v);
        }
      }

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
          st4(p.a_out + idx, na);
        } else {
          if (p.pa.active) inject_row(p.pa, n1, n2, zo, gy, gx, na);
          if (MODE == kModeForward) {
            // Born coupling r += 1e-6 s img, then extraction from r
#pragma unroll
            for (int jj = 0; jj < 4; ++jj)
              set_comp(nb, jj,
                       __fadd_rn(comp(nb, jj),
                                 __fmul_rn(__fmul_rn(1e-6f, comp(na, jj)),
                                           comp(im, jj))));
          }
          if (MODE == kModeForward || MODE == kModeBornLin) {
            if (p.pb.active) extract_row(p.pb, n1, n2, zo, gy, gx, nb);
            st4(p.a_out + idx, na);
            st4(p.b_out + idx, nb);
          } else if (MODE == kModeAdjoint) {
            // s is the new level when propagated, else the stored one
            float4 ni;
            ni.x = __fadd_rn(im.x, __fmul_rn(nb.x, na.x));
            ni.y = __fadd_rn(im.y, __fmul_rn(nb.y, na.y));
            ni.z = __fadd_rn(im.z, __fmul_rn(nb.z, na.z));
            ni.w = __fadd_rn(im.w, __fmul_rn(nb.w, na.w));
            st4(p.img_out + idx, ni);
            st4(p.a_out + idx, na);
            if (PB) st4(p.b_out + idx, nb);
          } else {  // source, model
            if (MODE == kModeModel) {
              if (p.pb.active) extract_row(p.pb, n1, n2, zo, gy, gx, na);
              if (p.g_out) st4(p.g_out + idx, ga);
            }
            st4(p.a_out + idx, na);
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
      if (NF > 0 && k + kZStages < K) issue_z(k + kZStages);
      if (j >= 0 && j + kOStages < J) issue_out(j + kOStages);
    }
  }

  if (abort_flag && tid == 0) {
    // drain whatever is still in flight (bounded) before the CTA retires
    for (int s = 0; s < kZStages + kOStages; ++s) {
      uint64_t *b = s < kZStages ? &zbars[s] : &obars[s - kZStages];
      const uint64_t t0 = global_ns();
      while (!mbar_try_wait(b, 0) && !mbar_try_wait(b, 1) &&
             global_ns() - t0 < 100000000ull) {
      }
    }
  }
}

__global__ void point_inject_kernel(const PointSet ps, int npts,
                                    float *field) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || !ps.active) return;
  for (int s = 0; s < npts; ++s)
    field[ps.slot_cell[s]] =
        __fadd_rn(field[ps.slot_cell[s]], point_value(ps, ps.slot_index[s]));
}

__global__ void divide_kernel(const float *a, const float *v, float *out,
                              long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = v[i] != 0.f ? __fdiv_rn(a[i], v[i]) : 0.f;
}

// ---------------------------------------------------------------------------
struct TileCfg {
  int tx, ty;
};
constexpr TileCfg kTileCfgs[] = {{64, 16}, {32, 16}, {32, 32}, {64, 8},
                                 {32, 8}};
constexpr int kNumTileCfgs = sizeof(kTileCfgs) / sizeof(kTileCfgs[0]);

template <int MODE, bool PA, bool PB, int TX, int TY>
size_t smem_bytes_t() {
  using M = ModeTraits<MODE, PA, PB>;
  using T = Tile<TX, TY>;
  return (size_t)kZStages * M::kNF * T::kCFloats * 4 +
         (size_t)kOStages * (M::kNF * T::kBoxPitch + M::kNC * T::kCFloats) * 4 +
         128;
}

template <int MODE, bool PA, bool PB, int TX, int TY>
cudaError_t launch_t(const StepMaps &maps, const StepParams &p,
                     cudaStream_t stream) {
  using T = Tile<TX, TY>;
  const size_t smem = smem_bytes_t<MODE, PA, PB, TX, TY>();
  auto kern = step_kernel<MODE, PA, PB, TX, TY>;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int nseg = (p.n3 - 2 * kRadius + p.zseg - 1) / p.zseg;
  dim3 grid(p.tiles_x * p.tiles_y, nseg);
  kern<<<grid, T::kThreads, smem, stream>>>(maps, p);
  return cudaGetLastError();
}

// Dispatch over (mode, pa, pb) for one tile shape; F::go is instantiated
// for every variant.
template <int TX, int TY, class F>
auto dispatch(int mode, bool pa, bool pb, F f) {
  switch (mode) {
    case kModeSource: return f.template go<kModeSource, true, false, TX, TY>();
    case kModeForward: return f.template go<kModeForward, true, true, TX, TY>();
    case kModeModel: return f.template go<kModeModel, true, false, TX, TY>();
    case kModeBornLin: return f.template go<kModeBornLin, true, true, TX, TY>();
    case kModeBornAdj: return f.template go<kModeBornAdj, true, false, TX, TY>();
    default:
      if (pa && pb) return f.template go<kModeAdjoint, true, true, TX, TY>();
      if (pa) return f.template go<kModeAdjoint, true, false, TX, TY>();
      if (pb) return f.template go<kModeAdjoint, false, true, TX, TY>();
      return f.template go<kModeAdjoint, false, false, TX, TY>();
  }
}

struct LaunchF {
  const StepMaps &maps;
  const StepParams &p;
  cudaStream_t s;
  template <int MODE, bool PA, bool PB, int TX, int TY>
  cudaError_t go() const {
    return launch_t<MODE, PA, PB, TX, TY>(maps, p, s);
  }
};

struct SmemF {
  template <int MODE, bool PA, bool PB, int TX, int TY>
  size_t go() const {
    return smem_bytes_t<MODE, PA, PB, TX, TY>();
  }
};

template <class F>
auto dispatch_cfg(int cfg, int mode, bool pa, bool pb, F f) {
  switch (cfg) {
    case 1: return dispatch<32, 16>(mode, pa, pb, f);
    case 2: return dispatch<32, 32>(mode, pa, pb, f);
    case 3: return dispatch<64, 8>(mode, pa, pb, f);
    case 4: return dispatch<32, 8>(mode, pa, pb, f);
    default: return dispatch<64, 16>(mode, pa, pb, f);
  }
}

}  // namespace

unsigned centre_mask(int mode, bool pa, bool pb) {
  switch (mode) {
    case kModeSource: return ModeTraits<kModeSource, true, false>::kMask;
    case kModeForward: return ModeTraits<kModeForward, true, true>::kMask;
    case kModeModel: return ModeTraits<kModeModel, true, false>::kMask;
    case kModeBornLin: return ModeTraits<kModeBornLin, true, true>::kMask;
    case kModeBornAdj: return ModeTraits<kModeBornAdj, true, false>::kMask;
    default:
      return (1u << kOldA) | (1u << kOldB) | (1u << kImg) |
             (pa ? (1u << kVelA) : 0u) | (pb ? (1u << kVelB) : 0u);
  }
}

int tile_cfg_count() { return kNumTileCfgs; }

void tile_cfg_dims(int cfg, int *tx, int *ty) {
  *tx = kTileCfgs[cfg].tx;
  *ty = kTileCfgs[cfg].ty;
}

size_t step_smem_bytes(int cfg, int mode, bool pa, bool pb) {
  return dispatch_cfg(cfg, mode, pa, pb, SmemF{});
}

cudaError_t launch_step(int mode, bool pa, bool pb, int cfg,
                        const StepMaps &maps, const StepParams &p,
                        cudaStream_t s) {
  if (mode < kModeSource || mode > kModeBornAdj) return cudaErrorInvalidValue;
  if (cfg < 0 || cfg >= kNumTileCfgs) return cudaErrorInvalidValue;
  return dispatch_cfg(cfg, mode, pa, pb, LaunchF{maps, p, s});
}

cudaError_t launch_point_inject(const PointSet &ps, int npts, float *field,
                                cudaStream_t stream) {
  point_inject_kernel<<<1, 32, 0, stream>>>(ps, npts, field);
  return cudaGetLastError();
}

cudaError_t launch_divide(const float *a, const float *v, float *out,
                          long long n, cudaStream_t stream) {
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
  divide_kernel<<<blocks, 256, 0, stream>>>(a, v, out, n);
  return cudaGetLastError();
}

}  // namespace born
