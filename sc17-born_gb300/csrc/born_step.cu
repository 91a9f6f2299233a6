// Fused 2.5D time-step kernels (see born_step.cuh for the design).
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

// Reference summation order of cpuProp::prop (cpu_prop.cc:233-248):
// ((((C0 p + CX1(..)) + CX2(..)) ... + CZ4(..)); v*S + p + p - old.
// Intrinsics keep every multiply and add separately rounded.
struct Nbr {
  float x[8], y[8], z[8];  // [m-1] for -m, [4+m-1] for +m
};

__device__ __forceinline__ float stencil_sum(const float *c, float p,
                                             const Nbr &n) {
  float s = __fmul_rn(c[0], p);
  s = __fadd_rn(s, __fmul_rn(c[2], __fadd_rn(n.x[0], n.x[4])));
  s = __fadd_rn(s, __fmul_rn(c[5], __fadd_rn(n.x[1], n.x[5])));
  s = __fadd_rn(s, __fmul_rn(c[8], __fadd_rn(n.x[2], n.x[6])));
  s = __fadd_rn(s, __fmul_rn(c[11], __fadd_rn(n.x[3], n.x[7])));
  s = __fadd_rn(s, __fmul_rn(c[3], __fadd_rn(n.y[0], n.y[4])));
  s = __fadd_rn(s, __fmul_rn(c[6], __fadd_rn(n.y[1], n.y[5])));
  s = __fadd_rn(s, __fmul_rn(c[9], __fadd_rn(n.y[2], n.y[6])));
  s = __fadd_rn(s, __fmul_rn(c[12], __fadd_rn(n.y[3], n.y[7])));
  s = __fadd_rn(s, __fmul_rn(c[1], __fadd_rn(n.z[0], n.z[4])));
  s = __fadd_rn(s, __fmul_rn(c[4], __fadd_rn(n.z[1], n.z[5])));
  s = __fadd_rn(s, __fmul_rn(c[7], __fadd_rn(n.z[2], n.z[6])));
  s = __fadd_rn(s, __fmul_rn(c[10], __fadd_rn(n.z[3], n.z[7])));
  return s;
}

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

__device__ __forceinline__ float4 ld4(const float *p) {
  return *reinterpret_cast<const float4 *>(p);
}
__device__ __forceinline__ float4 ldg4(const float *p) {
  return __ldg(reinterpret_cast<const float4 *>(p));
}
__device__ __forceinline__ void st4(float *p, const float4 &v) {
  *reinterpret_cast<float4 *>(p) = v;
}

// Gathers the x/y neighbours of cell j from a TMA box; z from the window.
template <int BX>
__device__ __forceinline__ void gather(const float *box, int brow, int bcol,
                                       const float4 (&q)[9], int j, Nbr &n,
                                       float &center) {
  const float *r = box + brow * BX + bcol;  // points at x (j = 0)
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    n.x[m - 1] = r[j - m];
    n.x[4 + m - 1] = r[j + m];
    n.y[m - 1] = r[j - m * BX];
    n.y[4 + m - 1] = r[j + m * BX];
    n.z[m - 1] = comp(q[4 - m], j);
    n.z[4 + m - 1] = comp(q[4 + m], j);
  }
  center = r[j];
}

// ---------------------------------------------------------------------------
template <int MODE, bool PA, bool PB, int TX, int TY>
__global__ void __launch_bounds__(TileShape<TX, TY>::kThreads)
    step_kernel(const __grid_constant__ CUtensorMap tm_a,
                const __grid_constant__ CUtensorMap tm_b,
                const StepParams p) {
  using T = TileShape<TX, TY>;
  constexpr int NF = (PA ? 1 : 0) + (PB ? 1 : 0);
  constexpr int BX = T::kBX;
  constexpr int PITCH = T::kBoxPitch;
  constexpr uint32_t kBoxBytes = T::kBoxFloats * 4u;
  extern __shared__ __align__(128) float smem_raw[];
  __shared__ __align__(8) uint64_t bars[kStages];
  __shared__ int abort_flag;
  __shared__ float s_bound[kNBound];
  // TMA destinations need 128-byte alignment: align the dynamic base here
  // (the launch reserves 128 spare bytes for this)
  float *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u) / 4u;


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
    const int ex = min(x - 4, n1 - 4 - x), ey = min(gy - 4, n2 - 4 - gy);
    exy[j] = min(ex, ey);
  }

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    // a wait elsewhere already gave up: the whole CTA leaves untouched
    abort_flag = *reinterpret_cast<volatile unsigned int *>(p.err) != 0u;
    mbar_fence_init();
  }
  if (tid < kNBound) s_bound[tid] = p.bound[tid];
  __syncthreads();
  if (abort_flag) return;  // uniform: read after the barrier

  const int K = (z1 - z0) + 2 * kRadius;  // planes z0-4 .. z1+3
  auto issue = [&](int k) {
    const int plane = z0 - kRadius + k;
    const int st = k % kStages;
    mbar_expect_tx(&bars[st], NF * kBoxBytes);
    float *dst = smem + st * NF * PITCH;
    if (PA) tma_load_3d(dst, &tm_a, x0 - kRadius, y0 - kRadius, plane, &bars[st]);
    if (PB)
      tma_load_3d(dst + (PA ? PITCH : 0), &tm_b, x0 - kRadius, y0 - kRadius,
                  plane, &bars[st]);
  };
  if (NF > 0 && tid == 0) {
    const int npro = K < kStages ? K : kStages;
    for (int k = 0; k < npro; ++k) issue(k);
  }

  float4 qa[9], qb[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    qa[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    qb[i] = qa[i];
  }
  const int brow = ly + kRadius, bcol = 4 * lx + kRadius;

  for (int k = 0; k < K; ++k) {
    const int st = k % kStages;
    const int zo = z0 + (k - 2 * kRadius);  // output plane once k >= 8
    const bool compute = k >= 2 * kRadius;
    const long long idx = (long long)zo * n12 + (long long)gy * n1 + gx;

    // centre loads for the output plane, issued before the barrier wait
    float4 oa = make_float4(0.f, 0.f, 0.f, 0.f), ob = oa, va = oa, vb = oa,
           im = oa;
    if (compute && valid) {
      oa = ld4(p.a_old + idx);
      if (PA || MODE == kModeSource) va = ldg4(p.a_vel + idx);
      if (MODE != kModeSource) {
        ob = ld4(p.b_old + idx);
        if (PB) vb = (MODE == kModeForward) ? va : ldg4(p.b_vel + idx);
        im = ld4(p.img + idx);
      }
    }

    bool ok = true;
    if (NF > 0) {
      ok = mbar_wait_bounded(&bars[st], (uint32_t)((k / kStages) & 1));
      if (!ok) {
        abort_flag = 1;
        atomicOr(p.err, kErrWaitTimeout);
      }
    }
    // newest plane's centre enters the z window
    {
      const float *sa = smem + st * NF * PITCH;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        qa[i] = qa[i + 1];
        qb[i] = qb[i + 1];
      }
      if (PA) qa[8] = *reinterpret_cast<const float4 *>(sa + brow * BX + bcol);
      if (PB)
        qb[8] = *reinterpret_cast<const float4 *>(sa + (PA ? PITCH : 0) +
                                                  brow * BX + bcol);
    }

    if (compute && ok) {
      const int so = (k - kRadius) % kStages;  // stage of the output plane
      const float *box_a = smem + so * NF * PITCH;
      const float *box_b = box_a + (PA ? PITCH : 0);
      const int ez = min(zo - 4, n3 - 4 - zo);
      const bool damp_a = (MODE != kModeSource);
      const bool damp_b = (MODE == kModeForward);

      // pending source injection owed to the previous level of s (adjoint)
      if (MODE == kModeAdjoint && PB && p.pb.active && valid)
        inject_row(p.pb, n1, n2, zo, gy, gx, ob);

      float4 na = oa, nb = ob;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int e = min(exy[j], ez);
        const float b = (e >= 0 && e < kNBound) ? s_bound[e] : 1.0f;
        if (PA) {
          Nbr n;
          float c;
          gather<BX>(box_a, brow, bcol, qa, j, n, c);
          float old = comp(oa, j);
          if (damp_a) old = __fmul_rn(old, b);
          float v = leapfrog(comp(va, j), stencil_sum(p.c, c, n), c, old);
          if (damp_a) v = __fmul_rn(v, b);
          set_comp(na, j, v);
        } else if (MODE == kModeAdjoint) {
          // receiver level not propagated (it == 0): both damping passes
          set_comp(na, j, __fmul_rn(__fmul_rn(comp(oa, j), b), b));
        }
        if (PB) {
          Nbr n;
          float c;
          gather<BX>(box_b, brow, bcol, qb, j, n, c);
          float old = comp(ob, j);
          if (damp_b) old = __fmul_rn(old, b);
          float v = leapfrog(comp(vb, j), stencil_sum(p.c, c, n), c, old);
          if (damp_b) v = __fmul_rn(v, b);
          set_comp(nb, j, v);
        }
      }

      if (valid) {
        if (p.pa.active) inject_row(p.pa, n1, n2, zo, gy, gx, na);
        if (MODE == kModeForward) {
          // Born coupling r += 1e-6 s img, then extraction from r
#pragma unroll
          for (int j = 0; j < 4; ++j)
            set_comp(nb, j,
                     __fadd_rn(comp(nb, j),
                               __fmul_rn(__fmul_rn(1e-6f, comp(na, j)),
                                         comp(im, j))));
          if (p.pb.active) extract_row(p.pb, n1, n2, zo, gy, gx, nb);
          st4(p.a_old + idx, na);
          st4(p.b_old + idx, nb);
        } else if (MODE == kModeAdjoint) {
          // s is the new level when propagated, else the stored one
          const float4 sv = nb;
          float4 ni;
          ni.x = __fadd_rn(im.x, __fmul_rn(sv.x, na.x));
          ni.y = __fadd_rn(im.y, __fmul_rn(sv.y, na.y));
          ni.z = __fadd_rn(im.z, __fmul_rn(sv.z, na.z));
          ni.w = __fadd_rn(im.w, __fmul_rn(sv.w, na.w));
          st4(p.img + idx, ni);
          st4(p.a_old + idx, na);
          if (PB) st4(p.b_old + idx, nb);
        } else {
          st4(p.a_old + idx, na);
        }
      }
    }

    __syncthreads();
    if (abort_flag) break;
    if (NF > 0 && tid == 0 && k >= kRadius && k - kRadius + kStages < K) {
      fence_proxy_async();
      issue(k - kRadius + kStages);
    }
  }

  if (NF > 0 && abort_flag && tid == 0) {
    // drain whatever is still in flight (bounded) before the CTA retires
    for (int s = 0; s < kStages; ++s) {
      uint64_t t0 = global_ns();
      while (!mbar_try_wait(&bars[s], 0) && !mbar_try_wait(&bars[s], 1) &&
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

// ---------------------------------------------------------------------------
struct TileCfg {
  int tx, ty;
};
constexpr TileCfg kTileCfgs[] = {{64, 16}, {32, 16}, {32, 32}, {64, 8}};
constexpr int kNumTileCfgs = sizeof(kTileCfgs) / sizeof(kTileCfgs[0]);

template <int MODE, bool PA, bool PB, int TX, int TY>
cudaError_t launch_t(const CUtensorMap &tm_a, const CUtensorMap &tm_b,
                     const StepParams &p, cudaStream_t stream) {
  using T = TileShape<TX, TY>;
  constexpr int NF = (PA ? 1 : 0) + (PB ? 1 : 0);
  const size_t smem = (size_t)kStages * NF * T::kBoxPitch * 4 + 128;
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
  kern<<<grid, T::kThreads, smem, stream>>>(tm_a, tm_b, p);
  return cudaGetLastError();
}

template <int TX, int TY>
cudaError_t launch_cfg(int mode, bool pa, bool pb, const CUtensorMap &tm_a,
                       const CUtensorMap &tm_b, const StepParams &p,
                       cudaStream_t s) {
  switch (mode) {
    case kModeSource:
      return launch_t<kModeSource, true, false, TX, TY>(tm_a, tm_b, p, s);
    case kModeForward:
      return launch_t<kModeForward, true, true, TX, TY>(tm_a, tm_b, p, s);
    case kModeAdjoint:
      if (pa && pb)
        return launch_t<kModeAdjoint, true, true, TX, TY>(tm_a, tm_b, p, s);
      if (pa)
        return launch_t<kModeAdjoint, true, false, TX, TY>(tm_a, tm_b, p, s);
      if (pb)
        return launch_t<kModeAdjoint, false, true, TX, TY>(tm_a, tm_b, p, s);
      return launch_t<kModeAdjoint, false, false, TX, TY>(tm_a, tm_b, p, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

int tile_cfg_count() { return kNumTileCfgs; }

void tile_cfg_dims(int cfg, int *tx, int *ty) {
  *tx = kTileCfgs[cfg].tx;
  *ty = kTileCfgs[cfg].ty;
}

size_t step_smem_bytes(int cfg, int nfields) {
  const int bx = kTileCfgs[cfg].tx + 8, by = kTileCfgs[cfg].ty + 8;
  const size_t pitch = ((size_t)bx * by * 4 + 127) / 128 * 128;
  return (size_t)kStages * nfields * pitch + 128;
}

cudaError_t launch_step(int mode, bool pa, bool pb, int cfg,
                        const CUtensorMap &tm_a, const CUtensorMap &tm_b,
                        const StepParams &p, cudaStream_t s) {
  if (mode == kModeSource && (!pa || pb)) return cudaErrorInvalidValue;
  if (mode == kModeForward && !(pa && pb)) return cudaErrorInvalidValue;
  switch (cfg) {
    case 0: return launch_cfg<64, 16>(mode, pa, pb, tm_a, tm_b, p, s);
    case 1: return launch_cfg<32, 16>(mode, pa, pb, tm_a, tm_b, p, s);
    case 2: return launch_cfg<32, 32>(mode, pa, pb, tm_a, tm_b, p, s);
    case 3: return launch_cfg<64, 8>(mode, pa, pb, tm_a, tm_b, p, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_point_inject(const PointSet &ps, int npts, float *field,
                                cudaStream_t stream) {
  point_inject_kernel<<<1, 32, 0, stream>>>(ps, npts, field);
  return cudaGetLastError();
}

}  // namespace born
