// Fused 2.5D time-step kernels (see born_step.cuh for the design): the FP32
// storage family, the dispatch over storage types and the small kernels
// around the time loops.
#include <algorithm>

#include "born_step_impl.cuh"

namespace born {

BORN_DEFINE_STORAGE_ENTRY(kStoreF32, f32)

namespace {

// Adds the injection of every point into `field` (one thread, point order,
// the reference's order of additions).  16-bit storage: the level's values
// are decoded and re-encoded with the scale of its record slot.
template <int ST>
__global__ void point_inject_kernel(const PointSet ps, int npts, void *field,
                                    const unsigned long long *lv, int rec) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || !ps.active) return;
  const float sc = Store<ST>::kLow ? rec_scale(lv, rec) : 1.f;
  for (int s = 0; s < npts; ++s) {
    const long long c = ps.slot_cell[s];
    if (Store<ST>::kLow) {
      const float v = ld1_level<ST>(field, c) * sc;
      st1_level<ST>(field, c,
                    __fadd_rn(v, point_value(ps, ps.slot_index[s])) / sc);
    } else {
      float *f = static_cast<float *>(field);
      f[c] = __fadd_rn(f[c], point_value(ps, ps.slot_index[s]));
    }
  }
}

// Failure-detection self-test: one thread waits, with the step kernels'
// bounded wait, on an mbarrier that no copy or thread ever completes; when
// the bound runs out it sets the error word and returns, as a step kernel
// whose TMA copy was lost would.
__global__ void wait_timeout_probe(unsigned int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  mbar_fence_init();
  if (!mbar_wait_bounded(&bar, 0)) atomicOr(err, kErrWaitTimeout);
}

__global__ void divide_kernel(const float *a, const float *v, float *out,
                              long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = v[i] != 0.f ? __fdiv_rn(a[i], v[i]) : 0.f;
}

__global__ void level_reset_kernel(unsigned long long *lv, int buf) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int s = 2 * buf; s < 2 * buf + 2; ++s) {
    lv[2 * s] = 0ull;                         // tag 0, max 0
    lv[2 * s + 1] = __float_as_uint(1.0f);    // scale 1
  }
}

__global__ void level_copy_kernel(unsigned long long *lv, int dst, int src,
                                  unsigned int tag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  lv[2 * dst] = ((unsigned long long)tag << 32) | (lv[2 * src] & 0xffffffffull);
  lv[2 * dst + 1] = lv[2 * src + 1];
}

__global__ void absmax_kernel(const float *x, long long n, unsigned int *out) {
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  const unsigned int w = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0) atomicMax(out, w);
}

// v_i = x_i, or x_i - y_i when y is given (a difference of two levels)
__device__ __forceinline__ float snap_value(const float *x, const float *y,
                                            long long i) {
  return y ? __fsub_rn(x[i], y[i]) : x[i];
}

__global__ void absmax_snap_kernel(const float *x, const float *y,
                                   long long n, unsigned int *out) {
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(snap_value(x, y, i)));
  const unsigned int w = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0) atomicMax(out, w);
}

// FP16 snapshot of v (an FP32 level, or the difference of two): the
// power-of-two scale 2^(ceil(log2 max|v|) - 15) (pow2_scale_for, from the
// maximum absmax_snap_kernel left in *maxw) keeps every stored value
// within FP16's finite range; each value is v / scale (an exact division)
// rounded to the nearest FP16, and the scale is recorded in *scale_out.
__global__ void snapshot_f16_kernel(const float *x, const float *y,
                                    long long n, const unsigned int *maxw,
                                    __half *out, float *scale_out) {
  const float scale = pow2_scale_for(__uint_as_float(*maxw));
  const float inv = 1.f / scale;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = __float2half_rn(clamp_f16(snap_value(x, y, i) * inv));
  if (blockIdx.x == 0 && threadIdx.x == 0) *scale_out = scale;
}

// x = stored value * scale (+ base, when given)
__global__ void restore_f16_kernel(const __half *in, long long n,
                                   const float *scale, const float *base,
                                   float *x) {
  const float sc = *scale;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = __half2float(in[i]) * sc;
    x[i] = base ? __fadd_rn(v, base[i]) : v;
  }
}

}  // namespace

cudaError_t launch_snapshot_f16(const float *x, const float *y, long long n,
                                unsigned int *maxw, void *out, float *scale,
                                cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(maxw, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  absmax_snap_kernel<<<blocks, 256, 0, stream>>>(x, y, n, maxw);
  snapshot_f16_kernel<<<blocks, 256, 0, stream>>>(
      x, y, n, maxw, static_cast<__half *>(out), scale);
  return cudaGetLastError();
}

cudaError_t launch_restore_f16(const void *in, long long n,
                               const float *scale, const float *base,
                               float *x, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  restore_f16_kernel<<<blocks, 256, 0, stream>>>(
      static_cast<const __half *>(in), n, scale, base, x);
  return cudaGetLastError();
}

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

static bool lp_mode(int mode) {
  return mode == kModeSource || mode == kModeForward || mode == kModeAdjoint;
}

size_t step_smem_bytes(int storage, int cfg, int mode, bool pa, bool pb) {
  switch (storage) {
    case kStoreBF16: return step_smem_bf16(cfg, mode, pa, pb);
    case kStoreF16: return step_smem_f16(cfg, mode, pa, pb);
    case kStoreF32Fused: return step_smem_f32fused(cfg, mode, pa, pb);
    case kStoreF32Exact:
      return mode == kModeForward ? step_smem_f32exact(cfg, mode, pa, pb)
                                  : step_smem_f32(cfg, mode, pa, pb);
    default: return step_smem_f32(cfg, mode, pa, pb);
  }
}

cudaError_t launch_step(int storage, int mode, bool pa, bool pb, int cfg,
                        const StepMaps &maps, const StepParams &p,
                        cudaStream_t s) {
  if (mode < kModeSource || mode > kModeBornAdj) return cudaErrorInvalidValue;
  if (cfg < 0 || cfg >= kNumTileCfgs) return cudaErrorInvalidValue;
  switch (storage) {
    case kStoreF32: return launch_step_f32(mode, pa, pb, cfg, maps, p, s);
    case kStoreBF16:
      if (!lp_mode(mode)) return cudaErrorInvalidValue;
      return launch_step_bf16(mode, pa, pb, cfg, maps, p, s);
    case kStoreF16:
      if (!lp_mode(mode)) return cudaErrorInvalidValue;
      return launch_step_f16(mode, pa, pb, cfg, maps, p, s);
    case kStoreF32Exact:
      return mode == kModeForward
                 ? launch_step_f32exact(mode, pa, pb, cfg, maps, p, s)
                 : launch_step_f32(mode, pa, pb, cfg, maps, p, s);
    case kStoreF32Fused:
      if (!lp_mode(mode)) return cudaErrorInvalidValue;
      return launch_step_f32fused(mode, pa, pb, cfg, maps, p, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_step_batched(int storage, int mode, bool pa, bool pb,
                                int cfg, const BatchShot *shots,
                                const int *block_start, int nshots, int total,
                                const StepVar &var, cudaStream_t s) {
  if (!lp_mode(mode)) return cudaErrorInvalidValue;
  if (cfg < 0 || cfg >= kNumTileCfgs || nshots < 1 || total < 0)
    return cudaErrorInvalidValue;
  switch (storage) {
    case kStoreF32:
      return launch_step_batched_f32(mode, pa, pb, cfg, shots,
                                               block_start, nshots, total, var,
                                               s);
    case kStoreBF16:
      return launch_step_batched_bf16(mode, pa, pb, cfg, shots,
                                                block_start, nshots, total,
                                                var, s);
    case kStoreF16:
      return launch_step_batched_f16(mode, pa, pb, cfg, shots,
                                               block_start, nshots, total, var,
                                               s);
    case kStoreF32Exact:
      if (mode == kModeForward)
        return launch_step_batched_f32exact(mode, pa, pb, cfg, shots,
                                            block_start, nshots, total, var,
                                            s);
      return launch_step_batched_f32(mode, pa, pb, cfg, shots, block_start,
                                     nshots, total, var, s);
    case kStoreF32Fused:
      return launch_step_batched_f32fused(mode, pa, pb, cfg, shots,
                                          block_start, nshots, total, var, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_point_inject(const PointSet &ps, int npts, void *field,
                                int storage, unsigned long long *lv, int rec,
                                cudaStream_t stream) {
  switch (storage) {
    case kStoreBF16:
      point_inject_kernel<kStoreBF16><<<1, 32, 0, stream>>>(ps, npts, field,
                                                            lv, rec);
      break;
    case kStoreF16:
      point_inject_kernel<kStoreF16><<<1, 32, 0, stream>>>(ps, npts, field, lv,
                                                           rec);
      break;
    default:  // FP32 levels, whatever the arithmetic
      point_inject_kernel<kStoreF32><<<1, 32, 0, stream>>>(ps, npts, field, lv,
                                                           rec);
  }
  return cudaGetLastError();
}

cudaError_t launch_divide(const float *a, const float *v, float *out,
                          long long n, cudaStream_t stream) {
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
  divide_kernel<<<blocks, 256, 0, stream>>>(a, v, out, n);
  return cudaGetLastError();
}

cudaError_t launch_level_reset(unsigned long long *lv, int buf,
                               cudaStream_t stream) {
  level_reset_kernel<<<1, 32, 0, stream>>>(lv, buf);
  return cudaGetLastError();
}

cudaError_t launch_level_copy(unsigned long long *lv, int dst, int src,
                              unsigned int tag, cudaStream_t stream) {
  level_copy_kernel<<<1, 32, 0, stream>>>(lv, dst, src, tag);
  return cudaGetLastError();
}

cudaError_t launch_wait_timeout_probe(unsigned int *err, cudaStream_t stream) {
  wait_timeout_probe<<<1, 32, 0, stream>>>(err);
  return cudaGetLastError();
}

cudaError_t launch_absmax(const float *x, long long n, unsigned int *out,
                          cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  absmax_kernel<<<blocks, 256, 0, stream>>>(x, n, out);
  return cudaGetLastError();
}

}  // namespace born
