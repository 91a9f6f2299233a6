// Born forward step with FP32 levels in the reference's operation order and
// the Born coupling formed exactly as the reference's double expression
// (born_couple.h); the other steps of this storage are the FP32 kernels.
#include <algorithm>

#include "../../include/born_gb300.h"
#include "born_step_impl.cuh"

namespace born {

BORN_DEFINE_STORAGE_ENTRY(kStoreF32Exact, f32exact)

namespace {
// the forward step's coupling arithmetic on plain arrays, two cells per
// thread as in the step kernel
__global__ void couple_check_kernel(const float *r, const float *s,
                                    const float *m, float *out, long long n) {
  const long long stride = 2ll * gridDim.x * blockDim.x;
  for (long long i = 2ll * (blockIdx.x * (long long)blockDim.x + threadIdx.x);
       i < n; i += stride) {
    if (i + 1 < n) {
      unsigned int f;
      float2 v = couple::couple_fast2(make_float2(r[i], r[i + 1]),
                                      make_float2(s[i], s[i + 1]),
                                      make_float2(m[i], m[i + 1]), &f);
      if (f & 1u) v.x = couple::couple_slow(r[i], s[i], m[i]);
      if (f & 2u) v.y = couple::couple_slow(r[i + 1], s[i + 1], m[i + 1]);
      out[i] = v.x;
      out[i + 1] = v.y;
    } else {
      out[i] = couple::couple_exact(r[i], s[i], m[i], nullptr);
    }
  }
}
}  // namespace

}  // namespace born

extern "C" int born_couple_exact_device(const float *r, const float *s,
                                        const float *m, float *out,
                                        long long n, void *stream) {
  if (n < 0 || (n > 0 && (!r || !s || !m || !out))) return BORN_EINVAL;
  if (n == 0) return BORN_OK;
  const long long pairs = (n + 1) / 2;
  const int blocks = (int)std::min<long long>((pairs + 255) / 256, 152 * 16);
  born::couple_check_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(
      r, s, m, out, n);
  return cudaGetLastError() == cudaSuccess ? BORN_OK : BORN_ECUDA;
}
