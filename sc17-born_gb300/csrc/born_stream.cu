// Streaming ceiling of a read/write mix of arrays: what plain float4 loads
// and stores sustain for the same number of arrays a step kernel streams
// (the adjoint step reads 7 arrays and writes 3 per cell, the forward step
// 6 and 2, the source step 3 and 1).  The step kernels' roofline is quoted
// against the machine's measured copy bandwidth; this gives the second, per-mix
// denominator.  Test and measurement support: no step uses it.
#include <cuda_runtime.h>

#include <vector>

#include "born_gb300.h"

namespace {

constexpr int kMaxReads = 8, kMaxWrites = 4;

struct Arrays {
  const float4 *in[kMaxReads];
  float4 *out[kMaxWrites];
};

// out_w[i] = sum of the inputs at i, grid-stride over n4 float4s
template <int R, int W>
__global__ void stream_mix(const __grid_constant__ Arrays a, long long n4) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    float4 s = a.in[0][i];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      const float4 v = a.in[r][i];
      s.x += v.x;
      s.y += v.y;
      s.z += v.z;
      s.w += v.w;
    }
#pragma unroll
    for (int w = 0; w < W; ++w) a.out[w][i] = s;
  }
}

template <int R, int W>
cudaError_t launch(const Arrays &a, long long n4, int blocks, cudaStream_t s) {
  stream_mix<R, W><<<blocks, 256, 0, s>>>(a, n4);
  return cudaGetLastError();
}

using LaunchFn = cudaError_t (*)(const Arrays &, long long, int, cudaStream_t);

template <int R>
LaunchFn pick_w(int w) {
  switch (w) {
    case 1: return launch<R, 1>;
    case 2: return launch<R, 2>;
    case 3: return launch<R, 3>;
    case 4: return launch<R, 4>;
    default: return nullptr;
  }
}

LaunchFn pick(int r, int w) {
  switch (r) {
    case 1: return pick_w<1>(w);
    case 2: return pick_w<2>(w);
    case 3: return pick_w<3>(w);
    case 4: return pick_w<4>(w);
    case 5: return pick_w<5>(w);
    case 6: return pick_w<6>(w);
    case 7: return pick_w<7>(w);
    case 8: return pick_w<8>(w);
    default: return nullptr;
  }
}

}  // namespace

extern "C" int born_stream_mix_gbs(int reads, int writes, long long n, int reps,
                                   float *gbs) {
  if (!gbs || reads < 1 || reads > kMaxReads || writes < 1 ||
      writes > kMaxWrites || n < 4 || n % 4 != 0 || reps < 1)
    return BORN_EINVAL;
  const LaunchFn fn = pick(reads, writes);
  if (!fn) return BORN_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
          cudaSuccess)
    return BORN_ECUDA;
  std::vector<float *> bufs(reads + writes, nullptr);
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = BORN_OK;
  for (float *&b : bufs)
    if (cudaMalloc(&b, (size_t)n * sizeof(float)) != cudaSuccess ||
        cudaMemset(b, 0, (size_t)n * sizeof(float)) != cudaSuccess) {
      rc = BORN_ENOMEM;
      break;
    }
  if (!rc && (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) !=
                  cudaSuccess ||
              cudaEventCreate(&e0) != cudaSuccess ||
              cudaEventCreate(&e1) != cudaSuccess))
    rc = BORN_ECUDA;
  float best = 0.f;
  if (!rc) {
    Arrays a{};
    for (int r = 0; r < reads; ++r) a.in[r] = reinterpret_cast<const float4 *>(bufs[r]);
    for (int w = 0; w < writes; ++w)
      a.out[w] = reinterpret_cast<float4 *>(bufs[reads + w]);
    const long long n4 = n / 4;
    // a few grid sizes (CTAs per SM), best sustained rate
    for (int per_sm : {8, 16}) {
      const int blocks = sms * per_sm;
      for (int i = 0; i < 3 && !rc; ++i)
        if (fn(a, n4, blocks, s) != cudaSuccess) rc = BORN_ECUDA;
      if (rc) break;
      cudaEventRecord(e0, s);
      for (int i = 0; i < reps && !rc; ++i)
        if (fn(a, n4, blocks, s) != cudaSuccess) rc = BORN_ECUDA;
      cudaEventRecord(e1, s);
      float ms = 0.f;
      if (!rc && (cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = BORN_ECUDA;
      if (rc) break;
      const double bytes = (double)(reads + writes) * 4.0 * (double)n * reps;
      const float rate = (float)(bytes / (ms * 1e-3) / 1e9);
      if (rate > best) best = rate;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  for (float *b : bufs)
    if (b) cudaFree(b);
  if (!rc) *gbs = best;
  return rc;
}
