// FP64 dot product that allocates nothing (born_dot_f64_noalloc).
//
// born_dot_f64 keeps its block partial sums in device memory that
// born_op_create allocates.  Some callers cannot allocate at the point where
// they need a dot product: applications whose device memory is all owned by
// their own pool (a framework that reserves the GPU's memory up front, so a
// cudaMalloc here would fail or fragment it), and code that keeps other
// streams busy and cannot accept the device-wide synchronisation that
// cudaMalloc/cudaFree imply.  This entry point gives them the same FP64 dot
// product with its scratch in a fixed file-scope device array instead; the
// caller passes the two vectors (device pointers) and a host double for the
// result.
//
// Scratch: kNoAllocPartials doubles (512 KiB) plus one result slot, held by
// every GPU that loads this library until the process exits.  Each block
// sums exactly kChunk elements (256 threads x 16) into one partial, so the
// longest vector is kNoAllocPartials * kChunk = 268,435,456 elements; longer
// vectors are rejected with BORN_EINVAL.  Every partial that the final pass
// reads is written by the same call, so nothing needs clearing between
// calls; but all calls share the one array, so calls that overlap on the GPU
// (two streams, two host threads) race and must be serialised by the caller.
//
// The array's address is looked up once per device (cudaGetSymbolAddress,
// with that device current) on the first call made on the device; make that
// first call before any stream capture begins.  The looked-up address is
// kept for the life of the process (device indices below kMaxDevices); a
// cudaDeviceReset reloads the module and leaves it stale, so the function
// must not be called again on a device that was reset.
//
// A CUDA error that the calling thread already has pending is not ours to
// clear: the call then returns BORN_ECUDA without launching, and the caller
// still finds its own error with cudaGetLastError.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/born_gb300.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 16;
constexpr long long kChunk = (long long)kNoAllocThreads * kNoAllocPerThread;
constexpr int kNoAllocPartials = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocPartials + 1];

double *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

__global__ void k_dot_chunks(const float *a, const float *b, long long n,
                             double *partial) {
  __shared__ double red[kNoAllocThreads];
  const long long base = blockIdx.x * kChunk;
  double acc = 0.0;
  for (int k = 0; k < kNoAllocPerThread; ++k) {
    const long long i = base + (long long)k * kNoAllocThreads + threadIdx.x;
    if (i < n) acc += (double)a[i] * (double)b[i];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kNoAllocThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_dot_chunks_final(const double *partial, int nparts,
                                   double *out) {
  __shared__ double red[kNoAllocThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kNoAllocThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Device address of the scratch array on the current device (set up once
// per device).
int scratch_for_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return BORN_ENODEV;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p),
                             g_noalloc_scratch) != cudaSuccess ||
        !p)
      return BORN_ECUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return BORN_OK;
}

}  // namespace

static_assert(BORN_DOT_NOALLOC_MAX == kNoAllocPartials * kChunk,
              "header limit and scratch size disagree");

extern "C" {

int born_dot_f64_noalloc(const float *a, const float *b, long long n,
                         double *out, void *stream) {
  if (!out || n < 0 || (n > 0 && (!a || !b))) return BORN_EINVAL;
  if (n > BORN_DOT_NOALLOC_MAX) {
    std::fprintf(stderr,
                 "born_dot_f64_noalloc: n = %lld exceeds the maximum of %lld "
                 "elements (its fixed scratch holds %d partial sums)\n",
                 n, (long long)BORN_DOT_NOALLOC_MAX, kNoAllocPartials);
    return BORN_EINVAL;
  }
  // an earlier failure of the caller's stays pending and is not reported
  // as ours by the launch checks below
  if (cudaPeekAtLastError() != cudaSuccess) return BORN_ECUDA;
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = (int)((n + kChunk - 1) / kChunk);
  if (nblocks > 0)
    k_dot_chunks<<<nblocks, kNoAllocThreads, 0, s>>>(a, b, n, scratch);
  k_dot_chunks_final<<<1, kNoAllocThreads, 0, s>>>(scratch, nblocks,
                                                   scratch + kNoAllocPartials);
  if (cudaGetLastError() != cudaSuccess) return BORN_ECUDA;
  if (cudaMemcpyAsync(out, scratch + kNoAllocPartials, sizeof(double),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return BORN_ECUDA;
  return BORN_OK;
}

}  // extern "C"
