// Velocity preparation on the device: vel_fd_3d::rand_subspace
// (base/vel_fd_3d.cc:29-134) with a counter-based random generator.
//
// The reference resamples the model velocity onto the padded compute grid
// (nearest index, clamped), perturbs the cells within nrand of each face by
// rejection sampling under a tapered bound (the "random boundary" that makes
// time-reversed source reconstruction lose its boundary reflections), and
// stores v^2 dt^2.  It draws with rand() inside tbb::parallel_for, so its
// output depends on thread scheduling; the host restatement in born_host.cc
// draws in a fixed order to stay comparable.  Here every cell draws from its
// own counter-based stream (SplitMix64 of seed, cell and attempt; Steele,
// Lea and Flood, OOPSLA 2014), so the field is deterministic and is made at
// HBM speed.  Cells outside the bands (nrand = 0 everywhere gives the plain
// model) are computed with the host code's exact float operations, so they
// match born_rand_subspace bit for bit.  The reference loops until a draw is
// accepted; here at most kMaxDraws draws are made, after which the cell
// keeps the largest value the bound allows.
#include <cuda_runtime.h>

#include <algorithm>

#include "born_internal.h"

namespace {

constexpr int kMaxDraws = 64;

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// uniform in [0, 1) with 24 random bits
__device__ __forceinline__ float uniform01(unsigned long long seed,
                                           unsigned long long cell,
                                           unsigned int draw) {
  const unsigned long long h =
      splitmix64(seed ^ splitmix64(cell * 0x100000001B3ull + draw));
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}

// Squared normalised distance into a band of nr cells (vel_fd_3d.cc:60-99).
__device__ __forceinline__ float band2(int i, int n, int nr) {
  if (i < nr) return __fdiv_rn((float)((nr - i) * (nr - i)), (float)(nr * nr));
  if (i >= n - nr) {
    const int k = i - (n - nr - 1);
    return __fdiv_rn((float)(k * k), (float)(nr * nr));
  }
  return 0.f;
}

// (int)((o + d i - vo) / vd), clamped: the host's float operations, each
// separately rounded (no contraction).
__device__ __forceinline__ int model_index(float o, float d, int i, float vo,
                                           float vd, int vn) {
  const float x =
      __fdiv_rn(__fsub_rn(__fadd_rn(o, __fmul_rn(d, (float)i)), vo), vd);
  const int k = (int)x;
  return k < 0 ? 0 : (k > vn - 1 ? vn - 1 : k);
}

struct VelArgs {
  const float *vel;
  int vn1, vn2, vn3;
  float vo1, vo2, vo3, vd1, vd2, vd3, vmax;
  unsigned long long seed;
  int nrand1, nrand2, nrand3;
  float dt;
  int n1, n2, n3;
  float o1, o2, o3, d1, d2, d3;
  float *out;
};

__global__ void k_rand_subspace(const VelArgs a) {
  const long long n = (long long)a.n1 * a.n2 * a.n3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % a.n1), iy = (int)((i / a.n1) % a.n2),
              iz = (int)(i / ((long long)a.n1 * a.n2));
    const int ix_v = model_index(a.o1, a.d1, ix, a.vo1, a.vd1, a.vn1);
    const int iy_v = model_index(a.o2, a.d2, iy, a.vo2, a.vd2, a.vn2);
    const int iz_v = model_index(a.o3, a.d3, iz, a.vo3, a.vd3, a.vn3);
    const float val =
        a.vel[ix_v + (long long)iy_v * a.vn1 + (long long)iz_v * a.vn1 * a.vn2];
    float dx2 = band2(ix, a.n1, a.nrand1);
    const float dy2 = band2(iy, a.n2, a.nrand2);
    const float dz2 = band2(iz, a.n3, a.nrand3);
    if (dx2 < 0.f || dx2 > 1.f) dx2 = 1.f;
    const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(dx2, dy2), dz2));
    float dev = 0.f;
    if (!((double)dist < .0001) && a.nrand2 != 0) {
      const double bound =
          (double)a.vmax * 1.03 * (1. - (double)fminf(1.f, dist) * .4);
      bool found = false;
      for (unsigned int k = 0; k < kMaxDraws && !found; ++k) {
        const float rnd =
            (float)((double)uniform01(a.seed, (unsigned long long)i, k) - .5 -
                    .49 * (double)dist);
        const float d = (float)((double)rnd * 1.3 * (double)dist * (double)val);
        if (fabs((double)__fadd_rn(d, val)) < bound &&
            (double)__fadd_rn(d, val) > 0.0001) {
          dev = d;
          found = true;
        }
      }
      if (!found && (double)val >= bound) dev = (float)(bound * 0.999) - val;
    }
    const float v = __fadd_rn(val, dev);
    a.out[i] = __fmul_rn(__fmul_rn(__fmul_rn(v, v), a.dt), a.dt);
  }
}

}  // namespace

extern "C" int born_make_velocity(born_handle *h, int slot, const float *vel,
                                  int vn1, int vn2, int vn3, float vo1,
                                  float vo2, float vo3, float vd1, float vd2,
                                  float vd3, float vmax,
                                  unsigned long long seed, int nrand1,
                                  int nrand2, int nrand3, float dt, float o1,
                                  float o2, float o3, float d1, float d2,
                                  float d3) {
  int rc = born_check_ready(h);
  if (rc) return rc;
  if (!vel || (slot != 1 && slot != 2) || vn1 < 1 || vn2 < 1 || vn3 < 1 ||
      nrand1 < 0 || nrand2 < 0 || nrand3 < 0 || !(vd1 > 0 && vd2 > 0 && vd3 > 0))
    return born_fail(h, BORN_EINVAL, "born_make_velocity: bad arguments");
  const size_t vbytes = (size_t)vn1 * vn2 * vn3 * 4;
  float *dvel = nullptr;
  if (cudaMalloc(&dvel, vbytes) != cudaSuccess)
    return born_fail(h, BORN_ENOMEM, "born_make_velocity: allocation failed");
  VelArgs a{dvel, vn1, vn2, vn3, vo1, vo2, vo3, vd1, vd2, vd3, vmax, seed,
            nrand1, nrand2, nrand3, dt, h->n1, h->n2, h->n3, o1, o2, o3,
            d1, d2, d3, slot == 1 ? h->vel1 : h->vel2};
  cudaError_t e = cudaMemcpyAsync(dvel, vel, vbytes, cudaMemcpyHostToDevice,
                                  h->stream);
  if (e == cudaSuccess) {
    const long long n = h->n123;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 32);
    k_rand_subspace<<<blocks, 256, 0, h->stream>>>(a);
    e = cudaGetLastError();
    h->launches++;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dvel);
  if (e != cudaSuccess)
    return born_fail(h, BORN_ECUDA, "born_make_velocity: %s",
                     cudaGetErrorString(e));
  (slot == 1 ? h->have_vel1 : h->have_vel2) = true;
  if (slot == 2) h->bg_gen++;
  return BORN_OK;
}

extern "C" int born_get_velocity(born_handle *h, int slot, float *out) {
  int rc = born_check_ready(h);
  if (rc) return rc;
  if (!out || (slot != 1 && slot != 2))
    return born_fail(h, BORN_EINVAL, "born_get_velocity: bad arguments");
  if (cudaMemcpyAsync(out, slot == 1 ? h->vel1 : h->vel2, (size_t)h->n123 * 4,
                      cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return born_fail(h, BORN_ECUDA, "born_get_velocity: copy failed");
  return born_check_device_error(h);
}
