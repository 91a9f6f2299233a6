// Internal definitions shared by the C ABI translation units (not part of
// the public interface).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/born_gb300.h"
#include "born_step.cuh"

// Device copy of one point set (sources or receivers).
struct DevPoints {
  int npts = 0, nt = 0;
  int zlo = 1 << 30, zhi = -1;  // planes holding points
  int *plane_off = nullptr, *cell_head = nullptr, *slot_cell = nullptr,
      *slot_index = nullptr;
  float *traces = nullptr;
  size_t traces_cap = 0;
  void release() {
    cudaFree(plane_off);
    cudaFree(cell_head);
    cudaFree(slot_cell);
    cudaFree(slot_index);
    cudaFree(traces);
    *this = DevPoints();
  }
};

struct born_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // grid
  bool have_space = false;
  int n1 = 0, n2 = 0, n3 = 0;
  long long n123 = 0;
  float coeffs[13] = {};
  float bound[born::kNBound] = {};
  // sinc tables (rows x 8)
  int jt_s = 0, jt_d = 0;
  std::vector<float> tab_s, tab_d;
  int jt = 1;  // the reference's _jt: last jt given to a time loop
  // device fields
  float *vel1 = nullptr, *vel2 = nullptr;
  float *s0 = nullptr, *s1 = nullptr;  // source levels (p0, p1 of source_prop)
  float *r0 = nullptr, *r1 = nullptr;  // receiver / scattered levels
  float *f0 = nullptr, *f1 = nullptr;  // forward background levels
  float *img = nullptr, *refl = nullptr;
  unsigned int *err_dev = nullptr;
  bool have_vel1 = false, have_vel2 = false, have_refl = false;
  DevPoints src, rec;
  bool src_levels_valid = false;
  const float *host_p0 = nullptr, *host_p1 = nullptr;
  int tile_cfg = -1, zseg = 0;
  // autotuner: best tile configuration per step mode (-1: not tuned yet)
  bool autotune = true;
  int tuned_cfg[6] = {-1, -1, -1, -1, -1, -1};
  float tuned_ms[6] = {0, 0, 0, 0, 0, 0};
  long long launches = 0;
  int ntblock = 0;
  // TMA descriptors by (buffer, tile config * 2 + kind); kind 0 = halo box,
  // 1 = centre tile
  std::map<std::pair<const void *, int>, CUtensorMap> maps;
  // exact linearised adjoint: checkpoints and the per-segment A s buffer
  float *ckpt = nullptr, *gbuf = nullptr;
  size_t ckpt_levels = 0, gbuf_levels = 0;
};


// Error helpers (born_api.cu)
int born_fail(born_handle *h, int code, const char *fmt, ...);
int born_check_ready(born_handle *h);
int born_check_device_error(born_handle *h);
