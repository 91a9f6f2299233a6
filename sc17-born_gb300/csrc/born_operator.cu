// Born operator (model image <-> shot data) and CG least-squares solver on
// device-resident vectors.
//
// born_op mirrors rtm_zero_op (base/rtm_zero_op_3d.cc) behind the
// my_operator contract forward/adjoint(add, model, data)
// (base/my_operator.h:18-25), but honours the model and data vectors it is
// given (the reference reads the model from a file member and writes data to
// a file, rtm_zero_op_3d.cc:161,193,295).  Per shot it runs, on the GPU:
//
//   forward (rtm_zero_op_3d.cc:137-194):
//     img   = laplac(window(model))            image_rtm_3d.cc:53-95, laplac_3d.cc:51-105
//     traces = rtmForward(img)                  cpu_prop.cc:22-54
//     data += deriv(map_data(traces))           map_data_3d.cc:57-75, deriv_3d.cc:31-56
//   adjoint (rtm_zero_op_3d.cc:240-296):
//     traces = map_data'(deriv'(data))          deriv_3d.cc:4-29, map_data_3d.cc:37-55
//     img   = rtmAdjoint(sourceProp, traces)    cpu_prop.cc:56-129
//     model += window'(laplac'(img))            laplac_3d.cc:4-49, image_rtm_3d.cc:24-51
//
// In exact mode the propagator pair is born_lin_forward / born_lin_adjoint
// (an exact transpose pair), so the whole operator passes the dot-product
// test and CG converges; reference mode reproduces rtm_zero_op.
//
// Vector algebra follows cgstep (base/cgstep.cc:11-54) with FP64 dot
// products (block partials in double, then one final block) and FP64 step
// lengths.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "born_host.h"
#include "born_internal.h"

namespace {

constexpr int kThreads = 256;

int grid_for(long long n) {
  return (int)std::min<long long>((n + kThreads - 1) / kThreads, 152 * 32);
}

// ---- image window (image_rtm_3d.cc:53-95 extract_sub, :24-51 add_image) ----
__global__ void k_extract_window(const float *whole, int w1, int w2, int w3,
                                 float *sub, int s1, int s2, int s3, int f1,
                                 int f2, int f3) {
  const long long n = (long long)s1 * s2 * s3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int i1 = (int)(i % s1), i2 = (int)((i / s1) % s2),
              i3 = (int)(i / ((long long)s1 * s2));
    const int o1 = i1 + f1, o2 = i2 + f2, o3 = i3 + f3;
    float v = 0.f;
    if (o1 >= 0 && o1 < w1 && o2 >= 0 && o2 < w2 && o3 >= 0 && o3 < w3)
      v = whole[o1 + (long long)o2 * w1 + (long long)o3 * w1 * w2];
    sub[i] = v;
  }
}

__global__ void k_add_window(float *whole, int w1, int w2, int w3,
                             const float *sub, int s1, int s2, int s3, int f1,
                             int f2, int f3) {
  const long long n = (long long)s1 * s2 * s3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int i1 = (int)(i % s1), i2 = (int)((i / s1) % s2),
              i3 = (int)(i / ((long long)s1 * s2));
    const int o1 = i1 + f1, o2 = i2 + f2, o3 = i3 + f3;
    if (o1 >= 0 && o1 < w1 && o2 >= 0 && o2 < w2 && o3 >= 0 && o3 < w3) {
      float *w = whole + o1 + (long long)o2 * w1 + (long long)o3 * w1 * w2;
      *w = __fadd_rn(*w, sub[i]);
    }
  }
}

// ---- laplac: first difference along axis 3 (laplac_3d.cc) ----
// forward: d[i+n12] += m[i]; d[i] -= m[i] for i < n12 (n3-1), in i order, so
// cell j first gains m[j-n12] then loses m[j].
__global__ void k_laplac_fwd(const float *m, float *d, long long n12,
                             long long n, int add) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    float v = add ? d[j] : 0.f;
    if (j >= n12) v = __fadd_rn(v, m[j - n12]);
    if (j < n - n12) v = __fsub_rn(v, m[j]);
    d[j] = v;
  }
}

__global__ void k_laplac_adj(float *m, const float *d, long long n12,
                             long long n, int add) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    float v = add ? m[j] : 0.f;
    if (j < n - n12) v = __fadd_rn(v, __fsub_rn(d[j + n12], d[j]));
    m[j] = v;
  }
}

// ---- map_data: traces of nt <-> padded traces of ntb (map_data_3d.cc) ----
__global__ void k_map_fwd(const float *m, float *d, int nt, int ntr, int ntb,
                          int add) {
  const long long n = (long long)nt * ntr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long tr = i / nt, it = i % nt;
    const float v = m[tr * ntb + it + 4];
    d[i] = add ? __fadd_rn(d[i], v) : v;
  }
}

__global__ void k_map_adj(float *m, const float *d, int nt, int ntr, int ntb,
                          int add) {
  const long long n = (long long)ntb * ntr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long tr = i / ntb, k = i % ntb - 4;
    float v = add ? m[i] : 0.f;
    if (k >= 0 && k < nt) v = __fadd_rn(v, d[tr * nt + k]);
    m[i] = v;
  }
}

// ---- deriv: time first difference / dt (deriv_3d.cc), one thread per
// trace so every sample sees the reference's sequence of updates, including
// the repeated contribution of each trace's first sample (the i3 head and
// i2 head statements).  traces [n3][n2][n1], n1 = time.
__global__ void k_deriv_fwd(const float *m, float *d, int n1, int n2, int n3,
                            float d1, int add) {
  const long long ntr = (long long)n2 * n3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < ntr; t += (long long)gridDim.x * blockDim.x) {
    const int i2 = (int)(t % n2);
    const float *mt = m + t * n1;
    float *dt = d + t * n1;
    if (!add)
      for (int i = 0; i < n1; ++i) dt[i] = 0.f;
    const int heads = i2 == 0 ? 2 : 1;
    for (int h = 0; h < heads; ++h) {
      dt[1] = __fadd_rn(dt[1], __fdiv_rn(mt[0], d1));
      dt[0] = __fsub_rn(dt[0], __fdiv_rn(mt[0], d1));
    }
    for (int i1 = 0; i1 < n1 - 1; ++i1) {
      const float q = __fdiv_rn(mt[i1], d1);
      dt[i1] = __fsub_rn(dt[i1], q);
      dt[i1 + 1] = __fadd_rn(dt[i1 + 1], q);
    }
  }
}

__global__ void k_deriv_adj(float *m, const float *d, int n1, int n2, int n3,
                            float d1, int add) {
  const long long ntr = (long long)n2 * n3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < ntr; t += (long long)gridDim.x * blockDim.x) {
    const int i2 = (int)(t % n2);
    float *mt = m + t * n1;
    const float *dt = d + t * n1;
    if (!add)
      for (int i = 0; i < n1; ++i) mt[i] = 0.f;
    const int heads = i2 == 0 ? 2 : 1;
    for (int h = 0; h < heads; ++h)
      mt[0] = __fadd_rn(mt[0], __fdiv_rn(__fsub_rn(dt[1], dt[0]), d1));
    for (int i1 = 0; i1 < n1 - 1; ++i1)
      mt[i1] = __fadd_rn(mt[i1], __fdiv_rn(__fsub_rn(dt[i1 + 1], dt[i1]), d1));
  }
}

// ---- FP64 vector algebra for CG ----
constexpr int kDotBlocks = 1024;

__global__ void k_dot_partial(const float *a, const float *b, long long n,
                              double *partial) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_dot_final(const double *partial, int nparts, double *out) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// x = x sc1 + y sc2 in double, stored as float (hypercube_float::scale_add)
__global__ void k_scale_add(float *x, double sc1, const float *y, double sc2,
                            long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = (float)((double)x[i] * sc1 + (double)y[i] * sc2);
}

__global__ void k_add(float *x, const float *y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = __fadd_rn(x[i], y[i]);
}

// x = y sc1 + z sc2 in double, stored as float (the four-argument
// hypercube_float::scale_add, hypercube_float.cc:140-151)
__global__ void k_lincomb(float *x, double sc1, const float *y, double sc2,
                          const float *z, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = (float)((double)y[i] * sc1 + (double)z[i] * sc2);
}

// x = x r in double, stored as float (hypercube_float.h:25-27)
__global__ void k_scale(float *x, double r, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = (float)((double)x[i] * r);
}

// x = (float) val (hypercube_float.cc:50-52)
__global__ void k_fill(float *x, float val, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = val;
}

}  // namespace

// ---------------------------------------------------------------------------
struct born_op {
  born_handle *h = nullptr;
  born_op_params p{};
  // compute grid
  int n1 = 0, n2 = 0, n3 = 0;
  float o1 = 0, o2 = 0, o3 = 0;
  int f = 0;  // boundary cells on each side of the model (nbound + fat)
  // model-grid sample of the compute grid's first cell per axis, as the
  // image window forms it from the two axes (image_rtm_3d.cc:33-35): -f, or
  // -f + 1 where the float origins truncate (spacings such as 10.1)
  int w1 = 0, w2 = 0, w3 = 0;
  float dt = 0;
  int jt = 1, nt = 0, nt_big = 0;
  std::vector<float> table;  // jt x 8
  std::vector<float> wavelet;  // time derivative of the raw wavelet
  std::vector<int> rec_locs;
  std::vector<std::vector<int>> src_locs;
  std::vector<std::vector<float>> src_vals;
  std::vector<float *> vrand;  // per shot (reference mode), device
  float *vnone = nullptr;      // device, shared by all shots
  float *traces_tmp = nullptr, *shot_tmp = nullptr;  // device scratch
  double *dot_partial = nullptr, *dot_out = nullptr;
  long long model_n = 0, data_n = 0, shot_n = 0;
  std::vector<float> host_vel;
  // the shot whose source and model the handle holds (op_select_shot), and
  // the handle's background generation when it was selected
  int cur_shot = -1;
  unsigned long long cur_gen = 0;
  // Exact mode: each shot's background checkpoints, kept across operator
  // applications.  The background s of a shot depends only on the fixed
  // background velocity and the shot's source, not on the model, so after
  // a shot's linearised forward its adjoint (and every later one) can skip
  // the forward sweep that would store them again; with one handle for all
  // shots the handle's own checkpoints only ever belong to the last shot.
  // A shot gets a slot while free device memory stays above a quarter of
  // the device; the slot's buffers are the handle's checkpoint buffers
  // while that shot's linearised forward or adjoint runs.
  struct CkptSlot {
    bool owned = false;
    float *buf = nullptr, *scale = nullptr;
    size_t bytes = 0, scale_levels = 0;
    bool valid = false;
    int jt = 0, nt = 0, interval = 0, kind = 0;
  };
  std::vector<CkptSlot> slots;
  CkptSlot own;  // the handle's own checkpoint state while a slot is in
  long long ckpt_reused_shots = 0;  // adjoints that skipped their sweep
};

namespace {

long long shot_size(const born_op *op) {
  return (long long)op->p.rec_nx * op->p.rec_ny * op->p.nt_data;
}

#define OPCK(op, call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return born_fail((op)->h, BORN_ECUDA, "%s: %s", #call,                 \
                       cudaGetErrorString(e_));                              \
  } while (0)

int op_select_shot(born_op *op, int ishot) {
  born_handle *h = op->h;
  // exact mode reads no random-boundary model: when this shot's source and
  // model are still the handle's (nothing changed them since, bg_gen says),
  // keep them, and with them the background checkpoints of its last
  // linearised forward
  if (op->p.exact && op->cur_shot == ishot && op->cur_gen == h->bg_gen)
    return BORN_OK;
  int rc = born_set_source_func(h, 9, op->nt_big, op->src_locs[ishot].data(),
                                op->src_vals[ishot].data());
  if (rc) return rc;
  const size_t bytes = (size_t)h->n123 * 4;
  if (!op->p.exact) {
    OPCK(op, cudaMemcpyAsync(h->vel1, op->vrand[ishot], bytes,
                             cudaMemcpyDeviceToDevice, h->stream));
    h->have_vel1 = true;
  }
  OPCK(op, cudaMemcpyAsync(h->vel2, op->vnone, bytes, cudaMemcpyDeviceToDevice,
                           h->stream));
  h->have_vel2 = true;
  h->bg_gen++;  // another shot's background
  op->cur_shot = ishot;
  op->cur_gen = h->bg_gen;
  return BORN_OK;
}

// Puts shot s's checkpoint slot into the handle (false: the shot has none
// and the handle's own checkpoints are used).
bool op_ckpt_swap_in(born_op *op, int s) {
  born_handle *h = op->h;
  born_op::CkptSlot &sl = op->slots[s];
  if (!sl.owned) {
    const int interval =
        op->p.ckpt_interval > 0 ? op->p.ckpt_interval : 50;
    const size_t levels = 2 * (size_t)((op->nt + interval - 1) / interval + 1);
    const size_t esize = h->ckpt_storage == BORN_CKPT_F16 ? 2 : 4;
    const size_t need = levels * (size_t)h->n123 * esize;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess ||
        need + total_b / 4 > free_b)
      return false;
    sl.owned = true;  // its buffers come from the handle's allocator
  }
  born_op::CkptSlot &o = op->own;
  o.buf = h->ckpt;
  o.bytes = h->ckpt_bytes;
  o.scale = h->ckpt_scale;
  o.scale_levels = h->ckpt_scale_levels;
  o.valid = h->ckpt_valid && h->ckpt_gen == h->bg_gen;
  o.jt = h->ckpt_jt;
  o.nt = h->ckpt_nt;
  o.interval = h->ckpt_interval;
  o.kind = h->ckpt_kind;
  h->ckpt = sl.buf;
  h->ckpt_bytes = sl.bytes;
  h->ckpt_scale = sl.scale;
  h->ckpt_scale_levels = sl.scale_levels;
  // the shot's background is the same as when the slot was filled
  h->ckpt_valid = sl.valid;
  h->ckpt_gen = h->bg_gen;
  h->ckpt_jt = sl.jt;
  h->ckpt_nt = sl.nt;
  h->ckpt_interval = sl.interval;
  h->ckpt_kind = sl.kind;
  return true;
}

// Takes shot s's checkpoints back from the handle (the handle's allocator
// may have replaced the buffers) and restores the handle's own.
void op_ckpt_swap_out(born_op *op, int s) {
  born_handle *h = op->h;
  born_op::CkptSlot &sl = op->slots[s];
  sl.buf = h->ckpt;
  sl.bytes = h->ckpt_bytes;
  sl.scale = h->ckpt_scale;
  sl.scale_levels = h->ckpt_scale_levels;
  sl.valid = h->ckpt_valid && h->ckpt_gen == h->bg_gen;
  sl.jt = h->ckpt_jt;
  sl.nt = h->ckpt_nt;
  sl.interval = h->ckpt_interval;
  sl.kind = h->ckpt_kind;
  const born_op::CkptSlot &o = op->own;
  h->ckpt = o.buf;
  h->ckpt_bytes = o.bytes;
  h->ckpt_scale = o.scale;
  h->ckpt_scale_levels = o.scale_levels;
  h->ckpt_valid = false;  // another shot's background is in the levels now
  h->ckpt_jt = o.jt;
  h->ckpt_nt = o.nt;
  h->ckpt_interval = o.interval;
  h->ckpt_kind = o.kind;
}

int op_dot(born_op *op, const float *a, const float *b, long long n,
           double *out) {
  born_handle *h = op->h;
  k_dot_partial<<<kDotBlocks, kThreads, 0, h->stream>>>(a, b, n,
                                                        op->dot_partial);
  k_dot_final<<<1, kThreads, 0, h->stream>>>(op->dot_partial, kDotBlocks,
                                             op->dot_out);
  OPCK(op, cudaGetLastError());
  h->launches += 2;
  OPCK(op, cudaMemcpyAsync(out, op->dot_out, sizeof(double),
                           cudaMemcpyDeviceToHost, h->stream));
  OPCK(op, cudaStreamSynchronize(h->stream));
  return BORN_OK;
}

}  // namespace

extern "C" {

int born_op_create(born_handle *h, const born_op_params *p,
                   const float *velocity, const float *shots,
                   const float *wavelet, born_op **out) {
  if (!h || !p || !velocity || !shots || !wavelet || !out) return BORN_EINVAL;
  *out = nullptr;
  if (p->n1 < 1 || p->n2 < 1 || p->n3 < 1 || p->nshots < 1 ||
      p->nt_data < 2 || p->rec_nx < 1 || p->rec_ny < 1 || p->nbound < 0 ||
      p->nt_wavelet < 2)
    return born_fail(h, BORN_EINVAL, "born_op_create: bad parameters");
  born_op *op = new born_op();
  op->h = h;
  op->p = *p;
  op->slots.resize(p->nshots);
  const long long nm = (long long)p->n1 * p->n2 * p->n3;
  op->model_n = nm;
  op->host_vel.assign(velocity, velocity + nm);
  float vmax = 0.f;
  for (long long i = 0; i < nm; ++i) vmax = std::max(vmax, velocity[i]);
  // fd_prop::calc_stability / set_fd_basics (fd_prop_3d.cc:6-66)
  const float dmin = p->d3 < p->d1 && p->d3 < p->d2 ? p->d3
                     : p->d2 < p->d1                ? p->d3
                                                    : p->d1;
  op->dt = born_calc_stability(vmax, dmin, p->dt_data, p->nt_data, &op->nt);
  op->jt = (int)(p->dt_data / op->dt);
  const int fat = 4;
  op->n1 = born_compute_size(p->n1, p->nbound, fat);
  op->n2 = born_compute_size(p->n2, p->nbound, fat);
  op->n3 = born_compute_size(p->n3, p->nbound, fat);
  op->f = p->nbound + fat;
  op->o1 = p->o1 - p->d1 * op->f;
  op->o2 = p->o2 - p->d2 * op->f;
  op->o3 = p->o3 - p->d3 * op->f;
  op->w1 = born_window_offset(op->o1, p->o1, p->d1);
  op->w2 = born_window_offset(op->o2, p->o2, p->d2);
  op->w3 = born_window_offset(op->o3, p->o3, p->d3);
  op->nt_big = p->nt_data + 8;
  // the linearised forward stores the background checkpoints the adjoint
  // uses (single-shot operators reuse them)
  h->ckpt_every = p->ckpt_interval > 0 ? p->ckpt_interval : 50;
  op->table.resize((size_t)op->jt * 8);
  born_sinc_table(op->jt, 8, op->table.data());
  // wavelet time derivative (source_func_3d.cc:120-124)
  op->wavelet.resize(p->nt_wavelet);
  born_wavelet_deriv(wavelet, p->nt_wavelet, p->dt_wavelet, op->wavelet.data());
  int rc = born_create_space(h, p->d1, p->d2, p->d3, 50.f, .0005f, .0005f,
                             op->n1, op->n2, op->n3);
  if (!rc) rc = born_set_sinc_table(h, 0, 8, op->jt, op->table.data());
  if (!rc) rc = born_set_sinc_table(h, 1, 8, op->jt, op->table.data());
  if (rc) {
    delete op;
    return rc;
  }
  const float o[3] = {op->o1, op->o2, op->o3};
  // receivers (data_rtm_3d.cc:79-88; map_data_3d.cc:17-31)
  op->rec_locs.resize((size_t)p->rec_nx * p->rec_ny);
  born_receiver_geometry(p->rec_nx, p->rec_ny, p->rec_ox, p->rec_dx, p->rec_oy,
                         p->rec_dy, p->rec_depth, o[0], o[1], o[2], p->d1,
                         p->d2, p->d3, op->n1, op->n2, op->rec_locs.data());
  std::vector<float> zeros((size_t)op->rec_locs.size() * op->nt_big, 0.f);
  rc = born_set_receiver_func(h, p->rec_nx, p->rec_ny, op->nt_big,
                              op->rec_locs.data(), zeros.data());
  // sources (source_func_3d.cc:76-109) and velocities (vel_fd_3d.cc:29-134)
  const size_t n123 = (size_t)op->n1 * op->n2 * op->n3;
  std::vector<float> vtmp(n123);
  if (!rc)
    rc = born_rand_subspace(velocity, p->n1, p->n2, p->n3, p->o1, p->o2, p->o3,
                            p->d1, p->d2, p->d3, vmax, 0, 0, 0, 0, op->dt,
                            op->n1, op->n2, op->n3, o[0], o[1], o[2], p->d1,
                            p->d2, p->d3, vtmp.data());
  if (!rc && cudaMalloc(&op->vnone, n123 * 4) != cudaSuccess) rc = BORN_ENOMEM;
  if (!rc && cudaMemcpy(op->vnone, vtmp.data(), n123 * 4,
                        cudaMemcpyHostToDevice) != cudaSuccess)
    rc = BORN_ECUDA;
  for (int s = 0; s < p->nshots && !rc; ++s) {
    std::vector<int> locs(9);
    std::vector<float> vals((size_t)9 * op->nt_big);
    born_source_geometry(shots[3 * s], shots[3 * s + 1], shots[3 * s + 2],
                         o[0], o[1], o[2], p->d1, p->d2, p->d3, op->n1, op->n2,
                         op->wavelet.data(), p->nt_wavelet, op->nt_big,
                         locs.data(), vals.data());
    op->src_locs.push_back(locs);
    op->src_vals.push_back(vals);
    if (!p->exact) {
      // seed = locs_s[3] % 10000 (rtm_zero_op_3d.cc:151,254)
      const int seed = locs[3] - (locs[3] / 10000) * 10000;
      rc = born_rand_subspace(velocity, p->n1, p->n2, p->n3, p->o1, p->o2,
                              p->o3, p->d1, p->d2, p->d3, vmax, seed,
                              p->nbound, p->nbound, p->nbound, op->dt, op->n1,
                              op->n2, op->n3, o[0], o[1], o[2], p->d1, p->d2,
                              p->d3, vtmp.data());
      float *dv = nullptr;
      if (!rc && cudaMalloc(&dv, n123 * 4) != cudaSuccess) rc = BORN_ENOMEM;
      if (!rc && cudaMemcpy(dv, vtmp.data(), n123 * 4,
                            cudaMemcpyHostToDevice) != cudaSuccess)
        rc = BORN_ECUDA;
      op->vrand.push_back(dv);
    }
  }
  op->shot_n = shot_size(op);
  op->data_n = op->shot_n * p->nshots;
  if (!rc &&
      (cudaMalloc(&op->traces_tmp, op->rec_locs.size() * op->nt_big * 4) !=
           cudaSuccess ||
       cudaMalloc(&op->shot_tmp, op->shot_n * 4) != cudaSuccess ||
       cudaMalloc(&op->dot_partial, kDotBlocks * sizeof(double)) !=
           cudaSuccess ||
       cudaMalloc(&op->dot_out, sizeof(double)) != cudaSuccess))
    rc = BORN_ENOMEM;
  if (rc) {
    born_op_destroy(op);
    return rc == BORN_ENOMEM
               ? born_fail(h, rc, "born_op_create: device allocation failed")
               : rc;
  }
  *out = op;
  return BORN_OK;
}

int born_op_destroy(born_op *op) {
  if (!op) return BORN_OK;
  cudaSetDevice(op->h->device);
  cudaStreamSynchronize(op->h->stream);
  for (float *v : op->vrand) cudaFree(v);
  for (born_op::CkptSlot &sl : op->slots) {
    cudaFree(sl.buf);
    cudaFree(sl.scale);
  }
  cudaFree(op->vnone);
  cudaFree(op->traces_tmp);
  cudaFree(op->shot_tmp);
  cudaFree(op->dot_partial);
  cudaFree(op->dot_out);
  delete op;
  return BORN_OK;
}

long long born_op_checkpoints_reused(const born_op *op) {
  return op ? op->ckpt_reused_shots : BORN_EINVAL;
}

int born_op_checkpoint_shots(const born_op *op) {
  if (!op) return BORN_EINVAL;
  int n = 0;
  for (const born_op::CkptSlot &sl : op->slots) n += sl.owned && sl.buf ? 1 : 0;
  return n;
}

int born_op_sizes(const born_op *op, long long *model_n, long long *data_n,
                  int *nt_fd, float *dt_fd) {
  if (!op) return BORN_EINVAL;
  if (model_n) *model_n = op->model_n;
  if (data_n) *data_n = op->data_n;
  if (nt_fd) *nt_fd = op->nt;
  if (dt_fd) *dt_fd = op->dt;
  return BORN_OK;
}

int born_op_forward(born_op *op, int add, const float *model, float *data) {
  if (!op || !model || !data) return BORN_EINVAL;
  born_handle *h = op->h;
  int rc = born_check_ready(h);
  if (rc) return rc;
  const born_op_params &p = op->p;
  const long long n123 = h->n123, n12 = (long long)h->n1 * h->n2;
  const int ntr = p.rec_nx * p.rec_ny;
  if (!add) OPCK(op, cudaMemsetAsync(data, 0, op->data_n * 4, h->stream));
  for (int s = 0; s < p.nshots; ++s) {
    rc = op_select_shot(op, s);
    if (rc) return rc;
    // img = laplac(window(model)) on the compute grid (rtm_zero_op_3d.cc:161-180)
    k_extract_window<<<grid_for(n123), kThreads, 0, h->stream>>>(
        model, p.n1, p.n2, p.n3, h->img, h->n1, h->n2, h->n3, op->w1, op->w2,
        op->w3);
    k_laplac_fwd<<<grid_for(n123), kThreads, 0, h->stream>>>(h->img, h->refl,
                                                             n12, n123, 0);
    OPCK(op, cudaGetLastError());
    h->launches += 2;
    h->have_refl = true;
    OPCK(op, cudaMemsetAsync(h->rec.traces, 0, (size_t)ntr * op->nt_big * 4,
                             h->stream));
    if (p.exact) {
      const bool slot = op_ckpt_swap_in(op, s);
      rc = born_lin_forward(h, op->jt, op->nt, nullptr);
      if (slot) op_ckpt_swap_out(op, s);
    } else {
      rc = born_rtm_forward(h, op->jt, op->nt, nullptr);
    }
    if (rc) return rc;
    // data += deriv(map_data(traces)) (rtm_zero_op_3d.cc:187-193)
    k_map_fwd<<<grid_for(op->shot_n), kThreads, 0, h->stream>>>(
        h->rec.traces, op->shot_tmp, p.nt_data, ntr, op->nt_big, 0);
    k_deriv_fwd<<<grid_for(ntr), kThreads, 0, h->stream>>>(
        op->shot_tmp, op->traces_tmp, p.nt_data, p.rec_nx, p.rec_ny,
        p.dt_data, 0);
    k_add<<<grid_for(op->shot_n), kThreads, 0, h->stream>>>(
        data + (long long)s * op->shot_n, op->traces_tmp, op->shot_n);
    OPCK(op, cudaGetLastError());
    h->launches += 3;
  }
  return born_check_device_error(h);
}

int born_op_adjoint(born_op *op, int add, float *model, const float *data) {
  if (!op || !model || !data) return BORN_EINVAL;
  born_handle *h = op->h;
  int rc = born_check_ready(h);
  if (rc) return rc;
  const born_op_params &p = op->p;
  const long long n123 = h->n123, n12 = (long long)h->n1 * h->n2;
  const int ntr = p.rec_nx * p.rec_ny;
  if (!add) OPCK(op, cudaMemsetAsync(model, 0, op->model_n * 4, h->stream));
  for (int s = 0; s < p.nshots; ++s) {
    rc = op_select_shot(op, s);
    if (rc) return rc;
    // traces = map_data'(deriv'(data)) (rtm_zero_op_3d.cc:265-271)
    k_deriv_adj<<<grid_for(ntr), kThreads, 0, h->stream>>>(
        op->shot_tmp, data + (long long)s * op->shot_n, p.nt_data, p.rec_nx,
        p.rec_ny, p.dt_data, 0);
    k_map_adj<<<grid_for((long long)ntr * op->nt_big), kThreads, 0,
                h->stream>>>(h->rec.traces, op->shot_tmp, p.nt_data, ntr,
                             op->nt_big, 0);
    OPCK(op, cudaGetLastError());
    h->launches += 2;
    if (p.exact) {
      const bool slot = op_ckpt_swap_in(op, s);
      rc = born_lin_adjoint(h, op->jt, op->nt,
                            p.ckpt_interval > 0 ? p.ckpt_interval : 50,
                            nullptr);
      if (slot) {
        if (h->ckpt_reused) op->ckpt_reused_shots++;
        op_ckpt_swap_out(op, s);
      }
    } else {
      rc = born_source_prop(h, op->jt, op->nt, nullptr, nullptr);
      if (!rc) rc = born_rtm_adjoint(h, op->jt, op->nt, 1, nullptr);
    }
    if (rc) return rc;
    // model += window'(laplac'(img)) (rtm_zero_op_3d.cc:289-295)
    k_laplac_adj<<<grid_for(n123), kThreads, 0, h->stream>>>(h->refl, h->img,
                                                             n12, n123, 0);
    k_add_window<<<grid_for(n123), kThreads, 0, h->stream>>>(
        model, p.n1, p.n2, p.n3, h->refl, h->n1, h->n2, h->n3, op->w1, op->w2,
        op->w3);
    OPCK(op, cudaGetLastError());
    h->launches += 2;
    h->have_refl = false;
  }
  return born_check_device_error(h);
}

int born_dot_f64(born_op *op, const float *a, const float *b, long long n,
                 double *out) {
  if (!op || !a || !b || !out || n < 0) return BORN_EINVAL;
  return op_dot(op, a, b, n, out);
}

// ---- device vectors for host code that holds them in my_vector objects
// (born_my_operator.h); every call is ordered on the operator's stream ----

namespace {
int vec_ready(born_op *op, long long n) {
  if (!op || n < 0) return BORN_EINVAL;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return BORN_ECUDA;
  if (dev != op->h->device && cudaSetDevice(op->h->device) != cudaSuccess)
    return born_fail(op->h, BORN_ECUDA, "cannot select the operator's device");
  return BORN_OK;
}
int vec_launched(born_op *op) {
  op->h->launches++;
  OPCK(op, cudaGetLastError());
  return BORN_OK;
}
}  // namespace

int born_vec_create(born_op *op, long long n, float **out) {
  int rc = vec_ready(op, n);
  if (rc) return rc;
  if (!out) return BORN_EINVAL;
  *out = nullptr;
  float *x = nullptr;
  if (cudaMalloc(&x, (size_t)std::max<long long>(n, 1) * 4) != cudaSuccess)
    return born_fail(op->h, BORN_ENOMEM, "born_vec_create: %lld floats", n);
  if (cudaMemsetAsync(x, 0, (size_t)n * 4, op->h->stream) != cudaSuccess) {
    cudaFree(x);
    return born_fail(op->h, BORN_ECUDA, "born_vec_create: clear failed");
  }
  *out = x;
  return BORN_OK;
}

int born_vec_destroy(born_op *op, float *x) {
  int rc = vec_ready(op, 0);
  if (rc) return rc;
  if (!x) return BORN_OK;
  // work queued on the stream may still read or write x
  OPCK(op, cudaStreamSynchronize(op->h->stream));
  OPCK(op, cudaFree(x));
  return BORN_OK;
}

int born_vec_fill(born_op *op, float *x, long long n, double val) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!x) return BORN_EINVAL;
  k_fill<<<grid_for(n), kThreads, 0, op->h->stream>>>(x, (float)val, n);
  return vec_launched(op);
}

int born_vec_scale(born_op *op, float *x, long long n, double r) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!x) return BORN_EINVAL;
  k_scale<<<grid_for(n), kThreads, 0, op->h->stream>>>(x, r, n);
  return vec_launched(op);
}

int born_vec_scale_add(born_op *op, float *x, double a, const float *y,
                       double b, long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!x || !y) return BORN_EINVAL;
  k_scale_add<<<grid_for(n), kThreads, 0, op->h->stream>>>(x, a, y, b, n);
  return vec_launched(op);
}

int born_vec_lincomb(born_op *op, float *x, double a, const float *y,
                     double b, const float *z, long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!x || !y || !z) return BORN_EINVAL;
  k_lincomb<<<grid_for(n), kThreads, 0, op->h->stream>>>(x, a, y, b, z, n);
  return vec_launched(op);
}

int born_vec_add(born_op *op, float *x, const float *y, long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!x || !y) return BORN_EINVAL;
  k_add<<<grid_for(n), kThreads, 0, op->h->stream>>>(x, y, n);
  return vec_launched(op);
}

int born_vec_copy(born_op *op, float *dst, const float *src, long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!dst || !src) return BORN_EINVAL;
  OPCK(op, cudaMemcpyAsync(dst, src, (size_t)n * 4, cudaMemcpyDeviceToDevice,
                           op->h->stream));
  return BORN_OK;
}

int born_vec_upload(born_op *op, float *dst, const float *host, long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!dst || !host) return BORN_EINVAL;
  OPCK(op, cudaMemcpyAsync(dst, host, (size_t)n * 4, cudaMemcpyHostToDevice,
                           op->h->stream));
  OPCK(op, cudaStreamSynchronize(op->h->stream));
  return BORN_OK;
}

int born_vec_download(born_op *op, float *host, const float *src,
                      long long n) {
  int rc = vec_ready(op, n);
  if (rc || n == 0) return rc;
  if (!host || !src) return BORN_EINVAL;
  OPCK(op, cudaMemcpyAsync(host, src, (size_t)n * 4, cudaMemcpyDeviceToHost,
                           op->h->stream));
  OPCK(op, cudaStreamSynchronize(op->h->stream));
  return BORN_OK;
}

// Claerbout CG (lin_solver.cc:104-132 with cgstep.cc:11-54):
//   rr = L m - d; per iteration g = L' rr, gg = L g, then the cgstep update.
int born_cg_solve(born_op *op, const float *data, float *model, int niter,
                  double *resid) {
  if (!op || !data || !model || niter < 0) return BORN_EINVAL;
  born_handle *h = op->h;
  const long long nm = op->model_n, nd = op->data_n;
  float *rr = nullptr, *g = nullptr, *gg = nullptr, *s = nullptr,
        *ss = nullptr;
  auto cleanup = [&]() {
    cudaFree(rr);
    cudaFree(g);
    cudaFree(gg);
    cudaFree(s);
    cudaFree(ss);
  };
  if (cudaMalloc(&rr, nd * 4) || cudaMalloc(&gg, nd * 4) ||
      cudaMalloc(&ss, nd * 4) || cudaMalloc(&g, nm * 4) ||
      cudaMalloc(&s, nm * 4)) {
    cleanup();
    return born_fail(h, BORN_ENOMEM, "born_cg_solve: allocation failed");
  }
  // init_rr (lin_solver.cc:91-95): rr = -d + L m0
  int rc = born_op_forward(op, 0, model, rr);
  if (!rc) {
    k_scale_add<<<grid_for(nd), kThreads, 0, h->stream>>>(rr, 1.0, data, -1.0,
                                                          nd);
    cudaMemsetAsync(s, 0, nm * 4, h->stream);
    cudaMemsetAsync(ss, 0, nd * 4, h->stream);
    h->launches++;
  }
  double rr_rr = 0;
  if (!rc) rc = op_dot(op, rr, rr, nd, &rr_rr);
  if (!rc && resid) resid[0] = rr_rr;
  const double small = 1e-20;  // cgstep.h:18
  bool forget = true;
  for (int iter = 0; iter < niter && !rc; ++iter) {
    rc = born_op_adjoint(op, 0, g, rr);
    if (!rc) rc = born_op_forward(op, 0, g, gg);
    if (rc) break;
    double alfa, beta;
    double gg_gg, gg_rr;
    rc = op_dot(op, gg, gg, nd, &gg_gg);
    if (!rc) rc = op_dot(op, gg, rr, nd, &gg_rr);
    if (rc) break;
    if (forget) {
      if (std::fabs(gg_gg) < small) {
        rc = born_fail(h, BORN_ESTATE, "cg: gg.gg vanished");
        break;
      }
      beta = 0;
      alfa = -gg_rr / gg_gg;
    } else {
      double ss_ss, gg_ss, ss_rr;
      rc = op_dot(op, ss, ss, nd, &ss_ss);
      if (!rc) rc = op_dot(op, gg, ss, nd, &gg_ss);
      if (!rc) rc = op_dot(op, ss, rr, nd, &ss_rr);
      if (rc) break;
      if (std::fabs(gg_gg) < small || std::fabs(ss_ss) < small) {
        rc = born_fail(h, BORN_ESTATE, "cg: gg.gg or ss.ss vanished");
        break;
      }
      const double determ =
          gg_gg * ss_ss * (1.0 - gg_ss / gg_gg * gg_ss / ss_ss);
      const double ggr = -gg_rr, ssr = -ss_rr;
      alfa = (ss_ss * ggr - gg_ss * ssr) / determ;
      beta = (-gg_ss * ggr + gg_gg * ssr) / determ;
    }
    k_scale_add<<<grid_for(nm), kThreads, 0, h->stream>>>(s, beta, g, alfa,
                                                          nm);
    k_scale_add<<<grid_for(nd), kThreads, 0, h->stream>>>(ss, beta, gg, alfa,
                                                          nd);
    k_add<<<grid_for(nm), kThreads, 0, h->stream>>>(model, s, nm);
    k_add<<<grid_for(nd), kThreads, 0, h->stream>>>(rr, ss, nd);
    h->launches += 4;
    if (cudaGetLastError() != cudaSuccess) {
      rc = born_fail(h, BORN_ECUDA, "cg: vector update failed");
      break;
    }
    rc = op_dot(op, rr, rr, nd, &rr_rr);
    if (!rc && resid) resid[iter + 1] = rr_rr;
    forget = false;
  }
  cudaStreamSynchronize(h->stream);
  cleanup();
  return rc;
}

}  // extern "C"
