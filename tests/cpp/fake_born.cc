// Host stand-in for the part of libborn_gb300's C ABI that
// csrc/born_my_operator.h calls (born_op_*, born_vec_*, born_dot_f64), for a
// CPU check of the adapter under the reference's own solver classes where
// no GPU is present.  The "device" vectors are host arrays and the operator
// is a fixed dense matrix; only the adapter's plumbing is under test here,
// the GPU operator itself is tested against the oracle elsewhere.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "born_gb300.h"

struct born_handle {
  int device;
};
struct born_op {
  long long nm = 0, nd = 0;
  std::vector<float> a;  // nd x nm
};

extern "C" {

int born_create(int device, born_handle **out) {
  *out = new born_handle{device};
  return BORN_OK;
}
int born_destroy(born_handle *h) {
  delete h;
  return BORN_OK;
}
const char *born_error_string(const born_handle *) { return ""; }

int born_op_create(born_handle *, const born_op_params *p, const float *,
                   const float *, const float *, born_op **out) {
  born_op *op = new born_op();
  op->nm = (long long)p->n1 * p->n2 * p->n3;
  op->nd = (long long)p->nshots * p->rec_nx * p->rec_ny * p->nt_data;
  op->a.resize((size_t)(op->nm * op->nd));
  unsigned s = 4321u;
  for (auto &x : op->a) {
    s = s * 1103515245u + 12345u;
    x = (float)((s >> 8) & 0xffff) / 65536.f - .5f;
  }
  *out = op;
  return BORN_OK;
}
int born_op_destroy(born_op *op) {
  delete op;
  return BORN_OK;
}
int born_op_sizes(const born_op *op, long long *mn, long long *dn, int *nt,
                  float *dt) {
  *mn = op->nm;
  *dn = op->nd;
  *nt = 0;
  *dt = 0.f;
  return BORN_OK;
}
int born_op_forward(born_op *op, int add, const float *m, float *d) {
  for (long long i = 0; i < op->nd; ++i) {
    double s = add ? d[i] : 0.0;
    for (long long j = 0; j < op->nm; ++j)
      s += (double)op->a[(size_t)(i * op->nm + j)] * m[j];
    d[i] = (float)s;
  }
  return BORN_OK;
}
int born_op_adjoint(born_op *op, int add, float *m, const float *d) {
  for (long long j = 0; j < op->nm; ++j) {
    double s = add ? m[j] : 0.0;
    for (long long i = 0; i < op->nd; ++i)
      s += (double)op->a[(size_t)(i * op->nm + j)] * d[i];
    m[j] = (float)s;
  }
  return BORN_OK;
}
int born_dot_f64(born_op *, const float *a, const float *b, long long n,
                 double *out) {
  double s = 0;
  for (long long i = 0; i < n; ++i) s += (double)a[i] * (double)b[i];
  *out = s;
  return BORN_OK;
}
int born_cg_solve(born_op *, const float *, float *, int, double *) {
  return BORN_ESTATE;  // not part of the adapter
}
int born_vec_create(born_op *, long long n, float **out) {
  *out = static_cast<float *>(std::calloc((size_t)(n > 0 ? n : 1), 4));
  return *out ? BORN_OK : BORN_ENOMEM;
}
int born_vec_destroy(born_op *, float *x) {
  std::free(x);
  return BORN_OK;
}
int born_vec_fill(born_op *, float *x, long long n, double val) {
  for (long long i = 0; i < n; ++i) x[i] = (float)val;
  return BORN_OK;
}
int born_vec_scale(born_op *, float *x, long long n, double r) {
  for (long long i = 0; i < n; ++i) x[i] = (float)(x[i] * r);
  return BORN_OK;
}
int born_vec_scale_add(born_op *, float *x, double a, const float *y,
                       double b, long long n) {
  for (long long i = 0; i < n; ++i) x[i] = (float)(x[i] * a + y[i] * b);
  return BORN_OK;
}
int born_vec_lincomb(born_op *, float *x, double a, const float *y, double b,
                     const float *z, long long n) {
  for (long long i = 0; i < n; ++i) x[i] = (float)(y[i] * a + z[i] * b);
  return BORN_OK;
}
int born_vec_add(born_op *, float *x, const float *y, long long n) {
  for (long long i = 0; i < n; ++i) x[i] += y[i];
  return BORN_OK;
}
int born_vec_copy(born_op *, float *dst, const float *src, long long n) {
  std::memcpy(dst, src, (size_t)n * 4);
  return BORN_OK;
}
int born_vec_upload(born_op *, float *dst, const float *host, long long n) {
  std::memcpy(dst, host, (size_t)n * 4);
  return BORN_OK;
}
int born_vec_download(born_op *, float *host, const float *src, long long n) {
  std::memcpy(host, src, (size_t)n * 4);
  return BORN_OK;
}

}  // extern "C"
