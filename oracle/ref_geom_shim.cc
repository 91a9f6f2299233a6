/*
 * extern "C" wrapper around the reference's own geometry and glue code of
 * the Born / RTM path, compiled from where it lies (oracle/Makefile, output
 * oracle/_ref/libref_geom.so): vel_fd_3d::rand_subspace, source_func::
 * set_compute_size / wavelet_source_func (wavelet derivative and source
 * points), map_data (receiver cells, trace lead), fd_prop::calc_stability
 * (FD time step and step count), image_rtm_3d's window (extract_sub,
 * add_image), laplac and deriv.  Test
 * infrastructure only: used to pin the oracle's restatement of these pieces
 * and to generate golden fixtures.  The reference reads its arrays through
 * SEP files; here they are in-memory arrays registered with the stand-in
 * genericIO (ref_stubs/genericIO.h).  The reference's out-of-core vector
 * (oc_float) is backed by files in the reference; its two members the
 * wavelet reader needs are given in-memory bodies below, the others are
 * never called here and abort.
 */
#include <fcntl.h>
#include <unistd.h>

#include <cstdlib>
#include <memory>
#include <vector>

#include "data_rtm_3d.h"
#include "deriv_3d.h"
#include "fd_prop_3d.h"
#include "float_3d.h"
#include "image_rtm_3d.h"
#include "laplac_3d.h"
#include "map_data_3d.h"
#include "source_func_3d.h"
#include "vel_fd_3d.h"

// ---------------------------------------------------------------------------
// oc_float members (file-backed in the reference)

void oc_float::tagInit(std::string tag) {
  _tag = tag;
  _file = _io->getRegFile(tag, SEP::usageIn);
}
void oc_float::readAll(std::shared_ptr<hypercube_float> h) {
  _file->readFloatStream(h->vals, h->getN123());
}
// a "new" file is the in-memory file registered under the tag beforehand
void oc_float::initNewFile(std::string tag, std::shared_ptr<SEP::genericIO> io,
                           std::shared_ptr<SEP::hypercube>,
                           const SEP::usage_code usage) {
  _io = io;
  _tag = tag;
  _file = _io->getRegFile(tag, usage);
}
#define ORACLE_NOT_USED std::abort()
std::shared_ptr<my_vector> oc_float::clone_vec() { ORACLE_NOT_USED; }
std::shared_ptr<my_vector> oc_float::clone_space() { ORACLE_NOT_USED; }
double oc_float::dot(std::shared_ptr<my_vector>) { ORACLE_NOT_USED; }
void oc_float::scale_add(const double, std::shared_ptr<my_vector>,
                         const double) {
  ORACLE_NOT_USED;
}
void oc_float::add(std::shared_ptr<my_vector>) { ORACLE_NOT_USED; }
void oc_float::random() { ORACLE_NOT_USED; }
void oc_float::scale(double) { ORACLE_NOT_USED; }
void oc_float::mult(std::shared_ptr<my_vector>) { ORACLE_NOT_USED; }
double oc_float::sum() { ORACLE_NOT_USED; }
void oc_float::scale_add(const double, std::shared_ptr<my_vector>, double,
                         std::shared_ptr<my_vector>) {
  ORACLE_NOT_USED;
}
double oc_float::my_min() { ORACLE_NOT_USED; }
double oc_float::my_max() { ORACLE_NOT_USED; }
bool oc_float::check_match(const std::shared_ptr<my_vector>) {
  ORACLE_NOT_USED;
}
void oc_float::set_val(double) { ORACLE_NOT_USED; }
void oc_float::info(char *, int) { ORACLE_NOT_USED; }

namespace {
// The reference prints progress on stderr; keep test output clean.
struct QuietStderr {
  int saved = -1;
  QuietStderr() {
    fflush(stderr);
    saved = dup(2);
    int fd = open("/dev/null", O_WRONLY);
    if (fd >= 0) {
      dup2(fd, 2);
      close(fd);
    }
  }
  ~QuietStderr() {
    if (saved < 0) return;
    fflush(stderr);
    dup2(saved, 2);
    close(saved);
  }
};

std::vector<SEP::axis> axes3(int n1, int n2, int n3, float o1 = 0.f,
                             float o2 = 0.f, float o3 = 0.f, float d1 = 1.f,
                             float d2 = 1.f, float d3 = 1.f) {
  return {SEP::axis(n1, o1, d1), SEP::axis(n2, o2, d2), SEP::axis(n3, o3, d3)};
}

std::shared_ptr<float_3d> f3(int n1, int n2, int n3, float d1 = 1.f) {
  auto v = std::make_shared<float_3d>(SEP::axis(n1, 0.f, d1), SEP::axis(n2),
                                      SEP::axis(n3));
  for (long long i = 0; i < (long long)n1 * n2 * n3; ++i) v->vals[i] = 0.f;
  return v;
}
}  // namespace

extern "C" {

// source_func::set_compute_size: the padded compute-grid size of one axis
int ref_geom_compute_size(int n_model, int nbound, int fat) {
  source_func s;
  auto dom = std::make_shared<SEP::hypercube>(
      axes3(n_model, n_model, n_model));
  s.set_compute_size(dom, 0.f, nbound, nbound, nbound, fat, 16);
  return s.ax.n;
}

// vel_fd_3d::rand_subspace of a model velocity onto a compute grid
int ref_geom_rand_subspace(const float *vel, int vn1, int vn2, int vn3,
                           float vo1, float vo2, float vo3, float vd1,
                           float vd2, float vd3, int irand, int nrand1,
                           int nrand2, int nrand3, float dt, int n1, int n2,
                           int n3, float o1, float o2, float o3, float d1,
                           float d2, float d3, float *out) {
  QuietStderr q;
  SEP::genericIO::register_file(
      "oracle_vel", axes3(vn1, vn2, vn3, vo1, vo2, vo3, vd1, vd2, vd3), vel);
  auto io = std::make_shared<SEP::genericIO>();
  vel_fd_3d v(io, "oracle_vel");
  auto space = std::make_shared<hypercube_float>(
      axes3(n1, n2, n3, o1, o2, o3, d1, d2, d3));
  auto r = v.rand_subspace(irand, nrand1, nrand2, nrand3, dt, space);
  for (long long i = 0; i < (long long)n1 * n2 * n3; ++i) out[i] = r->vals[i];
  return 0;
}

// wavelet_source_func: time derivative of a raw wavelet (its io
// constructor) and the source points and traces of one shot
int ref_geom_source(const float *raw, int nt_wav, float dt_wav, float sx,
                    float sy, float sz, float o1, float o2, float o3, float d1,
                    float d2, float d3, int n1, int n2, int n3, int nts,
                    int *locs, float *vals) {
  SEP::genericIO::register_file("oracle_wavelet",
                                {SEP::axis(nt_wav, 0.f, dt_wav)}, raw);
  auto io = std::make_shared<SEP::genericIO>();
  wavelet_source_func w(io, "oracle_wavelet");
  w.sx.push_back(sx);
  w.sy.push_back(sy);
  w.sz.push_back(sz);
  auto dom = std::make_shared<hypercube_float>(
      axes3(n1, n2, n3, o1, o2, o3, d1, d2, d3));
  std::vector<int> l(9);
  std::vector<float> t((size_t)nts * 9);
  w.get_source_func(dom, 0, nts, l, t);
  for (int i = 0; i < 9; ++i) locs[i] = l[i];
  for (size_t i = 0; i < t.size(); ++i) vals[i] = t[i];
  return 0;
}

// data_rtm_3d::get_source_func (receiver positions of a rec_nx x rec_ny
// surface grid in compute-grid units) followed by the map_data constructor
// (their cells)
int ref_geom_receivers(int rec_nx, int rec_ny, float rx0, float rdx,
                       float ry0, float rdy, float rz, float o1, float o2,
                       float o3, float d1, float d2, float d3, int n1, int n2,
                       int n3, int nt, int *locs) {
  const int npt = rec_nx * rec_ny;
  std::vector<float> zeros((size_t)nt * npt, 0.f);
  SEP::genericIO::register_file(
      "oracle_data",
      {SEP::axis(nt), SEP::axis(rec_nx, rx0, rdx), SEP::axis(rec_ny, ry0, rdy)},
      zeros.data());
  data_rtm_3d dr;
  dr._io = std::make_shared<SEP::genericIO>();
  dr.tagInit("oracle_data");
  dr.sz = rz;
  auto dom = std::make_shared<hypercube_float>(
      axes3(n1, n2, n3, o1, o2, o3, d1, d2, d3));
  auto time = std::make_shared<hypercube_float>(
      std::vector<SEP::axis>{SEP::axis(nt), SEP::axis(rec_nx),
                             SEP::axis(rec_ny)});
  std::vector<float> sx(npt), sy(npt), sz(npt);
  dr.get_source_func(dom, 0, sx, sy, sz, 8, nt, time);
  std::vector<int> l(npt);
  auto dummy = std::make_shared<hypercube_float>(axes3(1, 1, 1));
  map_data m(npt, sx, sy, sz, l, dom, dummy, dummy, nt + 8);
  for (int i = 0; i < npt; ++i) locs[i] = l[i];
  return 0;
}

// fd_prop::calc_stability: FD time step and step count from the data
// sampling and the velocity model's maximum and spacing
int ref_geom_calc_stability(const float *vel, int vn1, int vn2, int vn3,
                            float vd1, float vd2, float vd3, float dt_data,
                            int nt_data, float *dt_out, int *nt_out) {
  QuietStderr q;
  SEP::genericIO::register_file(
      "oracle_vel", axes3(vn1, vn2, vn3, 0.f, 0.f, 0.f, vd1, vd2, vd3), vel);
  fd_prop fp;
  fp.vel = std::make_shared<vel_fd_3d>(std::make_shared<SEP::genericIO>(),
                                       "oracle_vel");
  std::vector<float> ds{dt_data};
  fp.calc_stability(ds, nt_data);
  *dt_out = fp.dt;
  *nt_out = fp.nt;
  return 0;
}

// map_data constructor: receiver cells from fractional grid coordinates
int ref_geom_map_locs(int npt, const float *fx, const float *fy,
                      const float *fz, int n1, int n2, int *locs) {
  std::vector<float> x(fx, fx + npt), y(fy, fy + npt), z(fz, fz + npt);
  std::vector<int> l(npt);
  auto model = std::make_shared<hypercube_float>(axes3(n1, n2, 1));
  auto dummy = std::make_shared<hypercube_float>(axes3(1, 1, 1));
  map_data m(npt, x, y, z, l, model, dummy, dummy, 8);
  for (int i = 0; i < npt; ++i) locs[i] = l[i];
  return 0;
}

// map_data forward / adjoint: traces [n3][n2][ntb] with the 4-sample lead
// <-> data [n3][n2][nt]
int ref_geom_map_data(int adjoint, int add, float *m, float *d, int nt,
                      int n2, int n3, int ntb) {
  auto dummy = std::make_shared<hypercube_float>(axes3(1, 1, 1));
  map_data op;
  op.ntb = ntb;
  auto mv = f3(ntb, n2, n3), dv = f3(nt, n2, n3);
  for (long long i = 0; i < (long long)ntb * n2 * n3; ++i) mv->vals[i] = m[i];
  for (long long i = 0; i < (long long)nt * n2 * n3; ++i) dv->vals[i] = d[i];
  if (adjoint)
    op.adjoint(add != 0, mv, dv);
  else
    op.forward(add != 0, mv, dv);
  for (long long i = 0; i < (long long)ntb * n2 * n3; ++i) m[i] = mv->vals[i];
  for (long long i = 0; i < (long long)nt * n2 * n3; ++i) d[i] = dv->vals[i];
  (void)dummy;
  return 0;
}

// laplac (first difference along axis 3) forward / adjoint on n3 x n2 x n1
int ref_geom_laplac(int adjoint, int add, float *m, float *d, int n1, int n2,
                    int n3) {
  auto mv = f3(n1, n2, n3), dv = f3(n1, n2, n3);
  const long long n = (long long)n1 * n2 * n3;
  for (long long i = 0; i < n; ++i) {
    mv->vals[i] = m[i];
    dv->vals[i] = d[i];
  }
  laplac op(mv, dv);
  if (adjoint)
    op.adjoint(add != 0, mv, dv);
  else
    op.forward(add != 0, mv, dv);
  for (long long i = 0; i < n; ++i) {
    m[i] = mv->vals[i];
    d[i] = dv->vals[i];
  }
  return 0;
}

// deriv (time first difference / d1) forward / adjoint on n3 x n2 x n1
int ref_geom_deriv(int adjoint, int add, float *m, float *d, int n1, int n2,
                   int n3, float d1) {
  auto mv = f3(n1, n2, n3, d1), dv = f3(n1, n2, n3, d1);
  const long long n = (long long)n1 * n2 * n3;
  for (long long i = 0; i < n; ++i) {
    mv->vals[i] = m[i];
    dv->vals[i] = d[i];
  }
  deriv op(mv, dv);
  if (adjoint)
    op.adjoint(add != 0, mv, dv);
  else
    op.forward(add != 0, mv, dv);
  for (long long i = 0; i < n; ++i) {
    m[i] = mv->vals[i];
    d[i] = dv->vals[i];
  }
  return 0;
}

// image_rtm_3d::extract_sub (extract != 0: whole -> sub) or add_image
// (whole += sub) for a window given by its axes; the whole image's axes are
// those of the velocity file, as in the image_rtm_3d constructor
int ref_geom_image_window(int extract, float *whole, int w1, int w2, int w3,
                          float wo1, float wo2, float wo3, float wd1,
                          float wd2, float wd3, float *sub, int s1, int s2,
                          int s3, float so1, float so2, float so3, float sd1,
                          float sd2, float sd3) {
  QuietStderr q;
  const auto wax = axes3(w1, w2, w3, wo1, wo2, wo3, wd1, wd2, wd3);
  SEP::genericIO::register_file("oracle_image_vel", wax, whole);
  SEP::genericIO::register_file("oracle_image", wax, whole);
  auto io = std::make_shared<SEP::genericIO>();
  auto v = std::make_shared<vel_fd_3d>(io, "oracle_image_vel");
  image_rtm_3d img(io, "oracle_image", v);
  const long long nw = (long long)w1 * w2 * w3, ns = (long long)s1 * s2 * s3;
  if (extract) {
    auto out = img.extract_sub(SEP::axis(s1, so1, sd1), SEP::axis(s2, so2, sd2),
                               SEP::axis(s3, so3, sd3));
    for (long long i = 0; i < ns; ++i) sub[i] = out->vals[i];
  } else {
    for (long long i = 0; i < nw; ++i) img.image->vals[i] = whole[i];
    auto part = std::make_shared<hypercube_float>(
        axes3(s1, s2, s3, so1, so2, so3, sd1, sd2, sd3));
    for (long long i = 0; i < ns; ++i) part->vals[i] = sub[i];
    img.add_image(part);
    for (long long i = 0; i < nw; ++i) whole[i] = img.image->vals[i];
  }
  return 0;
}

}  // extern "C"
