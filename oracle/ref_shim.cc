/*
 * extern "C" wrapper around the reference's own cpuProp and sinc_bob, built
 * from base/cpu_prop.cc and base/sinc_bob.cc where they lie (oracle/Makefile,
 * output in oracle/_ref).  Test infrastructure only: used to pin the oracle
 * restatement and to generate the golden fixtures in tests/golden.  The
 * reference prints one stderr line per time step; ref_quiet(1) sends fd 2 to
 * /dev/null around the time loops.
 */
#include <fcntl.h>
#include <unistd.h>

#include <memory>
#include <vector>

#include "cpu_prop.h"
#include "sinc_bob.h"

namespace {
int g_quiet = 0;
struct QuietStderr {
  int saved = -1;
  QuietStderr() {
    if (!g_quiet) return;
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
std::vector<std::vector<float>> unflatten(int rows, int cols, const float *t) {
  std::vector<std::vector<float>> out(rows, std::vector<float>(cols));
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) out[r][c] = t[r * cols + c];
  return out;
}
}  // namespace

extern "C" {

void ref_quiet(int q) { g_quiet = q; }

void *ref_create(float d1, float d2, float d3, int nx, int ny, int nz) {
  auto io = std::make_shared<SEP::genericIO>();
  cpuProp *p = new cpuProp(io);
  p->createSpace(d1, d2, d3, 50.f, .0005f, .0005f, nx, ny, nz);
  return p;
}

void ref_destroy(void *h) { delete static_cast<cpuProp *>(h); }

void ref_set_sinc_s(void *h, int nsinc, int jts, const float *flat) {
  auto t = unflatten(jts, nsinc, flat);
  static_cast<cpuProp *>(h)->transferSincTableS(nsinc, jts, t);
}

void ref_set_sinc_d(void *h, int nsinc, int jtd, const float *flat) {
  auto t = unflatten(jtd, nsinc, flat);
  static_cast<cpuProp *>(h)->transferSincTableD(nsinc, jtd, t);
}

void ref_set_source(void *h, int npts, int nt_big, const int *locs,
                    float *vals) {
  std::vector<int> l(locs, locs + npts);
  static_cast<cpuProp *>(h)->transferSourceFunc(npts, nt_big, l, vals);
}

void ref_set_vel1(void *h, int nx, int ny, int nz, float *v) {
  static_cast<cpuProp *>(h)->transferVelFunc1(nx, ny, nz, v);
}

void ref_set_vel2(void *h, int nx, int ny, int nz, float *v) {
  static_cast<cpuProp *>(h)->transferVelFunc2(nx, ny, nz, v);
}

void ref_set_receivers(void *h, int rec_nx, int rec_ny, int nt_big,
                       const int *locs, float *rec) {
  std::vector<int> l(locs, locs + (long long)rec_nx * rec_ny);
  static_cast<cpuProp *>(h)->transferReceiverFunc(rec_nx, rec_ny, nt_big, l,
                                                  rec);
}

void ref_source_prop(void *h, int nx, int ny, int nz, float *p0, float *p1,
                     int jts, int npts, int nt) {
  QuietStderr q;
  static_cast<cpuProp *>(h)->sourceProp(nx, ny, nz, false, true, p0, p1, jts,
                                        npts, nt);
}

void ref_rtm_adjoint(void *h, int n1, int n2, int n3, int jtd, float *p0,
                     float *p1, float *img, int npts, int nt) {
  QuietStderr q;
  static_cast<cpuProp *>(h)->rtmAdjoint(n1, n2, n3, jtd, p0, p1, img, npts,
                                        nt);
}

void ref_rtm_forward(void *h, int n1, int n2, int n3, int jt, float *img,
                     float *rec, int npts, int nt, int nt_big, int rec_nx,
                     int rec_ny) {
  QuietStderr q;
  static_cast<cpuProp *>(h)->rtmForward(n1, n2, n3, jt, img, rec, npts, nt,
                                        nt_big, rec_nx, rec_ny);
}

void ref_prop(void *h, float *p0, float *p1, float *vel) {
  static_cast<cpuProp *>(h)->prop(p0, p1, vel);
}

void ref_damp(void *h, float *p0, float *p1) {
  static_cast<cpuProp *>(h)->damp(p0, p1);
}

void ref_image_add(void *h, float *img, float *rec_field, float *src_field) {
  static_cast<cpuProp *>(h)->imageAdd(img, rec_field, src_field);
}

void ref_image_condition(void *h, float *rec, float *src, float *img) {
  static_cast<cpuProp *>(h)->imageCondition(rec, src, img);
}

void ref_sinc_table(int ntab, int nsinc, float *out) {
  sinc_bob s(ntab, nsinc);
  for (int r = 0; r < ntab; r++)
    for (int c = 0; c < nsinc; c++) out[r * nsinc + c] = s.table[r][c];
}
}
