/*
 * Oracle for the Born / RTM hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU propagator (base/cpu_prop.cc)
 * and of the host-side geometry that feeds it (base/sinc_bob.cc,
 * base/fd_prop_3d.cc, base/source_func_3d.cc, base/map_data_3d.cc,
 * base/data_rtm_3d.cc, base/vel_fd_3d.cc, base/laplac_3d.cc,
 * base/deriv_3d.cc, base/image_rtm_3d.cc).  It exists to check the CUDA
 * product against; nothing in the product links or calls it.  The float
 * instance keeps the reference's operation order; the double instance is the
 * FP64 accuracy oracle.
 *
 * Pinning: the propagator and the sinc tables are checked bit for bit
 * against the reference's own cpu_prop.cc / sinc_bob.cc compiled from source
 * (oracle/Makefile -> oracle/_ref), through the fixtures in tests/golden.
 * The geometry helpers sit in files that need the SEP hypercube/genericIO
 * libraries, which are not available, so they are restated from the source
 * text only.
 */
#ifndef BORN_ORACLE_H
#define BORN_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_NBOUND 40

typedef struct {
  int nx, ny, nz;
  long long n123;
  float coeffs[13];
  float bound[ORACLE_NBOUND];
  int nsinc_s, jt_s;
  const float *table_s; /* jt_s rows x nsinc_s */
  int nsinc_d, jt_d;
  const float *table_d;
  int npts_s, nt_src;
  const int *locs_s;
  const float *source; /* npts_s x nt_src */
  int nrec, nt_rec;
  const int *locs_r;
  float *rec; /* nrec x nt_rec, read by injection, accumulated by extraction */
  const float *vel1, *vel2;
  int dir, jt;
} oracle_propf;

typedef struct {
  int nx, ny, nz;
  long long n123;
  double coeffs[13];
  double bound[ORACLE_NBOUND];
  int nsinc_s, jt_s;
  const double *table_s;
  int nsinc_d, jt_d;
  const double *table_d;
  int npts_s, nt_src;
  const int *locs_s;
  const double *source;
  int nrec, nt_rec;
  const int *locs_r;
  double *rec;
  const double *vel1, *vel2;
  int dir, jt;
} oracle_propd;

/* ---- propagator state (cpuProp setters) ---- */
void oracle_create_space(oracle_propf *s, float d1, float d2, float d3, int nx,
                         int ny, int nz);
void oracle_create_space_d(oracle_propd *s, float d1, float d2, float d3,
                           int nx, int ny, int nz);
int oracle_num_threads(void);
void oracle_set_num_threads(int n);

/* ---- float (parity) oracle, base/cpu_prop.cc ---- */
void oracle_prop_stepf(const oracle_propf *s, float *p0, const float *p1,
                       const float *vel);
void oracle_dampf(const oracle_propf *s, float *p0, float *p1);
void oracle_inject_sourcef(const oracle_propf *s, int id, int ii, float *p);
void oracle_inject_receiversf(const oracle_propf *s, int id, int ii, float *p);
void oracle_data_extractf(const oracle_propf *s, int id, int ii,
                          const float *p);
void oracle_image_addf(const oracle_propf *s, const float *img,
                       float *rec_field, const float *src_field);
void oracle_image_conditionf(const oracle_propf *s, const float *rec,
                             const float *src, float *img);
void oracle_source_propf(oracle_propf *s, float *p0, float *p1, int jts,
                         int nt);
void oracle_rtm_adjointf(oracle_propf *s, float *src_p0, float *src_p1,
                         float *img, int jtd, int nt);
void oracle_rtm_forwardf(oracle_propf *s, int jt, const float *img,
                         float *rec, int nt);

/* nonlinear modelling and its exact linearisation (no reference
 * counterpart; built from the same primitives, see oracle_prop_impl.h) */
void oracle_modelf(oracle_propf *s, int jt, float *rec, int nt);
void oracle_lin_forwardf(oracle_propf *s, int jt, const float *m, float *rec,
                         int nt);
void oracle_modeld(oracle_propd *s, int jt, double *rec, int nt);
void oracle_lin_forwardd(oracle_propd *s, int jt, const double *m,
                         double *rec, int nt);
/* exact adjoint of oracle_lin_forward: mbar (n123) from traces rec */
void oracle_lin_adjointf(oracle_propf *s, int jt, const float *rec,
                         float *mbar, int nt);
void oracle_lin_adjointd(oracle_propd *s, int jt, const double *rec,
                         double *mbar, int nt);

/* ---- double (accuracy) oracle ---- */
void oracle_source_propd(oracle_propd *s, double *p0, double *p1, int jts,
                         int nt);
void oracle_rtm_adjointd(oracle_propd *s, double *src_p0, double *src_p1,
                         double *img, int jtd, int nt);
void oracle_rtm_forwardd(oracle_propd *s, int jt, const double *img,
                         double *rec, int nt);

/* ---- geometry (restated; see header comment) ---- */
/* sinc_bob(nt, ns).table flattened: ntab rows x nsinc (base/sinc_bob.cc:4-100) */
void oracle_sinc_table(int ntab, int nsinc, float *out);
/* fd_prop::calc_stability (base/fd_prop_3d.cc:6-33): returns dt, sets *nt */
float oracle_calc_stability(float vmax, float dmin, float dt_data,
                            int nt_data, int *nt_out);
/* source_func::set_compute_size (base/source_func_3d.cc:4-61) for one axis */
int oracle_compute_size(int n_model, int nbound, int fat);
/* wavelet_source_func::get_source_func (base/source_func_3d.cc:76-109) */
void oracle_source_geometry(float sx, float sy, float sz, float o1, float o2,
                            float o3, float d1, float d2, float d3, int n1,
                            int n2, const float *wavelet, int nt_wav, int nts,
                            int *locs, float *vals);
/* wavelet ctor time derivative (base/source_func_3d.cc:120-124) */
void oracle_wavelet_deriv(const float *raw, int nt, float dt, float *out);
/* data_rtm_3d::get_source_func + map_data ctor (data_rtm_3d.cc:79-88,
 * map_data_3d.cc:4-35): receiver linear indices on the compute grid */
void oracle_receiver_geometry(int rec_nx, int rec_ny, float rx0, float rdx,
                              float ry0, float rdy, float rz, float o1,
                              float o2, float o3, float d1, float d2, float d3,
                              int n1, int n2, int *locs);
/* vel_fd_3d::rand_subspace (base/vel_fd_3d.cc:29-134), single-threaded in
 * (iz, iy, ix) order so the rand() stream is deterministic. */
void oracle_rand_subspace(const float *vel, int vn1, int vn2, int vn3,
                          float vo1, float vo2, float vo3, float vd1,
                          float vd2, float vd3, float vmax, int irand,
                          int nrand1, int nrand2, int nrand3, float dt, int n1,
                          int n2, int n3, float o1, float o2, float o3,
                          float d1, float d2, float d3, float *out);
/* laplac forward/adjoint (base/laplac_3d.cc:4-105): first difference in z */
void oracle_laplac_forward(int add, const float *m, float *d, int n1, int n2,
                           int n3);
void oracle_laplac_adjoint(int add, float *m, const float *d, int n1, int n2,
                           int n3);
/* deriv forward/adjoint (base/deriv_3d.cc:4-56): time first difference */
void oracle_deriv_forward(int add, const float *m, float *d, int n1, int n2,
                          int n3, float d1);
void oracle_deriv_adjoint(int add, float *m, const float *d, int n1, int n2,
                          int n3, float d1);
/* map_data forward/adjoint (base/map_data_3d.cc:37-75) */
void oracle_map_data_forward(int add, const float *m, float *d, int nt,
                             int n2, int n3, int ntb);
void oracle_map_data_adjoint(int add, float *m, const float *d, int nt,
                             int n2, int n3, int ntb);
/* image window (base/image_rtm_3d.cc:24-95): f1..f3 = sub-grid origin in
 * whole-image samples; extract writes sub, add accumulates into whole. */
void oracle_extract_sub(const float *whole, int w1, int w2, int w3, float *sub,
                        int s1, int s2, int s3, int f1, int f2, int f3);
void oracle_add_image(float *whole, int w1, int w2, int w3, const float *sub,
                      int s1, int s2, int s3, int f1, int f2, int f3);
/* window offset of one axis from the axes' origins and the whole image's
 * spacing (base/image_rtm_3d.cc:33-35, :64-66): float, truncated */
int oracle_window_offset(float o_sub, float o_whole, float d_whole);

#ifdef __cplusplus
}
#endif
#endif
