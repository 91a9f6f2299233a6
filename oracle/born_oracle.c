/*
 * Oracle for the Born / RTM hot path — TEST INFRASTRUCTURE ONLY.
 * See born_oracle.h for what is restated from where and how it is pinned.
 * Build: cc -O2 -fno-fast-math -ffp-contract=off -fopenmp -fPIC -shared
 * (oracle/Makefile).  -ffp-contract=off matters on aarch64, where GCC would
 * otherwise fuse multiply-adds and change the rounding.
 */
#include "born_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* cpuProp::createSpace, base/cpu_prop.cc:296-332.  Coefficients are formed
 * in double and stored as float; the taper table is the hard-coded 40-entry
 * exp(-0.0005 (40 - i)) whatever bc_a / bc_b say (cpu_prop.cc:329-332). */
#define C_C00(d) (8.0 / (5.0 * (double)(d) * (double)(d)))
static void coeff_table(double *c, float d1, float d2, float d3) {
  c[0] = -1025.0 / 576.0 * (C_C00(d1) + C_C00(d2) + C_C00(d3));
  c[1] = C_C00(d1);
  c[2] = C_C00(d2);
  c[3] = C_C00(d3);
  c[4] = -C_C00(d1) / 8.0;
  c[5] = -C_C00(d2) / 8.0;
  c[6] = -C_C00(d3) / 8.0;
  c[7] = C_C00(d1) / 63.0;
  c[8] = C_C00(d2) / 63.0;
  c[9] = C_C00(d3) / 63.0;
  c[10] = -C_C00(d1) / 896.0;
  c[11] = -C_C00(d2) / 896.0;
  c[12] = -C_C00(d3) / 896.0;
}

void oracle_create_space(oracle_propf *s, float d1, float d2, float d3, int nx,
                         int ny, int nz) {
  memset(s, 0, sizeof(*s));
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->n123 = (long long)nx * ny * nz;
  double c[13];
  coeff_table(c, d1, d2, d3);
  for (int i = 0; i < 13; i++) s->coeffs[i] = (float)c[i];
  const float bcb = .0005f, bca = 40.f;
  for (int i = 0; i < ORACLE_NBOUND; i++) s->bound[i] = expf(-bcb * (bca - i));
  s->jt = 1;
  s->jt_s = 1;
  s->jt_d = 1;
}

void oracle_create_space_d(oracle_propd *s, float d1, float d2, float d3,
                           int nx, int ny, int nz) {
  memset(s, 0, sizeof(*s));
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->n123 = (long long)nx * ny * nz;
  coeff_table(s->coeffs, d1, d2, d3);
  for (int i = 0; i < ORACLE_NBOUND; i++)
    s->bound[i] = exp(-0.0005 * (40.0 - i));
  s->jt = 1;
  s->jt_s = 1;
  s->jt_d = 1;
}

#define REAL float
#define SFX f
#include "oracle_prop_impl.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX d
#include "oracle_prop_impl.h"
#undef REAL
#undef SFX

/* ---------------------------------------------------------------------- */
/* sinc_bob (base/sinc_bob.cc:4-100): least-squares tapered sinc (Hale,
 * after Larner), Toeplitz solve in double with float storage.  The C++
 * original calls cos() on float arguments, which resolves to the float
 * overload; cosf() is the C spelling of the same call. */
static void toep(int m, const float *r, float *f, const float *g, float *a) {
  double c, e, v, w, bot;
  a[0] = 1.f;
  v = r[0];
  f[0] = g[0] / r[0];
  for (int j = 1; j < m; j++) {
    e = a[j] = f[j] = 0.f;
    for (int i = 0; i < j; i++) e += a[i] * r[j - i];
    c = e / v;
    v -= e * c;
    int jh = j / 2;
    for (int i = 0; i <= jh; i++) {
      bot = a[j - i] - c * a[i];
      a[i] -= c * a[j - i];
      a[j - i] = bot;
    }
    w = 0;
    for (int i = 0; i < j; i++) w += f[i] * r[j - i];
    c = (g[j] - w) / v;
    for (int i = 0; i <= j; i++) f[i] += c * a[j - i];
  }
}

static void mksinc(float *sinc, int lsinc, float d, float *space) {
  float pi = 3.141592654;
  float pi2 = pi * 2;
  float snyq = 0.5;
  float snat = snyq * (0.066 + 0.265 * log((double)lsinc));
  float s0 = 0.0;
  float ds = (snat - s0) / (lsinc * 2 - 1);
  float eta = lsinc / 2 - 1.0 + d;
  float *b = space, *c = b + lsinc, *work = c + lsinc;
  for (int j = 0; j < lsinc; j++) {
    float s;
    for (s = s0, b[j] = c[j] = 0.0f; s <= snat; s += ds) {
      b[j] += cosf(pi2 * s * j);
      c[j] += cosf(pi2 * s * (eta - j));
    }
  }
  toep(lsinc, b, sinc, c, work);
}

void oracle_sinc_table(int ntab, int nsinc, float *out) {
  float dtab = 1. / (float)ntab;
  float t = 0.f;
  float *junk = (float *)malloc(sizeof(float) * nsinc * 3);
  for (int it = 0; it < ntab; it++, t += dtab) {
    for (int k = 0; k < nsinc; k++) out[it * nsinc + k] = 0.f;
    mksinc(out + it * nsinc, nsinc, t, junk);
  }
  free(junk);
}

/* fd_prop::calc_stability, base/fd_prop_3d.cc:6-33. */
float oracle_calc_stability(float vmax, float dmin, float dt_data,
                            int nt_data, int *nt_out) {
  float d = .47 * dmin / vmax;
  float dt = dt_data / ceilf(dt_data / d);
  if (nt_out) *nt_out = (nt_data - 1) * (int)(dt_data / dt) + 1;
  return dt;
}

/* source_func::set_compute_size, base/source_func_3d.cc:4-34: pad nbound+fat
 * each side, then round up to a multiple of 16. */
int oracle_compute_size(int n_model, int nbound, int fat) {
  int n = n_model + 2 * (nbound + fat);
  int rem = n - (n / 16) * 16;
  if (rem != 0) rem = 16 - rem;
  return n + rem;
}

/* wavelet_source_func::get_source_func, base/source_func_3d.cc:76-109:
 * 3x3 points on the plane iz-1 with Gaussian weights, traces carrying a
 * 4-sample lead. */
void oracle_source_geometry(float sx, float sy, float sz, float o1, float o2,
                            float o3, float d1, float d2, float d3, int n1,
                            int n2, const float *wavelet, int nt_wav, int nts,
                            int *locs, float *vals) {
  float fz = (sz - o3) / d3 + .5;
  float fy = (sy - o2) / d2 + .5;
  float fx = (sx - o1) / d1 + .5;
  int iy = (int)fy, ix = (int)fx, iz = (int)fz;
  int i = 0;
  for (int it = 0; it < nts * 9; it++) vals[it] = 0;
  int ncopy = nt_wav < nts - 4 ? nt_wav : nts - 4;
  for (int i3 = iz - 1; i3 <= iz - 1; i3++) {
    float zn = fz - i3;
    for (int i2 = iy - 1; i2 <= iy + 1; i2++) {
      float yn = fy - i2;
      for (int i1 = ix - 1; i1 <= ix + 1; i1++, i++) {
        float xn = fx - i1;
        locs[i] = i1 + i2 * n1 + i3 * n1 * n2;
        float scale = expf(-zn * zn - xn * xn - yn * yn);
        for (int it = 0; it < ncopy; it++)
          vals[nts * i + it + 4] = scale * wavelet[it];
      }
    }
  }
}

/* wavelet_source_func ctor, base/source_func_3d.cc:120-124. */
void oracle_wavelet_deriv(const float *raw, int nt, float dt, float *out) {
  out[nt - 1] = 0;
  for (int it = 0; it < nt - 1; it++) out[it] = (raw[it + 1] - raw[it]) / dt;
}

/* data_rtm_3d::get_source_func (data_rtm_3d.cc:79-88) followed by the
 * map_data ctor (map_data_3d.cc:17-31): truncating grid indices. */
void oracle_receiver_geometry(int rec_nx, int rec_ny, float rx0, float rdx,
                              float ry0, float rdy, float rz, float o1,
                              float o2, float o3, float d1, float d2, float d3,
                              int n1, int n2, int *locs) {
  int i = 0;
  for (int i3 = 0; i3 < rec_ny; i3++) {
    for (int i2 = 0; i2 < rec_nx; i2++, i++) {
      float s_z = (rz - o3) / d3;
      float s_x = (rx0 + rdx * i2 - o1) / d1;
      float s_y = (ry0 + rdy * i3 - o2) / d2;
      int ix = (int)s_x, iz = (int)s_z, iy = (int)s_y;
      locs[i] = ix + iy * n1 + iz * n1 * n2;
    }
  }
}

static float taper2(int i, int n, int nr) {
  if (i < nr) return (float)((nr - i) * (nr - i)) / (float)(nr * nr);
  if (i >= n - nr)
    return (float)((i - (n - nr - 1)) * (i - (n - nr - 1))) / (float)(nr * nr);
  return 0;
}

static int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

/* vel_fd_3d::rand_subspace, base/vel_fd_3d.cc:29-134. */
void oracle_rand_subspace(const float *vel, int vn1, int vn2, int vn3,
                          float vo1, float vo2, float vo3, float vd1,
                          float vd2, float vd3, float vmax, int irand,
                          int nrand1, int nrand2, int nrand3, float dt, int n1,
                          int n2, int n3, float o1, float o2, float o3,
                          float d1, float d2, float d3, float *out) {
  srand(irand);
  long long i = 0;
  for (int iz = 0; iz < n3; iz++) {
    int iz_v = clampi((int)((o3 + d3 * iz - vo3) / vd3), 0, vn3 - 1);
    float dz2 = taper2(iz, n3, nrand3);
    for (int iy = 0; iy < n2; iy++) {
      int iy_v = clampi((int)((o2 + d2 * iy - vo2) / vd2), 0, vn2 - 1);
      float dy2 = taper2(iy, n2, nrand2);
      for (int ix = 0; ix < n1; ix++, i++) {
        int ix_v = clampi((int)((o1 + d1 * ix - vo1) / vd1), 0, vn1 - 1);
        float val = vel[ix_v + (long long)iy_v * vn1 + (long long)iz_v * vn1 * vn2];
        float dx2 = taper2(ix, n1, nrand1);
        if (dx2 < 0. || dx2 > 1) dx2 = 1;
        float dist = sqrtf(dx2 + dy2 + dz2);
        int found = dist < .0001;
        float dev = 0.;
        while (!found && nrand2 != 0) {
          float rnd = (float)rand() / RAND_MAX - .5 - .49 * dist;
          dev = rnd * 1.3 * dist * val;
          float mn = dist < 1.f ? dist : 1.f;
          if (fabsf(dev + val) < vmax * 1.03 * (1. - mn * .4) &&
              dev + val > 0.0001)
            found = 1;
        }
        out[i] = (val + dev) * (val + dev) * dt * dt;
      }
    }
  }
}

/* laplac, base/laplac_3d.cc:4-49 (adjoint) and 51-105 (forward). */
void oracle_laplac_forward(int add, const float *m, float *d, int n1, int n2,
                           int n3) {
  long long n12 = (long long)n1 * n2;
  if (!add) memset(d, 0, sizeof(float) * n12 * n3);
  for (long long i = 0; i < n12 * (n3 - 1); i++) {
    d[i + n12] += m[i];
    d[i] -= m[i];
  }
}

void oracle_laplac_adjoint(int add, float *m, const float *d, int n1, int n2,
                           int n3) {
  long long n12 = (long long)n1 * n2;
  if (!add) memset(m, 0, sizeof(float) * n12 * n3);
  for (long long i = 0; i < n12 * (n3 - 1); i++) m[i] += d[i + n12] - d[i];
}

/* deriv, base/deriv_3d.cc:4-29 (adjoint) and 31-56 (forward), including the
 * reference's repeated contribution of the first sample of each trace. */
void oracle_deriv_forward(int add, const float *m, float *d, int n1, int n2,
                          int n3, float d1) {
  long long n12 = (long long)n1 * n2;
  if (!add) memset(d, 0, sizeof(float) * n12 * n3);
  for (int i3 = 0; i3 < n3; i3++) {
    d[1 + i3 * n12] += m[i3 * n12] / d1;
    d[i3 * n12] -= m[i3 * n12] / d1;
    for (int i2 = 0; i2 < n2; i2++) {
      long long b = (long long)i2 * n1 + i3 * n12;
      d[1 + b] += m[b] / d1;
      d[b] -= m[b] / d1;
      for (int i1 = 0; i1 < n1 - 1; i1++) {
        d[i1 + b] -= m[b + i1] / d1;
        d[i1 + b + 1] += m[b + i1] / d1;
      }
    }
  }
}

void oracle_deriv_adjoint(int add, float *m, const float *d, int n1, int n2,
                          int n3, float d1) {
  long long n12 = (long long)n1 * n2;
  if (!add) memset(m, 0, sizeof(float) * n12 * n3);
  for (int i3 = 0; i3 < n3; i3++) {
    m[i3 * n12] += (d[i3 * n12 + 1] - d[i3 * n12]) / d1;
    for (int i2 = 0; i2 < n2; i2++) {
      long long b = (long long)i2 * n1 + i3 * n12;
      m[b] += (d[b + 1] - d[b]) / d1;
      for (int i1 = 0; i1 < n1 - 1; i1++)
        m[b + i1] += (d[i1 + b + 1] - d[i1 + b]) / d1;
    }
  }
}

/* map_data, base/map_data_3d.cc:37-55 (adjoint) and 57-75 (forward). */
void oracle_map_data_forward(int add, const float *m, float *d, int nt,
                             int n2, int n3, int ntb) {
  if (!add) memset(d, 0, sizeof(float) * (size_t)nt * n2 * n3);
  for (int i3 = 0; i3 < n3; i3++)
    for (int i2 = 0; i2 < n2; i2++)
      for (int it = 0; it < nt; it++)
        d[it + (long long)i2 * nt + (long long)i3 * nt * n2] +=
            m[(long long)ntb * i2 + it + 4 + (long long)i3 * ntb * n2];
}

void oracle_map_data_adjoint(int add, float *m, const float *d, int nt,
                             int n2, int n3, int ntb) {
  if (!add) memset(m, 0, sizeof(float) * (size_t)ntb * n2 * n3);
  for (int i3 = 0; i3 < n3; i3++)
    for (int i2 = 0; i2 < n2; i2++)
      for (int it = 0; it < nt; it++)
        m[(long long)ntb * i2 + it + 4 + (long long)i3 * ntb * n2] +=
            d[it + (long long)i2 * nt + (long long)i3 * nt * n2];
}

/* image_rtm_3d::extract_sub / add_image, base/image_rtm_3d.cc:24-95. */
void oracle_extract_sub(const float *whole, int w1, int w2, int w3, float *sub,
                        int s1, int s2, int s3, int f1, int f2, int f3) {
  memset(sub, 0, sizeof(float) * (size_t)s1 * s2 * s3);
  for (int i3 = 0; i3 < s3; i3++) {
    if (i3 + f3 < 0 || i3 + f3 >= w3) continue;
    for (int i2 = 0; i2 < s2; i2++) {
      if (i2 + f2 < 0 || i2 + f2 >= w2) continue;
      for (int i1 = 0; i1 < s1; i1++) {
        if (i1 + f1 < 0 || i1 + f1 >= w1) continue;
        sub[i1 + (long long)i2 * s1 + (long long)i3 * s1 * s2] =
            whole[i1 + f1 + (long long)(i2 + f2) * w1 +
                  (long long)(i3 + f3) * w1 * w2];
      }
    }
  }
}

void oracle_add_image(float *whole, int w1, int w2, int w3, const float *sub,
                      int s1, int s2, int s3, int f1, int f2, int f3) {
  for (int i3 = 0; i3 < s3; i3++) {
    if (i3 + f3 < 0 || i3 + f3 >= w3) continue;
    for (int i2 = 0; i2 < s2; i2++) {
      if (i2 + f2 < 0 || i2 + f2 >= w2) continue;
      for (int i1 = 0; i1 < s1; i1++) {
        if (i1 + f1 < 0 || i1 + f1 >= w1) continue;
        whole[i1 + f1 + (long long)(i2 + f2) * w1 +
              (long long)(i3 + f3) * w1 * w2] +=
            sub[i1 + (long long)i2 * s1 + (long long)i3 * s1 * s2];
      }
    }
  }
}

/* image_rtm_3d.cc:33-35 (and :64-66): f = (int)((sub.o - whole.o) / whole.d)
 * with the axes' float origins and spacing. */
int oracle_window_offset(float o_sub, float o_whole, float d_whole) {
  const float diff = o_sub - o_whole;
  return (int)(diff / d_whole);
}
