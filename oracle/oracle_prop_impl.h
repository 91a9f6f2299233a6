/*
 * Oracle (test infrastructure only): the propagator time loops of the
 * reference CPU path, restated in C.  Included twice by born_oracle.c: once
 * with REAL=float (the parity oracle, same operation order as the reference)
 * and once with REAL=double (the FP64 accuracy oracle).  Only the tests, the
 * smoke check and the CPU-baseline leg of bench.py load this code.
 *
 * Reference: base/cpu_prop.cc (ntuhpc/sc17-born).  Every function cites the
 * lines it follows.  Operation order is kept exactly (left-to-right sums, no
 * fused multiply-add: compile with -ffp-contract=off) so that the float
 * instance reproduces the compiled reference bit for bit.
 */
#ifndef REAL
#error "define REAL and SFX before including oracle_prop_impl.h"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)
#define PROPT CAT(oracle_prop, SFX)

/* Coefficient slots, base/cpu_prop.cc:6-18: slot 1/4/7/10 ("CZ") is applied
 * to the +-n12 neighbours, 2/5/8/11 ("CX") to +-1, 3/6/9/12 ("CY") to +-nx. */
#ifndef ORACLE_K_SLOTS
#define ORACLE_K_SLOTS
enum { K_C0 = 0, K_CZ1 = 1, K_CX1 = 2, K_CY1 = 3, K_CZ2 = 4, K_CX2 = 5,
       K_CY2 = 6, K_CZ3 = 7, K_CX3 = 8, K_CY3 = 9, K_CZ4 = 10, K_CX4 = 11,
       K_CY4 = 12 };
#endif

/* cpuProp::prop, base/cpu_prop.cc:224-253.  p0 <- v*(L p1) + p1 + p1 - p0
 * over the interior [4, n-4) of every axis, in place into p0. */
void FN(oracle_prop_step)(const PROPT *s, REAL *p0, const REAL *p1,
                          const REAL *vel) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const long long n12 = (long long)nx * ny;
  const REAL *c = s->coeffs;
#pragma omp parallel for schedule(static)
  for (int i3 = 4; i3 < nz - 4; i3++) {
    for (int i2 = 4; i2 < ny - 4; i2++) {
      long long ii = (long long)i2 * nx + 4 + n12 * i3;
      for (int i1 = 4; i1 < nx - 4; i1++, ii++) {
        p0[ii] = vel[ii] *
                     (c[K_C0] * p1[ii] + c[K_CX1] * (p1[ii - 1] + p1[ii + 1]) +
                      c[K_CX2] * (p1[ii - 2] + p1[ii + 2]) +
                      c[K_CX3] * (p1[ii - 3] + p1[ii + 3]) +
                      c[K_CX4] * (p1[ii - 4] + p1[ii + 4]) +
                      c[K_CY1] * (p1[ii - nx] + p1[ii + nx]) +
                      c[K_CY2] * (p1[ii - 2 * nx] + p1[ii + 2 * nx]) +
                      c[K_CY3] * (p1[ii - 3 * nx] + p1[ii + 3 * nx]) +
                      c[K_CY4] * (p1[ii - 4 * nx] + p1[ii + 4 * nx]) +
                      c[K_CZ1] * (p1[ii - n12] + p1[ii + n12]) +
                      c[K_CZ2] * (p1[ii - 2 * n12] + p1[ii + 2 * n12]) +
                      c[K_CZ3] * (p1[ii - 3 * n12] + p1[ii + 3 * n12]) +
                      c[K_CZ4] * (p1[ii - 4 * n12] + p1[ii + 4 * n12])) +
                 p1[ii] + p1[ii] - p0[ii];
      }
    }
  }
}

/* cpuProp::damp, base/cpu_prop.cc:141-165.  edge = distance to the interior
 * face, min over the three axes; cells with 0 <= edge < 40 are scaled. */
void FN(oracle_damp)(const PROPT *s, REAL *p0, REAL *p1) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const long long n12 = (long long)nx * ny;
#pragma omp parallel for schedule(static)
  for (int i3 = 4; i3 < nz - 4; i3++) {
    int e3 = i3 - 4 < nz - 4 - i3 ? i3 - 4 : nz - 4 - i3;
    for (int i2 = 4; i2 < ny - 4; i2++) {
      int e2 = i2 - 4 < ny - 4 - i2 ? i2 - 4 : ny - 4 - i2;
      if (e3 < e2) e2 = e3;
      long long ii = (long long)i2 * nx + 4 + n12 * i3;
      for (int i1 = 4; i1 < nx - 4; i1++, ii++) {
        int e1 = i1 - 4 < nx - 4 - i1 ? i1 - 4 : nx - 4 - i1;
        int edge = e2 < e1 ? e2 : e1;
        if (edge >= 0 && edge < ORACLE_NBOUND) {
          p0[ii] *= s->bound[edge];
          p1[ii] *= s->bound[edge];
        }
      }
    }
  }
}

/* cpuProp::injectSource, base/cpu_prop.cc:166-179. */
void FN(oracle_inject_source)(const PROPT *s, int id, int ii, REAL *p) {
  if (id + 7 >= s->nt_src) return;
  const REAL *t = s->table_s + (long long)ii * s->nsinc_s;
  for (int i = 0; i < s->npts_s; i++) {
    const REAL *v = s->source + (long long)s->nt_src * i + id;
    p[s->locs_s[i]] += (REAL)s->dir / (REAL)s->jt *
                       (t[0] * v[0] + t[1] * v[1] + t[2] * v[2] + t[3] * v[3] +
                        t[4] * v[4] + t[5] * v[5] + t[6] * v[6] + t[7] * v[7]);
  }
}

/* cpuProp::injectReceivers, base/cpu_prop.cc:180-197. */
void FN(oracle_inject_receivers)(const PROPT *s, int id, int ii, REAL *p) {
  if (id + 7 >= s->nt_rec) return;
  const REAL sc = (REAL)s->dir / (REAL)s->jt;
  const REAL *t = s->table_d + (long long)ii * s->nsinc_d;
  for (int i = 0; i < s->nrec; i++) {
    const REAL *v = s->rec + (long long)s->nt_rec * i + id;
    p[s->locs_r[i]] +=
        sc * (t[0] * v[0] + t[1] * v[1] + t[2] * v[2] + t[3] * v[3] +
              t[4] * v[4] + t[5] * v[5] + t[6] * v[6] + t[7] * v[7]);
  }
}

/* cpuProp::dataExtract, base/cpu_prop.cc:198-215. */
void FN(oracle_data_extract)(const PROPT *s, int id, int ii, const REAL *p) {
  if (id + 7 >= s->nt_rec) return;
  const REAL *t = s->table_d + (long long)ii * s->nsinc_d;
  for (int i = 0; i < s->nrec; i++) {
    REAL *r = s->rec + (long long)s->nt_rec * i + id;
    const REAL v = p[s->locs_r[i]];
    for (int k = 0; k < 8; k++) r[k] += v * t[k];
  }
}

/* cpuProp::imageAdd, base/cpu_prop.cc:216-223: the Born coupling.  The
 * constant is a double literal in the reference, so the product and the sum
 * are formed in double and rounded once on the store. */
void FN(oracle_image_add)(const PROPT *s, const REAL *img, REAL *rec_field,
                          const REAL *src_field) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < s->n123; i++)
    rec_field[i] += .000001 * src_field[i] * img[i];
}

/* cpuProp::imageCondition, base/cpu_prop.cc:97-105. */
void FN(oracle_image_condition)(const PROPT *s, const REAL *rec,
                                const REAL *src, REAL *img) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < s->n123; i++) img[i] += src[i] * rec[i];
}

/* cpuProp::sourceProp, base/cpu_prop.cc:106-129.  nt+1 steps with vel1, no
 * damping, injection at +1/jt into the new level.  For odd nt the reference
 * copies p0 into p1 at the end (both then hold the same level). */
void FN(oracle_source_prop)(PROPT *s, REAL *p0, REAL *p1, int jts, int nt) {
  s->jt = jts;
  s->dir = 1;
  for (int it = 0; it <= nt; it++) {
    int id = it / s->jt_s;
    int ii = it - id * s->jt_s;
    FN(oracle_prop_step)(s, p0, p1, s->vel1);
    FN(oracle_inject_source)(s, id, ii, p0);
    REAL *pt = p1;
    p1 = p0;
    p0 = pt;
  }
  if (nt % 2 == 1) memcpy(p1, p0, sizeof(REAL) * (size_t)s->n123);
}

/* cpuProp::rtmAdjoint, base/cpu_prop.cc:56-96.  Reverse time; the source
 * field is rebuilt by back-propagation through vel1, the receiver field is
 * propagated through vel2, damped and fed with the data at -1/jt. */
void FN(oracle_rtm_adjoint)(PROPT *s, REAL *src_p0, REAL *src_p1, REAL *img,
                            int jtd, int nt) {
  (void)jtd; /* the reference uses the table's own jt (cpu_prop.cc:75) */
  REAL *rec0 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *rec1 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *r_p0 = rec0, *r_p1 = rec1;
  s->dir = -1;
  for (int it = nt - 1; it >= 0; it--) {
    int id_s = (it + 1) / s->jt_s;
    int i_s = it + 1 - id_s * s->jt_s;
    int id = it / s->jt_d;
    int ii = it - id * s->jt_d;
    if (it > 0) FN(oracle_prop_step)(s, r_p0, r_p1, s->vel2);
    if (it < nt - 1) {
      FN(oracle_prop_step)(s, src_p0, src_p1, s->vel1);
      FN(oracle_inject_source)(s, id_s, i_s, src_p1);
    }
    FN(oracle_damp)(s, r_p0, r_p1);
    FN(oracle_inject_receivers)(s, id, ii, r_p0);
    FN(oracle_image_condition)(s, r_p0, src_p0, img);
    REAL *pt = src_p0;
    src_p0 = src_p1;
    src_p1 = pt;
    pt = r_p0;
    r_p0 = r_p1;
    r_p1 = pt;
  }
  free(rec0);
  free(rec1);
}

/* cpuProp::rtmForward, base/cpu_prop.cc:22-54.  Born forward: background s
 * and scattered r, both through vel2 and damped; source into s at +1/jt;
 * r += 1e-6 s img; r sampled into the traces. */
void FN(oracle_rtm_forward)(PROPT *s, int jt, const REAL *img, REAL *rec,
                            int nt) {
  s->jt = jt;
  s->rec = rec;
  REAL *b0 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *b1 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *b2 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *b3 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *r_p0 = b0, *r_p1 = b1, *s_p0 = b2, *s_p1 = b3;
  s->dir = 1;
  for (int it = 0; it < nt; it++) {
    int id = it / jt;
    int ii = it - id * jt;
    FN(oracle_prop_step)(s, s_p0, s_p1, s->vel2);
    FN(oracle_prop_step)(s, r_p0, r_p1, s->vel2);
    FN(oracle_damp)(s, s_p0, s_p1);
    FN(oracle_damp)(s, r_p0, r_p1);
    FN(oracle_inject_source)(s, id, ii, s_p0);
    FN(oracle_image_add)(s, img, r_p0, s_p0);
    FN(oracle_data_extract)(s, id, ii, r_p0);
    REAL *pt = s_p0;
    s_p0 = s_p1;
    s_p1 = pt;
    pt = r_p0;
    r_p0 = r_p1;
    r_p1 = pt;
  }
  free(b0);
  free(b1);
  free(b2);
  free(b3);
}

/* A p (the stencil sum of cpuProp::prop without the velocity factor) over
 * the interior, in the same summation order; exterior cells are left 0. */
static void FN(oracle_stencil_sum)(const PROPT *s, const REAL *p1, REAL *out) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const long long n12 = (long long)nx * ny;
  const REAL *c = s->coeffs;
#pragma omp parallel for schedule(static)
  for (int i3 = 4; i3 < nz - 4; i3++) {
    for (int i2 = 4; i2 < ny - 4; i2++) {
      long long ii = (long long)i2 * nx + 4 + n12 * i3;
      for (int i1 = 4; i1 < nx - 4; i1++, ii++) {
        out[ii] = c[K_C0] * p1[ii] + c[K_CX1] * (p1[ii - 1] + p1[ii + 1]) +
                  c[K_CX2] * (p1[ii - 2] + p1[ii + 2]) +
                  c[K_CX3] * (p1[ii - 3] + p1[ii + 3]) +
                  c[K_CX4] * (p1[ii - 4] + p1[ii + 4]) +
                  c[K_CY1] * (p1[ii - nx] + p1[ii + nx]) +
                  c[K_CY2] * (p1[ii - 2 * nx] + p1[ii + 2 * nx]) +
                  c[K_CY3] * (p1[ii - 3 * nx] + p1[ii + 3 * nx]) +
                  c[K_CY4] * (p1[ii - 4 * nx] + p1[ii + 4 * nx]) +
                  c[K_CZ1] * (p1[ii - n12] + p1[ii + n12]) +
                  c[K_CZ2] * (p1[ii - 2 * n12] + p1[ii + 2 * n12]) +
                  c[K_CZ3] * (p1[ii - 3 * n12] + p1[ii + 3 * n12]) +
                  c[K_CZ4] * (p1[ii - 4 * n12] + p1[ii + 4 * n12]);
      }
    }
  }
}

/* Nonlinear modelling: the background field of cpuProp::rtmForward
 * (cpu_prop.cc:36-41: vel2, taper, source at +1/jt) with the receiver
 * traces sampled from it as dataExtract does from r (cpu_prop.cc:45). */
void FN(oracle_model)(PROPT *s, int jt, REAL *rec, int nt) {
  s->jt = jt;
  s->rec = rec;
  s->dir = 1;
  REAL *b0 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *b1 = (REAL *)calloc((size_t)s->n123, sizeof(REAL));
  REAL *p0 = b0, *p1 = b1;
  for (int it = 0; it < nt; it++) {
    int id = it / jt, ii = it - id * jt;
    FN(oracle_prop_step)(s, p0, p1, s->vel2);
    FN(oracle_damp)(s, p0, p1);
    FN(oracle_inject_source)(s, id, ii, p0);
    FN(oracle_data_extract)(s, id, ii, p0);
    REAL *pt = p0;
    p0 = p1;
    p1 = pt;
  }
  free(b0);
  free(b1);
}

/* Exact linearisation of oracle_model with respect to vel2 along m:
 * r_{t+1} = B (vel2 A r_t + 2 r_t - B r_{t-1} + m (A s_t)), traces from r. */
void FN(oracle_lin_forward)(PROPT *s, int jt, const REAL *m, REAL *rec,
                            int nt) {
  s->jt = jt;
  s->rec = rec;
  s->dir = 1;
  const size_t n = (size_t)s->n123;
  REAL *b0 = (REAL *)calloc(n, sizeof(REAL)), *b1 = (REAL *)calloc(n, sizeof(REAL));
  REAL *b2 = (REAL *)calloc(n, sizeof(REAL)), *b3 = (REAL *)calloc(n, sizeof(REAL));
  REAL *g = (REAL *)calloc(n, sizeof(REAL));
  REAL *s_p0 = b0, *s_p1 = b1, *r_p0 = b2, *r_p1 = b3;
  for (int it = 0; it < nt; it++) {
    int id = it / jt, ii = it - id * jt;
    FN(oracle_stencil_sum)(s, s_p1, g);
    FN(oracle_prop_step)(s, s_p0, s_p1, s->vel2);
    FN(oracle_prop_step)(s, r_p0, r_p1, s->vel2);
    for (size_t i = 0; i < n; i++) r_p0[i] = r_p0[i] + m[i] * g[i];
    FN(oracle_damp)(s, s_p0, s_p1);
    FN(oracle_damp)(s, r_p0, r_p1);
    FN(oracle_inject_source)(s, id, ii, s_p0);
    FN(oracle_data_extract)(s, id, ii, r_p0);
    REAL *pt = s_p0;
    s_p0 = s_p1;
    s_p1 = pt;
    pt = r_p0;
    r_p0 = r_p1;
    r_p1 = pt;
  }
  free(b0);
  free(b1);
  free(b2);
  free(b3);
  free(g);
}

/* Exact adjoint of oracle_lin_forward (no reference counterpart: the
 * reference's RTM adjoint is not the transpose of its Born forward).  The
 * forward is the state recursion, per step t (taper B, stencil A, V = vel2,
 * g_t = A s_t the background's stencil sum, E_t the trace extraction):
 *   x_{t+1} = B y_t,   y_{t+1} = B (V A y_t + 2 y_t - x_t + m g_t),
 *   d_t = E_t y_{t+1},   x_0 = y_0 = 0,
 * whose transpose in z_t = B ybar_{t+1} is, for t = nt-1 .. 0,
 *   z_t = B (A (V z_{t+1}) + 2 z_{t+1} - B z_{t+2} + E_t^T d_t),
 *   mbar = sum_t g_t z_t
 * (A restricted to the interior is symmetric; the exterior band is never
 * written).  All g_t are kept (n123 x nt values: small grids only).  rec:
 * the traces d [nrec][nt_rec]; mbar (n123) is overwritten. */
void FN(oracle_lin_adjoint)(PROPT *s, int jt, const REAL *rec, REAL *mbar,
                            int nt) {
  s->jt = jt;
  s->dir = 1;
  const size_t n = (size_t)s->n123;
  REAL *g = (REAL *)calloc(n * (size_t)(nt > 0 ? nt : 1), sizeof(REAL));
  REAL *b0 = (REAL *)calloc(n, sizeof(REAL)), *b1 = (REAL *)calloc(n, sizeof(REAL));
  REAL *s_p0 = b0, *s_p1 = b1;
  for (int it = 0; it < nt; it++) {
    int id = it / jt, ii = it - id * jt;
    FN(oracle_stencil_sum)(s, s_p1, g + n * (size_t)it);
    FN(oracle_prop_step)(s, s_p0, s_p1, s->vel2);
    FN(oracle_damp)(s, s_p0, s_p1);
    FN(oracle_inject_source)(s, id, ii, s_p0);
    REAL *pt = s_p0;
    s_p0 = s_p1;
    s_p1 = pt;
  }
  REAL *z0 = (REAL *)calloc(n, sizeof(REAL)), *z1 = (REAL *)calloc(n, sizeof(REAL));
  REAL *z2 = (REAL *)calloc(n, sizeof(REAL)), *vz = (REAL *)calloc(n, sizeof(REAL));
  REAL *a = (REAL *)calloc(n, sizeof(REAL)), *one = (REAL *)malloc(n * sizeof(REAL));
  for (size_t i = 0; i < n; i++) {
    mbar[i] = 0;
    one[i] = 1;
  }
  /* the taper factor of every cell: oracle_damp applied to ones */
  REAL *bt = (REAL *)malloc(n * sizeof(REAL));
  for (size_t i = 0; i < n; i++) bt[i] = 1;
  FN(oracle_damp)(s, bt, one);
  for (int it = nt - 1; it >= 0; it--) {
    int id = it / jt, ii = it - id * jt;
    for (size_t i = 0; i < n; i++) vz[i] = s->vel2[i] * z1[i];
    FN(oracle_stencil_sum)(s, vz, a);
    for (size_t i = 0; i < n; i++)
      z0[i] = a[i] + 2 * z1[i] - bt[i] * z2[i];
    /* E_t^T d_t: the transpose of oracle_data_extract */
    if (id + 7 < s->nt_rec) {
      const REAL *t = s->table_d + (long long)ii * s->nsinc_d;
      for (int r = 0; r < s->nrec; r++) {
        const REAL *v = rec + (long long)s->nt_rec * r + id;
        REAL acc = 0;
        for (int k = 0; k < 8; k++) acc += t[k] * v[k];
        z0[s->locs_r[r]] += acc;
      }
    }
    const REAL *gt = g + n * (size_t)it;
    for (size_t i = 0; i < n; i++) {
      z0[i] *= bt[i];
      mbar[i] += gt[i] * z0[i];
    }
    REAL *pt = z2;
    z2 = z1;
    z1 = z0;
    z0 = pt;
  }
  free(g);
  free(b0);
  free(b1);
  free(z0);
  free(z1);
  free(z2);
  free(vz);
  free(a);
  free(one);
  free(bt);
}

#undef FN
#undef PROPT
#undef CAT
#undef CAT_
