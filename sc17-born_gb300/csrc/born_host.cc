// Host-side geometry and per-shot glue (see born_host.h).  Arithmetic types
// follow the reference line by line (float storage, double where the
// reference forms a double), so the tables and indices match it exactly.
#include "born_host.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/born_gb300.h"

namespace {

// Toeplitz solver r f = g (Claerbout FGDP p.57), double accumulators over
// float arrays (base/sinc_bob.cc:73-100).
void toeplitz_solve(int m, const float *r, float *f, const float *g,
                    float *a) {
  a[0] = 1.f;
  double v = r[0];
  f[0] = g[0] / r[0];
  for (int j = 1; j < m; ++j) {
    double e;
    e = a[j] = f[j] = 0.f;
    for (int i = 0; i < j; ++i) e += a[i] * r[j - i];
    double c = e / v;
    v -= e * c;
    for (int i = 0; i <= j / 2; ++i) {
      const double bot = a[j - i] - c * a[i];
      a[i] -= c * a[j - i];
      a[j - i] = bot;
    }
    double w = 0;
    for (int i = 0; i < j; ++i) w += f[i] * r[j - i];
    c = (g[j] - w) / v;
    for (int i = 0; i <= j; ++i) f[i] += c * a[j - i];
  }
}

// One row of the tapered-sinc table for fractional shift d
// (base/sinc_bob.cc:36-64): spectra matched up to 0.066 + 0.265 ln(lsinc)
// of Nyquist, sampled in float steps.
void sinc_row(float *out, int lsinc, float d) {
  const float pi = 3.141592654;
  const float pi2 = pi * 2;
  const float snyq = 0.5;
  const float snat = snyq * (0.066 + 0.265 * std::log((double)lsinc));
  const float s0 = 0.0;
  const float ds = (snat - s0) / (lsinc * 2 - 1);
  const float eta = lsinc / 2 - 1.0 + d;
  std::vector<float> b(lsinc), c(lsinc), work(lsinc);
  for (int j = 0; j < lsinc; ++j) {
    b[j] = c[j] = 0.0f;
    for (float s = s0; s <= snat; s += ds) {
      b[j] += std::cos(pi2 * s * j);
      c[j] += std::cos(pi2 * s * (eta - j));
    }
  }
  toeplitz_solve(lsinc, b.data(), out, c.data(), work.data());
}

inline int clampi(int v, int lo, int hi) { return std::max(lo, std::min(hi, v)); }

// Squared normalised distance into a random-boundary band of nr cells
// (base/vel_fd_3d.cc:60-68 and the two analogous blocks).
inline float band2(int i, int n, int nr) {
  if (i < nr) return (float)((nr - i) * (nr - i)) / (float)(nr * nr);
  if (i >= n - nr) {
    const int k = i - (n - nr - 1);
    return (float)(k * k) / (float)(nr * nr);
  }
  return 0;
}

}  // namespace

extern "C" {

int born_sinc_table(int ntab, int nsinc, float *out) {
  if (ntab < 1 || nsinc < 2 || nsinc % 2 || !out) return BORN_EINVAL;
  const float dtab = 1. / (float)ntab;
  float t = 0.;
  for (int it = 0; it < ntab; ++it, t += dtab) {
    std::fill(out + (size_t)it * nsinc, out + (size_t)(it + 1) * nsinc, 0.f);
    sinc_row(out + (size_t)it * nsinc, nsinc, t);
  }
  return BORN_OK;
}

float born_calc_stability(float vmax, float dmin, float dt_data, int nt_data,
                          int *nt_out) {
  const float d = .47 * dmin / vmax;
  const float dt = dt_data / std::ceil(dt_data / d);
  if (nt_out) *nt_out = (nt_data - 1) * (int)(dt_data / dt) + 1;
  return dt;
}

int born_compute_size(int n_model, int nbound, int fat) {
  const int n = n_model + 2 * (nbound + fat);
  const int rem = n % 16;
  return rem ? n + 16 - rem : n;
}

int born_source_geometry(float sx, float sy, float sz, float o1, float o2,
                         float o3, float d1, float d2, float d3, int n1,
                         int n2, const float *wavelet, int nt_wav, int nts,
                         int *locs, float *vals) {
  if (!wavelet || !locs || !vals || nts < 5) return BORN_EINVAL;
  const float fz = (sz - o3) / d3 + .5;
  const float fy = (sy - o2) / d2 + .5;
  const float fx = (sx - o1) / d1 + .5;
  const int iz = (int)fz, iy = (int)fy, ix = (int)fx;
  std::fill(vals, vals + (size_t)nts * 9, 0.f);
  const int ncopy = std::min(nt_wav, nts - 4);
  const int i3 = iz - 1;  // the 3x3 points sit on one plane
  const float zn = fz - i3;
  int i = 0;
  for (int i2 = iy - 1; i2 <= iy + 1; ++i2) {
    const float yn = fy - i2;
    for (int i1 = ix - 1; i1 <= ix + 1; ++i1, ++i) {
      const float xn = fx - i1;
      locs[i] = i1 + i2 * n1 + i3 * n1 * n2;
      const float w = std::exp(-zn * zn - xn * xn - yn * yn);
      for (int it = 0; it < ncopy; ++it)
        vals[(size_t)nts * i + it + 4] = w * wavelet[it];
    }
  }
  return BORN_OK;
}

int born_wavelet_deriv(const float *raw, int nt, float dt, float *out) {
  if (!raw || !out || nt < 1) return BORN_EINVAL;
  out[nt - 1] = 0;
  for (int it = 0; it + 1 < nt; ++it) out[it] = (raw[it + 1] - raw[it]) / dt;
  return BORN_OK;
}

int born_receiver_geometry(int rec_nx, int rec_ny, float rx0, float rdx,
                           float ry0, float rdy, float rz, float o1, float o2,
                           float o3, float d1, float d2, float d3, int n1,
                           int n2, int *locs) {
  if (!locs || rec_nx < 0 || rec_ny < 0) return BORN_EINVAL;
  for (int i3 = 0, i = 0; i3 < rec_ny; ++i3) {
    for (int i2 = 0; i2 < rec_nx; ++i2, ++i) {
      const float s_z = (rz - o3) / d3;
      const float s_x = (rx0 + rdx * i2 - o1) / d1;
      const float s_y = (ry0 + rdy * i3 - o2) / d2;
      locs[i] = (int)s_x + (int)s_y * n1 + (int)s_z * n1 * n2;
    }
  }
  return BORN_OK;
}

int born_rand_subspace(const float *vel, int vn1, int vn2, int vn3, float vo1,
                       float vo2, float vo3, float vd1, float vd2, float vd3,
                       float vmax, int irand, int nrand1, int nrand2,
                       int nrand3, float dt, int n1, int n2, int n3, float o1,
                       float o2, float o3, float d1, float d2, float d3,
                       float *out) {
  if (!vel || !out) return BORN_EINVAL;
  srand(irand);
  size_t i = 0;
  for (int iz = 0; iz < n3; ++iz) {
    const int iz_v = clampi((int)((o3 + d3 * iz - vo3) / vd3), 0, vn3 - 1);
    const float dz2 = band2(iz, n3, nrand3);
    for (int iy = 0; iy < n2; ++iy) {
      const int iy_v = clampi((int)((o2 + d2 * iy - vo2) / vd2), 0, vn2 - 1);
      const float dy2 = band2(iy, n2, nrand2);
      for (int ix = 0; ix < n1; ++ix, ++i) {
        const int ix_v = clampi((int)((o1 + d1 * ix - vo1) / vd1), 0, vn1 - 1);
        const float val =
            vel[ix_v + (size_t)iy_v * vn1 + (size_t)iz_v * vn1 * vn2];
        float dx2 = band2(ix, n1, nrand1);
        if (dx2 < 0. || dx2 > 1) dx2 = 1;
        const float dist = std::sqrt(dx2 + dy2 + dz2);
        bool found = dist < .0001;
        float dev = 0.;
        // rejection sampling under the tapered bound (vel_fd_3d.cc:115-122)
        while (!found && nrand2 != 0) {
          const float rnd = (float)rand() / RAND_MAX - .5 - .49 * dist;
          dev = rnd * 1.3 * dist * val;
          if (std::fabs(dev + val) <
                  vmax * 1.03 * (1. - std::min(1.f, dist) * .4) &&
              dev + val > 0.0001)
            found = true;
        }
        out[i] = (val + dev) * (val + dev) * dt * dt;
      }
    }
  }
  return BORN_OK;
}

int born_laplac_forward(int add, const float *m, float *d, int n1, int n2,
                        int n3) {
  if (n1 < 1 || n2 < 1 || n3 < 1) return BORN_EINVAL;
  const size_t n12 = (size_t)n1 * n2;
  if (!add) std::fill(d, d + n12 * n3, 0.f);
  for (size_t i = 0; i < n12 * (n3 - 1); ++i) {
    d[i + n12] += m[i];
    d[i] -= m[i];
  }
  return BORN_OK;
}

int born_laplac_adjoint(int add, float *m, const float *d, int n1, int n2,
                        int n3) {
  if (n1 < 1 || n2 < 1 || n3 < 1) return BORN_EINVAL;
  const size_t n12 = (size_t)n1 * n2;
  if (!add) std::fill(m, m + n12 * n3, 0.f);
  for (size_t i = 0; i < n12 * (n3 - 1); ++i) m[i] += d[i + n12] - d[i];
  return BORN_OK;
}

int born_deriv_forward(int add, const float *m, float *d, int n1, int n2,
                       int n3, float d1) {
  const size_t n12 = (size_t)n1 * n2;
  if (!add) std::fill(d, d + n12 * n3, 0.f);
  for (int i3 = 0; i3 < n3; ++i3) {
    const size_t p = i3 * n12;
    d[1 + p] += m[p] / d1;
    d[p] -= m[p] / d1;
    for (int i2 = 0; i2 < n2; ++i2) {
      const size_t b = p + (size_t)i2 * n1;
      d[1 + b] += m[b] / d1;
      d[b] -= m[b] / d1;
      for (int i1 = 0; i1 < n1 - 1; ++i1) {
        d[b + i1] -= m[b + i1] / d1;
        d[b + i1 + 1] += m[b + i1] / d1;
      }
    }
  }
  return BORN_OK;
}

int born_deriv_adjoint(int add, float *m, const float *d, int n1, int n2,
                       int n3, float d1) {
  const size_t n12 = (size_t)n1 * n2;
  if (!add) std::fill(m, m + n12 * n3, 0.f);
  for (int i3 = 0; i3 < n3; ++i3) {
    const size_t p = i3 * n12;
    m[p] += (d[p + 1] - d[p]) / d1;
    for (int i2 = 0; i2 < n2; ++i2) {
      const size_t b = p + (size_t)i2 * n1;
      m[b] += (d[b + 1] - d[b]) / d1;
      for (int i1 = 0; i1 < n1 - 1; ++i1)
        m[b + i1] += (d[b + i1 + 1] - d[b + i1]) / d1;
    }
  }
  return BORN_OK;
}

int born_map_data_forward(int add, const float *m, float *d, int nt, int n2,
                          int n3, int ntb) {
  if (!add) std::fill(d, d + (size_t)nt * n2 * n3, 0.f);
  for (int i3 = 0; i3 < n3; ++i3)
    for (int i2 = 0; i2 < n2; ++i2) {
      float *dt = d + (size_t)i2 * nt + (size_t)i3 * nt * n2;
      const float *mt = m + (size_t)ntb * i2 + 4 + (size_t)i3 * ntb * n2;
      for (int it = 0; it < nt; ++it) dt[it] += mt[it];
    }
  return BORN_OK;
}

int born_map_data_adjoint(int add, float *m, const float *d, int nt, int n2,
                          int n3, int ntb) {
  if (!add) std::fill(m, m + (size_t)ntb * n2 * n3, 0.f);
  for (int i3 = 0; i3 < n3; ++i3)
    for (int i2 = 0; i2 < n2; ++i2) {
      const float *dt = d + (size_t)i2 * nt + (size_t)i3 * nt * n2;
      float *mt = m + (size_t)ntb * i2 + 4 + (size_t)i3 * ntb * n2;
      for (int it = 0; it < nt; ++it) mt[it] += dt[it];
    }
  return BORN_OK;
}

int born_extract_sub(const float *whole, int w1, int w2, int w3, float *sub,
                     int s1, int s2, int s3, int f1, int f2, int f3) {
  std::fill(sub, sub + (size_t)s1 * s2 * s3, 0.f);
  for (int i3 = 0; i3 < s3; ++i3) {
    if (i3 + f3 < 0 || i3 + f3 >= w3) continue;
    for (int i2 = 0; i2 < s2; ++i2) {
      if (i2 + f2 < 0 || i2 + f2 >= w2) continue;
      for (int i1 = 0; i1 < s1; ++i1) {
        if (i1 + f1 < 0 || i1 + f1 >= w1) continue;
        sub[i1 + (size_t)i2 * s1 + (size_t)i3 * s1 * s2] =
            whole[i1 + f1 + (size_t)(i2 + f2) * w1 +
                  (size_t)(i3 + f3) * w1 * w2];
      }
    }
  }
  return BORN_OK;
}

int born_add_image(float *whole, int w1, int w2, int w3, const float *sub,
                   int s1, int s2, int s3, int f1, int f2, int f3) {
  for (int i3 = 0; i3 < s3; ++i3) {
    if (i3 + f3 < 0 || i3 + f3 >= w3) continue;
    for (int i2 = 0; i2 < s2; ++i2) {
      if (i2 + f2 < 0 || i2 + f2 >= w2) continue;
      for (int i1 = 0; i1 < s1; ++i1) {
        if (i1 + f1 < 0 || i1 + f1 >= w1) continue;
        whole[i1 + f1 + (size_t)(i2 + f2) * w1 + (size_t)(i3 + f3) * w1 * w2] +=
            sub[i1 + (size_t)i2 * s1 + (size_t)i3 * s1 * s2];
      }
    }
  }
  return BORN_OK;
}

int born_window_offset(float o_sub, float o_whole, float d_whole) {
  const float diff = o_sub - o_whole;
  return (int)(diff / d_whole);
}

}  // extern "C"
