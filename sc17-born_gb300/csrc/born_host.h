// Host-side geometry and per-shot glue of the Born / RTM path (C ABI).
//
// These run on the CPU once per shot and prepare what the propagator
// consumes: sinc interpolation tables, time step, padded compute grid,
// source and receiver points, the v^2 dt^2 velocity with an optional random
// boundary, and the small linear maps around the propagator (z first
// difference, time derivative, trace lead mapping, image window).  Each
// function names the reference code it restates.
#ifndef BORN_HOST_H
#define BORN_HOST_H

#ifdef __cplusplus
extern "C" {
#endif

/* sinc_bob(ntab, nsinc).table, row-major ntab x nsinc
 * (base/sinc_bob.cc:4-100; Hale/Larner least-squares tapered sinc). */
int born_sinc_table(int ntab, int nsinc, float *out);

/* fd_prop::calc_stability (base/fd_prop_3d.cc:6-33): FD dt from the data dt
 * and the 0.47 dmin / vmax bound; *nt_out = (nt_data-1) * jt + 1. */
float born_calc_stability(float vmax, float dmin, float dt_data, int nt_data,
                          int *nt_out);

/* source_func::set_compute_size (base/source_func_3d.cc:4-34) per axis:
 * n + 2 (nbound + fat), rounded up to a multiple of 16. */
int born_compute_size(int n_model, int nbound, int fat);

/* wavelet_source_func::get_source_func (base/source_func_3d.cc:76-109):
 * 9 points (3x3 on the plane iz-1) and their traces [9][nts] with a 4-sample
 * lead.  (o, d) describe the compute grid. */
int born_source_geometry(float sx, float sy, float sz, float o1, float o2,
                         float o3, float d1, float d2, float d3, int n1,
                         int n2, const float *wavelet, int nt_wav, int nts,
                         int *locs, float *vals);

/* wavelet_source_func ctor (base/source_func_3d.cc:120-124): forward
 * difference / dt, last sample zero. */
int born_wavelet_deriv(const float *raw, int nt, float dt, float *out);

/* data_rtm_3d::get_source_func + map_data ctor (base/data_rtm_3d.cc:79-88,
 * base/map_data_3d.cc:17-31): receiver cells of a rec_nx x rec_ny grid. */
int born_receiver_geometry(int rec_nx, int rec_ny, float rx0, float rdx,
                           float ry0, float rdy, float rz, float o1, float o2,
                           float o3, float d1, float d2, float d3, int n1,
                           int n2, int *locs);

/* vel_fd_3d::rand_subspace (base/vel_fd_3d.cc:29-134): resample the model
 * velocity onto the compute grid (clamped), random boundary within nrand
 * cells of each face (rand() seeded with irand, drawn in z, y, x order),
 * output v^2 dt^2.  nrand2 == 0 disables the random boundary. */
int born_rand_subspace(const float *vel, int vn1, int vn2, int vn3, float vo1,
                       float vo2, float vo3, float vd1, float vd2, float vd3,
                       float vmax, int irand, int nrand1, int nrand2,
                       int nrand3, float dt, int n1, int n2, int n3, float o1,
                       float o2, float o3, float d1, float d2, float d3,
                       float *out);

/* laplac (base/laplac_3d.cc:4-105): first difference along axis 3. */
int born_laplac_forward(int add, const float *m, float *d, int n1, int n2,
                        int n3);
int born_laplac_adjoint(int add, float *m, const float *d, int n1, int n2,
                        int n3);

/* deriv (base/deriv_3d.cc:4-56): time first difference / d1, with the
 * reference's repeated contribution of each trace's first sample. */
int born_deriv_forward(int add, const float *m, float *d, int n1, int n2,
                       int n3, float d1);
int born_deriv_adjoint(int add, float *m, const float *d, int n1, int n2,
                       int n3, float d1);

/* map_data (base/map_data_3d.cc:37-75): traces of nt samples <-> padded
 * traces of ntb samples with a 4-sample lead. */
int born_map_data_forward(int add, const float *m, float *d, int nt, int n2,
                          int n3, int ntb);
int born_map_data_adjoint(int add, float *m, const float *d, int nt, int n2,
                          int n3, int ntb);

/* image_rtm_3d::extract_sub / add_image (base/image_rtm_3d.cc:24-95):
 * window of the model-grid image at sample offsets (f1, f2, f3). */
int born_extract_sub(const float *whole, int w1, int w2, int w3, float *sub,
                     int s1, int s2, int s3, int f1, int f2, int f3);
int born_add_image(float *whole, int w1, int w2, int w3, const float *sub,
                   int s1, int s2, int s3, int f1, int f2, int f3);
/* Sample offset of a window axis within the whole image's axis, as
 * image_rtm_3d.cc:33-35 and :64-66 form it from the two axes: (o_sub -
 * o_whole) / d_whole in float, truncated toward zero.  For origins that are
 * not exact multiples of the spacing this can be one sample short of the
 * rounded value; the window functions above take the offsets it returns. */
int born_window_offset(float o_sub, float o_whole, float d_whole);

/* SEP regular files (the reference's genericIO datasets): header text of
 * key=value pairs (n1..n6, o1..o6, d1..d6, esize=4, data_format xdr_float or
 * native_float, in= binary path, relative to the header's folder). */
typedef struct {
  int ndim;            /* highest axis given in the header */
  long long n[6];
  float o[6], d[6];
  int big_endian;      /* 1 for xdr_float */
  char in[1024];       /* resolved path of the binary data */
} born_sep_info;
int born_sep_read_info(const char *header, born_sep_info *info);
/* count must equal n1*...*n6 of the header */
int born_sep_read(const char *header, float *out, long long count);
/* writes header and header@ (binary), big_endian selects xdr_float */
int born_sep_write(const char *header, const born_sep_info *info,
                   const float *data, int big_endian);
/* JSON regular files (the other kind SEP genericIO reads; the form
 * scripts/run.py:20-36 writes): a JSON object with n1.., o1.., d1..,
 * label1.. and "filename" (the data file, relative to the JSON's folder),
 * 4-byte floats in host order unless "data_format" is "xdr_float". */
int born_json_read_info(const char *path, born_sep_info *info);
/* Either kind, by name: paths ending in ".json" are JSON, others SEP.
 * Writing makes a SEP header with big-endian data in path + "@", or a JSON
 * description with host-order data in path + ".dat". */
int born_regfile_read_info(const char *path, born_sep_info *info);
int born_regfile_read(const char *path, float *out, long long count);
int born_regfile_write(const char *path, const born_sep_info *info,
                       const float *data);
/* util/Add (util/Add.cc:5-41): out = in1 + in2 (same sizes, else
 * BORN_EINVAL); out takes in1's axes and may be in1 or in2. */
int born_add_regfiles(const char *in1, const char *in2, const char *out);

#ifdef __cplusplus
}
#endif
#endif
