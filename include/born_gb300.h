/*
 * born_gb300 — C ABI of the GB300 (sm_103a) Born-modelling / RTM propagator.
 *
 * Two layers, both plain C (host pointers, sizes, int status codes):
 *
 *  1. Drop-in entry points with the exact names and signatures of the
 *     reference's GPU C ABI, base/gpu/gpu_funcs_3d.h:4-37, as bound by
 *     base/gpu_prop.cc:6-70.  They drive one process-wide default handle on
 *     the current device; like the reference they return void, but instead
 *     of exit(-1) (base/gpu/gpu_funcs_3d.cu:58-70) they record an error that
 *     born_default_status() / born_default_error() report.
 *
 *  2. A handle-based API (born_*) with per-handle device state and one CUDA
 *     stream per handle; every call returns BORN_OK (0) or a negative
 *     BORN_E* code and never exits.  Handles are thread-compatible: use one
 *     handle per host thread.
 *
 * Grid: compute grid [n3][n2][n1] float, n1 fastest, n1 a multiple of 4 and
 * every n >= 9; the reference sizes it to multiples of 16
 * (base/source_func_3d.cc:21-34).  Interior cells [4, n-4) are updated;
 * sources and receivers must lie in the interior; n1*n2*n3 < 2^31.
 * Velocities are given as v^2 dt^2 (base/vel_fd_3d.cc:125).
 */
#ifndef BORN_GB300_H
#define BORN_GB300_H

#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define BORN_OK 0
#define BORN_EINVAL (-1)   /* bad argument or size */
#define BORN_ECUDA (-2)    /* CUDA runtime / driver error */
#define BORN_ENOMEM (-3)   /* device allocation failed */
#define BORN_ESTATE (-4)   /* call sequence violated (e.g. no grid yet) */
#define BORN_ETIMEOUT (-5) /* a device-side wait gave up (bounded spin) */
#define BORN_ENODEV (-6)   /* no usable CUDA device */

typedef struct born_handle born_handle;

/* ======================================================================
 * 1. Reference-compatible entry points (base/gpu/gpu_funcs_3d.h)
 * ====================================================================== */

/* gpu_funcs_3d.h:7 (setup_cuda, gpu_funcs_3d.cu:21-56).  Creates the default
 * handle on the current device.  This build drives one GPU per process;
 * ngpus > 1 is accepted and recorded, shots are spread by the caller. */
void setup_cuda(int ngpus);

/* gpu_funcs_3d.h:35-36 (create_gpu_space, gpu_funcs_3d.cu:1286-1317).
 * Grid sizes, 8th-order coefficients from the spacings, taper table. */
void create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b,
                      float bc_b_y, int nx, int ny, int nz);

/* gpu_funcs_3d.h:18-21: ns rows x nsinc taps, row-major (gpu_prop.cc:15-24) */
void transfer_sinc_table_s(int nsinc, int ns, float *tables);
void transfer_sinc_table_d(int nsinc, int ns, float *tabled);

/* gpu_funcs_3d.h:23-24: npts source points, traces [npts][nt] */
void transfer_source_func(int npts, int nt, int *locs, float *vals);

/* gpu_funcs_3d.h:25 (load_source): kept for link compatibility; no-op. */
void load_source(int it);

/* gpu_funcs_3d.h:26-29: nx*ny receivers, traces [nx*ny][nt] */
void transfer_receiver_func(int nx, int ny, int nt, int *locs, float *vals);

/* gpu_funcs_3d.h:31-33: v^2 dt^2 of the random-boundary (1) and plain (2)
 * velocity models */
void transfer_vel_func1(int nx, int ny, int nz, float *vel);
void transfer_vel_func2(int nx, int ny, int nz, float *vel);

/* gpu_funcs_3d.h:10-11 (source_prop, gpu_funcs_3d.cu:199-446).  nt+1 steps
 * of source propagation (cpu_prop.cc:106-129).  The two final levels stay on
 * the device for rtm_adjoint; when get_last is true and p0/p1 are non-null
 * they are also copied to the host arrays, as cpuProp does. */
void source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0,
                 float *p1, int jt, int npts, int nt);

/* gpu_funcs_3d.h:13-14 (rtm_adjoint, gpu_funcs_3d.cu:832-1154).  Reverse-time
 * RTM adjoint (cpu_prop.cc:56-96).  p0_s_cpu/p1_s_cpu name the two source
 * levels, read as born_rtm_adjoint_host reads them (by default: when they are
 * the host arrays last given to source_prop, in either order, the
 * device-resident levels are used in that order; other non-null arrays are
 * uploaded).  The full padded image is accumulated onto img (zero on entry at
 * every reference call site, rtm_zero_op_3d.cc:259). */
void rtm_adjoint(int n1, int n2, int n3, int j, float *p0_s_cpu,
                 float *p1_s_cpu, float *img, int npts, int nt);

/* gpu_funcs_3d.h:15 (set_ntblock): trace blocking is not needed (traces
 * stay resident); recorded only. */
void set_ntblock(int nt);

/* gpu_funcs_3d.h:16-17 (rtm_forward; the reference GPU body is commented
 * out, gpu_funcs_3d.cu:448-804, so this follows cpuProp::rtmForward,
 * cpu_prop.cc:22-54).  Born forward of img into the receiver traces, which
 * are accumulated onto the traces last transferred and written to dat. */
void rtm_forward(int n1, int n2, int n3, int jt, float *img, float *dat,
                 int npts_src, int nt, int nt_big, int nx, int ny);

/* Status of the last default-handle call (0 or a BORN_E* code) and its
 * message; these replace the reference's exit(-1). */
int born_default_status(void);
const char *born_default_error(void);
born_handle *born_default_handle(void);

/* ======================================================================
 * 2. Handle-based API
 * ====================================================================== */

/* Creates a handle on CUDA device `device` (its own non-blocking stream). */
int born_create(int device, born_handle **out);
int born_destroy(born_handle *h);
const char *born_error_string(const born_handle *h);

/* cpuProp::createSpace / create_gpu_space */
int born_create_space(born_handle *h, float d1, float d2, float d3, float bc_a,
                      float bc_b, float bc_y, int nx, int ny, int nz);
/* which = 0: source table (transferSincTableS), 1: data table (…D) */
int born_set_sinc_table(born_handle *h, int which, int nsinc, int jt,
                        const float *table);
int born_set_source_func(born_handle *h, int npts, int nt_big, const int *locs,
                         const float *vals);
int born_set_receiver_func(born_handle *h, int rec_nx, int rec_ny, int nt_big,
                           const int *locs, const float *traces);
/* slot 1: random-boundary model (vel1), slot 2: plain model (vel2) */
int born_set_velocity(born_handle *h, int slot, int nx, int ny, int nz,
                      const float *v2dt2);
/* Velocity slot (1 or 2) made on the device from a model velocity (host,
 * vn3 x vn2 x vn1 m/s, origin vo, spacing vd): vel_fd_3d::rand_subspace
 * (vel_fd_3d.cc:29-134) with a counter-based generator (SplitMix64 of seed,
 * cell and draw) instead of rand(), so the random boundary is deterministic;
 * cells outside the nrand bands equal born_rand_subspace's bit for bit.  At
 * most 64 draws per cell (the reference loops until one is accepted).
 * (o, d) describe the compute grid; output is v^2 dt^2. */
int born_make_velocity(born_handle *h, int slot, const float *vel, int vn1,
                       int vn2, int vn3, float vo1, float vo2, float vo3,
                       float vd1, float vd2, float vd3, float vmax,
                       unsigned long long seed, int nrand1, int nrand2,
                       int nrand3, float dt, float o1, float o2, float o3,
                       float d1, float d2, float d3);
int born_get_velocity(born_handle *h, int slot, float *out);
/* Reflectivity for the Born forward (the image the forward reads). */
int born_set_reflectivity(born_handle *h, const float *img);

/* Time loops.  Null host pointers leave results on the device, which is how
 * a caller chains calls without host round trips. */
int born_source_prop(born_handle *h, int jts, int nt, float *p0_out,
                     float *p1_out);
/* swap = 0: the adjoint's (src_p0, src_p1) are source_prop's (p0, p1);
 * swap = 1: they are (p1, p0), which is how rtm_zero_op_3d.cc:272-282
 * calls it.  img (in/out, nullable): the image is accumulated onto its
 * contents, as cpuProp does (cpu_prop.cc:101); null starts from zero and
 * leaves the image on the device. */
int born_rtm_adjoint(born_handle *h, int jtd, int nt, int swap, float *img);

/* baseProp::rtmAdjoint(..., p0, p1, img, ...) (base_prop.h:57-62) on host
 * arrays of the two source levels, as the reference's operator calls it
 * after sourceProp (rtm_zero_op_3d.cc:272-282).  How p0/p1 are read is the
 * handle's host-level policy (born_set_host_levels):
 *  BORN_HOST_LEVELS_RESIDENT (default): like the reference's GPU path, which
 *    keeps the source levels on the device (gpu_funcs_3d.cu:14,436-445):
 *    when p0/p1 are the arrays the last born_source_prop wrote (in either
 *    order) the device-resident levels are used in that order, and their
 *    contents are not read; any other arrays are uploaded;
 *  BORN_HOST_LEVELS_VERIFY: as RESIDENT, but born_source_prop records a
 *    64-bit checksum of each host array it writes and this call re-computes
 *    it: arrays whose contents changed since are uploaded;
 *  BORN_HOST_LEVELS_UPLOAD: like cpuProp, the arrays are always read (one
 *    upload of both levels per call).
 * The device levels are advanced by the reverse-time reconstruction, as
 * cpuProp advances the arrays it is given; a second call on unchanged
 * arrays continues from there under RESIDENT and VERIFY.  p0/p1 non-null;
 * FP32 level storage when an upload is needed. */
#define BORN_HOST_LEVELS_RESIDENT 0
#define BORN_HOST_LEVELS_VERIFY 1
#define BORN_HOST_LEVELS_UPLOAD 2
int born_set_host_levels(born_handle *h, int policy);
int born_rtm_adjoint_host(born_handle *h, int jtd, int nt, const float *p0,
                          const float *p1, float *img);
int born_rtm_forward(born_handle *h, int jt, int nt, float *traces_out);

/* Nonlinear modelling through vel2 with the taper (the background of
 * rtmForward, cpu_prop.cc:36-45): traces accumulate into the device traces
 * of born_set_receiver_func (copied to traces_out when non-null). */
int born_model(born_handle *h, int jt, int nt, float *traces_out);
/* Exact linearised Born forward: derivative of born_model with respect to
 * vel2 (v^2 dt^2) along the perturbation given by born_set_reflectivity.
 * Traces accumulate into the device traces. */
int born_lin_forward(born_handle *h, int jt, int nt, float *traces_out);
/* Exact adjoint of born_lin_forward: reads the device traces, returns the
 * model-space gradient (n1*n2*n3) in model_out (also left in the device
 * image).  The background is checkpointed every `interval` steps (two levels
 * per checkpoint) and recomputed segment by segment.  The checkpoints come
 * from a forward sweep of the background, which is skipped when the
 * checkpoints already held are those of the same background: stored by
 * born_lin_forward (every born_set_checkpoint_interval steps, 50 by
 * default) or by an earlier adjoint, with vel2, the source points and
 * traces, the source sinc table and the grid unchanged since and the same
 * jt, nt and interval.  The result does not depend on which way the
 * checkpoints were made (the background step is the same arithmetic). */
int born_lin_adjoint(born_handle *h, int jt, int nt, int interval,
                     float *model_out);
/* Checkpoint interval at which born_lin_forward stores the background (0:
 * it stores none; 2 * ceil(nt / interval) levels of n1*n2*n3 floats are
 * kept per handle). */
int born_set_checkpoint_interval(born_handle *h, int interval);
/* 1 when the last born_lin_adjoint reused checkpoints instead of sweeping
 * the background, else 0. */
int born_checkpoints_reused(const born_handle *h);
/* Storage of the exact adjoint's checkpoints: FP32 (default; the gradient is
 * the exact transpose), or FP16 (half the memory): each checkpoint keeps
 * the current level s_t and the difference s_{t-1} - s_t, each with its own
 * power-of-two scale 2^(ceil(log2 max|v|) - 15) chosen on the device, and
 * s_{t-1} is rebuilt in FP32 from the two; each segment is then recomputed
 * from levels rounded to FP16, so the gradient is the transpose to about
 * FP16 rounding. */
#define BORN_CKPT_F32 0
#define BORN_CKPT_F16 1
int born_set_checkpoint_storage(born_handle *h, int storage);

/* Phase timing of born_lin_adjoint (off by default): with enable != 0 the
 * loop records a CUDA event at every phase boundary on the handle's stream
 * and, at its end, waits for them; born_phase_times then gives the last
 * call's ms in ms[0..3] = forward sweep (with the checkpoint stores),
 * segment restores and recompute (storing A s), reverse adjoint steps,
 * final division by v^2 dt^2. */
int born_time_phases(born_handle *h, int enable);
int born_phase_times(const born_handle *h, float *ms, int n);

/* Device results and state transfers (host arrays of n1*n2*n3 floats, or
 * npts*nt_big for traces) */
int born_get_image(born_handle *h, float *img_out);
/* Device address of the image (n1*n2*n3 floats on the handle's device,
 * written on the handle's stream; valid until the next create_space or
 * destroy), for stacking images across shots and GPUs without a host copy
 * (the reference sums shot images on the host, util/Add).  Null without a
 * grid. */
float *born_image_device(born_handle *h);
int born_get_traces(born_handle *h, float *traces_out);
int born_get_source_levels(born_handle *h, float *p0_out, float *p1_out);
int born_set_source_levels(born_handle *h, const float *p0, const float *p1);
int born_zero_traces(born_handle *h);
int born_synchronize(born_handle *h);

/* ======================================================================
 * 3. Born operator (model image <-> shot data) and CG least squares
 *
 * born_op is rtm_zero_op (base/rtm_zero_op_3d.h:10-43) behind the
 * my_operator contract forward/adjoint(add, model, data)
 * (base/my_operator.h:18-25): add = 0 zeroes the output first.  Unlike the
 * reference (which reads the model from a file member and writes data to a
 * file, rtm_zero_op_3d.cc:161,193,295) it reads and writes the vectors it is
 * given.  Vectors are DEVICE pointers on the handle's device:
 *   model: velocity/image grid n3 x n2 x n1 floats,
 *   data:  nshots x rec_ny x rec_nx x nt_data floats (time fastest).
 * exact = 0 reproduces rtm_zero_op (random-boundary RTM adjoint, 1e-6 Born
 * coupling); exact = 1 uses the exact linearised pair, so adjoint is the
 * transpose of forward (dot-product test) and CG converges.
 * ====================================================================== */
typedef struct born_op born_op;
typedef struct {
  int n1, n2, n3;          /* model grid (velocity and image) */
  float o1, o2, o3, d1, d2, d3;
  int nt_data;             /* data time samples */
  float dt_data;
  int rec_nx, rec_ny;      /* receiver grid at rec_depth */
  float rec_ox, rec_dx, rec_oy, rec_dy, rec_depth;
  int nshots;              /* shot positions given to born_op_create */
  int nt_wavelet;          /* raw source wavelet (its time derivative is
                              injected, source_func_3d.cc:120-124) */
  float dt_wavelet;
  int nbound;              /* absorbing / random boundary cells (fd_prop_3d.cc:48-53) */
  int exact;               /* 0: reference operator, 1: exact linearised pair */
  int ckpt_interval;       /* exact adjoint checkpoint interval (0: 50) */
} born_op_params;

/* velocity: host n3 x n2 x n1 m/s; shots: host nshots x (x, y, z);
 * wavelet: host nt_wavelet samples.  Builds the compute grid, sinc tables,
 * receiver and source geometry and the v^2 dt^2 models (one random-boundary
 * model per shot in reference mode) on the device of h. */
int born_op_create(born_handle *h, const born_op_params *p,
                   const float *velocity, const float *shots,
                   const float *wavelet, born_op **out);
int born_op_destroy(born_op *op);
int born_op_sizes(const born_op *op, long long *model_n, long long *data_n,
                  int *nt_fd, float *dt_fd);
/* Exact mode keeps each shot's background checkpoints across operator
 * applications (the background does not depend on the model), as many
 * shots as fit while a quarter of the device memory stays free, so a
 * shot's adjoint after its linearised forward skips the checkpoint sweep.
 * born_op_checkpoint_shots: shots holding checkpoints;
 * born_op_checkpoints_reused: shot adjoints that skipped their sweep. */
int born_op_checkpoint_shots(const born_op *op);
long long born_op_checkpoints_reused(const born_op *op);
int born_op_forward(born_op *op, int add, const float *model, float *data);
int born_op_adjoint(born_op *op, int add, float *model, const float *data);
/* FP64 dot product of two device float vectors (block partials in double),
 * the dot of hypercube_float (hypercube_float.cc:120-130) on the device. */
int born_dot_f64(born_op *op, const float *a, const float *b, long long n,
                 double *out);

/* Device vectors of n floats on the operator's device, and the vector
 * algebra of the reference's hypercube_float (the my_vector that
 * rtm_zero_op and lin_solver use, base/my_vector.h:7-91), ordered on the
 * operator's stream: factors are double, each element is formed in double
 * and stored as float, as hypercube_float does.  csrc/born_my_operator.h
 * wraps them in a my_vector subclass so that the reference's lin_solver /
 * cgstep drive the operator unchanged.
 *   create:    x = 0 (cudaMalloc);  destroy: waits for the stream, frees
 *   fill:      x = val                    (hypercube_float.cc:50-52)
 *   scale:     x = x r                    (hypercube_float.h:25-27)
 *   scale_add: x = x a + y b              (hypercube_float.cc:213-222)
 *   lincomb:   x = y a + z b              (hypercube_float.cc:140-151)
 *   add:       x = x + y  (float add)     (hypercube_float.cc:223-228)
 *   copy, upload (host -> device), download (device -> host); the two host
 *   copies return when done. */
int born_vec_create(born_op *op, long long n, float **out);
int born_vec_destroy(born_op *op, float *x);
int born_vec_fill(born_op *op, float *x, long long n, double val);
int born_vec_scale(born_op *op, float *x, long long n, double r);
int born_vec_scale_add(born_op *op, float *x, double a, const float *y,
                       double b, long long n);
int born_vec_lincomb(born_op *op, float *x, double a, const float *y,
                     double b, const float *z, long long n);
int born_vec_add(born_op *op, float *x, const float *y, long long n);
int born_vec_copy(born_op *op, float *dst, const float *src, long long n);
int born_vec_upload(born_op *op, float *dst, const float *host, long long n);
int born_vec_download(born_op *op, float *host, const float *src,
                      long long n);
/* Least squares by Claerbout's CG (lin_solver.cc:104-132, cgstep.cc:11-54):
 * model (device, in: starting model, out: solution); resid (host, niter+1
 * doubles, nullable) receives rr.rr before and after every iteration. */
int born_cg_solve(born_op *op, const float *data, float *model, int niter,
                  double *resid);

/* ======================================================================
 * 4. Batched shots
 *
 * A batch advances several fully set-up shot handles together: every time
 * step is one launch covering all shots' tiles (shots may have different
 * grids), and with graphs on (default) each whole time loop is recorded once
 * into a CUDA graph and replayed.  All shots must share the sinc tables,
 * trace lengths and grid spacing.  Results stay in each shot handle (read
 * them with born_get_image / born_get_traces; work later queued on a shot's
 * stream waits for the batch).  A shot handle must not run its own time
 * loops while a batch that holds it is running.  Reallocating a shot's
 * buffers (create_space, new point sets, new sinc tables) makes the batch
 * rebuild its descriptors and graphs on the next call.
 * ====================================================================== */
typedef struct born_batch born_batch;
int born_batch_create(born_handle *const *shots, int nshots,
                      born_batch **out);
int born_batch_destroy(born_batch *b);
const char *born_batch_error(const born_batch *b);
int born_batch_set_graph(born_batch *b, int use_graph);
void *born_batch_stream(born_batch *b);
/* Kernels the batch has run (a replayed time loop counts its kernels) and
 * replays of recorded time loops. */
long long born_batch_launches(const born_batch *b);
long long born_batch_graph_launches(const born_batch *b);
/* born_source_prop / born_rtm_adjoint (swap = 1) / born_rtm_forward for
 * every shot of the batch, with device-resident results. */
int born_batch_source_prop(born_batch *b, int jts, int nt);
int born_batch_rtm_adjoint(born_batch *b, int jtd, int nt);
int born_batch_rtm_forward(born_batch *b, int jt, int nt);
int born_batch_synchronize(born_batch *b);

/* FP64 dot product that allocates nothing.  No counterpart in the
 * reference.  For callers that cannot allocate device memory where they need
 * a dot product: applications whose GPU memory is all owned by their own
 * pool, and code that keeps other streams busy and cannot take the
 * device-wide synchronisation of cudaMalloc/cudaFree.  a, b: device float
 * vectors of n elements on the current device; out: host double; stream: a
 * cudaStream_t (null for the default stream); the call waits for the result.
 * Its scratch is a fixed file-scope device array of 65536 partial sums
 * (512 KiB, held by every GPU that loads the library until exit), so n is
 * limited to BORN_DOT_NOALLOC_MAX elements; larger n returns BORN_EINVAL.
 * All calls share that array: calls that overlap on the GPU race.  The first
 * call on a device looks up the array's address on that device; make it
 * before any stream capture begins.  The address is kept for the life of
 * the process, for device indices 0..63 (higher indices return
 * BORN_ENODEV); after cudaDeviceReset the kept address is stale, so do not
 * call this function on a device that was reset.  If the calling thread
 * already has a CUDA error pending, the call returns BORN_ECUDA and leaves
 * that error pending (it launches nothing). */
#define BORN_DOT_NOALLOC_MAX 268435456LL
int born_dot_f64_noalloc(const float *a, const float *b, long long n,
                         double *out, void *stream);

/* Measurement: the bandwidth (GB/s, read + write bytes) that plain float4
 * loads and stores sustain over `reads` input and `writes` output arrays of
 * n floats each (1 <= reads <= 8, 1 <= writes <= 4, n a multiple of 4), on
 * the current device: the streaming ceiling of a step kernel's mix of arrays
 * (RTM adjoint 7 + 3, Born forward 6 + 2, source propagation 3 + 1).  No
 * reference counterpart.  Allocates and frees (reads + writes) * n floats;
 * best of two grid sizes, `reps` timed launches each. */
int born_stream_mix_gbs(int reads, int writes, long long n, int reps,
                        float *gbs);

/* Tuning: tile configuration index (0..born_tile_config_count()-1, or -1 for
 * the built-in choice) and z-segment depth (0 = automatic). */
int born_tile_config_count(void);
int born_set_tiling(born_handle *h, int tile_cfg, int zseg);
/* Step launches with programmatic dependent launch (default on): each time
 * step's grid may become resident while the previous step's last CTAs
 * finish, and waits for that grid on the device before reading or writing
 * anything, which hides the launch gap between steps.  enable = 0 launches
 * every step plainly.  Results are the same either way. */
int born_set_launch_overlap(born_handle *h, int enable);
/* Closing host copies of the time loops (source_prop's levels, the RTM
 * image, the forward's traces), default on: when the destination is
 * page-locked host memory of 8 MiB or more and the loop has 100 steps or
 * more, the call first copies into it on a side stream while the loop runs,
 * then overwrites every byte with the result.  The first copy into such an
 * array after other host arrays were copied took 2-24 ms per 199 MB on
 * GB300, against 0.96 ms for the next one; the warming copy takes that cost
 * off the loop's critical path.  The destination's contents are undefined
 * during the call and after a failed one (a successful call leaves the
 * result); enable = 0 leaves it untouched until the closing copy. */
int born_set_host_prewarm(born_handle *h, int enable);
/* Warming copies made so far by the handle. */
long long born_host_prewarm_count(const born_handle *h);
/* Autotuner: with enable != 0, times every tile configuration of each step
 * mode on the current grid now (needs the grid and both velocities) and
 * uses the fastest; time loops also tune a mode lazily on first use while
 * enabled and no fixed tiling is set, and loops of 400 steps or more then
 * refine the tile and its z segments on their own steps (every tiling gives
 * the same results; born_loop_tile_ms reports what they measured).  enable = 0 turns both off.
 * A new grid (born_create_space) clears every choice. */
int born_autotune(born_handle *h, int enable);
/* Tile configuration in use for a step mode (0 source, 1 rtm forward,
 * 2 rtm adjoint, 3 modelling, 4 linearised forward, 5 its adjoint) and the
 * tuner's time per launch. */
int born_tuned_config(const born_handle *h, int mode, int *cfg,
                      float *ms_per_launch);
/* z-segment depth (planes per CTA) that a step of the mode uses now on the
 * current grid: the fixed one, else the one tuned with the tile, else the
 * sizing rule's.  Negative BORN_E* on error. */
int born_tuned_zseg(born_handle *h, int mode);
/* Time loops of 400 steps or more refine a mode's tiling, tile and z
 * segments together, on their own steps (every tiling gives the same
 * results; a loop too short for the whole sweep leaves the rest to the next
 * loop of the mode): ms[c] receives the time per launch the last complete
 * refinement of the mode measured for tile configuration c with its best z
 * segmentation (0 when not measured), for c < n, under the current
 * storage. */
int born_loop_tile_ms(const born_handle *h, int mode, float *ms, int n);
/* Failure-detection self-test: launches one kernel whose bounded device
 * wait (the step kernels' wait on their TMA copies) waits on something that
 * never completes; after about 2 s it gives up, sets the handle's error word
 * and returns.  Returns BORN_ETIMEOUT when detection works; the error word is
 * then cleared and the handle stays usable.  No reference counterpart (the
 * reference's kernels do not wait on each other). */
int born_selftest_wait_timeout(born_handle *h);
/* Kernels launched on this handle since creation (for accounting). */
long long born_kernel_launches(const born_handle *h);

/* Storage of the propagated wavefield levels.  No counterpart in the
 * reference (its levels are float).  BF16 and FP16 store every level as
 * 16-bit values with a power-of-two scale of its own (chosen on the device
 * from a bound on the level's magnitude, so FP16 neither overflows nor
 * underflows), while the stencil, the taper, injection, extraction, the Born
 * coupling and the image stay FP32; velocities, reflectivity, image and
 * traces stay FP32.  16-bit storage halves the bytes of every level read and
 * write; its error against an FP64 propagation is that of rounding every
 * stored level (it grows with the number of steps).  Supported by the
 * source, rtm adjoint and rtm forward loops (handle and batch); modelling,
 * the exact linearised pair, host copies of the source levels and the
 * operator need FP32 and return BORN_ESTATE otherwise.  Needs nx % 8 == 0.
 * Changing it clears the levels (run source_prop again). */
#define BORN_STORE_F32 0
#define BORN_STORE_BF16 1
#define BORN_STORE_F16 2
/* FP32 levels with the stencil and leapfrog formed by fused multiply-adds
 * in the source, adjoint and forward loops: not bit-identical to the
 * reference (within a relative L2 of 1e-5 of it), fewer instructions per
 * cell.  The other loops keep the reference order. */
#define BORN_STORE_F32_FUSED 3
/* FP32 levels in the reference's operation order, and the rtm forward
 * loop's Born coupling r += 1e-6 s img formed exactly as the reference's
 * double expression (base/cpu_prop.cc:216-223, a double literal times float
 * fields, rounded once to float): traces bit-identical to the reference
 * instead of within about 2e-6 relative L2.  The coupling is evaluated in
 * float arithmetic (exact products and sums plus a rounding-boundary test)
 * and falls back to double for the few cells the test cannot decide.  Every
 * other step is the BORN_STORE_F32 one. */
#define BORN_STORE_F32_EXACT 4
/* The exact coupling's arithmetic on device arrays of n values:
 * out[i] = (float)((double)r[i] + 1e-6 * (double)s[i] * (double)m[i]), as
 * the rtm forward step under BORN_STORE_F32_EXACT forms it (two cells per
 * thread); for testing that arithmetic on chosen inputs.  Enqueued on
 * `stream` (a cudaStream_t; null for the legacy default stream). */
int born_couple_exact_device(const float *r, const float *s, const float *m,
                             float *out, long long n, void *stream);
int born_set_storage(born_handle *h, int storage);
int born_get_storage(const born_handle *h);
/* Raw CUDA stream of the handle (cudaStream_t), for event timing. */
void *born_stream(born_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* BORN_GB300_H */
