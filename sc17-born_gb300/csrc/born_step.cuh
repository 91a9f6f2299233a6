// Fused 2.5D time-step kernels for the Born / RTM hot path on sm_103a.
//
// One launch advances one FD time step of one or two coupled wavefields over
// the interior [4, n-4)^3 of a [n3][n2][n1] float grid (n1 fastest).  Work is
// split into xy tiles (TX x TY cells) and z segments; each CTA marches its
// segment plane by plane.  All HBM reads are asynchronous TMA copies
// (cp.async.bulk.tensor.3d) completing on mbarriers, in two small rings:
//   * z ring (kZStages): the TX x TY centre tile of every propagated field's
//     current level for each new plane; its values enter the 9-plane z window
//     kept in registers;
//   * output ring (out_stages(mode) deep): for the plane being written, the
//     (TX+8) x (TY+8) halo box of every propagated field (x/y neighbours) and
//     the per-cell inputs (previous levels, velocities, image or
//     reflectivity), one TX x TY tile each.
// A plane's centre is thus read twice (z ring, then inside its box four
// planes later, from L2), which keeps the shared memory per CTA small enough
// for three 128-thread CTAs per SM.
// The stencil's neighbour sums and running sums, the leapfrog and the
// imaging adds run on packed FP32 pairs (add/sub.rn.f32x2: two cells per
// instruction, each lane rounded like the scalar form); the products of the
// reference-order arithmetic stay scalar mul.rn (see f32x2 in
// born_step_impl.cuh).
// The new level (and the image) are written once with float4 stores, so HBM
// sees the compulsory bytes only.
//
// Reference semantics fused into the pass (base/cpu_prop.cc):
//   prop (224-253)       stencil, same left-to-right sum, no FMA contraction
//                        (bit-identical, also in the packed pairs)
//   damp (141-165)       the new level is scaled by b(edge); the scaling that
//                        the reference applies in place to the current level
//                        is applied when that level is read back as "old"
//   injectSource (166-179) / injectReceivers (180-197)
//                        at the cell that owns each point, in point order
//   imageAdd (216-223)   Born coupling r += 1e-6 s img
//   dataExtract (198-215) receiver traces accumulate in place
//   imageCondition (97-105) img += s r
// plus the exact linearised Born pair (modes kModeBornLin / kModeBornAdj)
// and plain nonlinear modelling (kModeModel), used for the dot-product and
// finite-difference checks and for least-squares migration.
//
// The levels of the propagated fields may be stored as FP32 (the parity
// path, reference operation order; or with fused multiply-adds), BF16 or
// FP16 (Storage): 16-bit levels carry a power-of-two scale each, chosen on
// the device from a bound on the level's magnitude, and are decoded to FP32
// as they are read; the arithmetic stays FP32.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace born {

constexpr int kRadius = 4;
constexpr int kNBound = 40;  // taper table length (cpu_prop.cc:329-332)

enum StepMode : int {
  kModeSource = 0,   // sourceProp step (one field, no taper)
  kModeForward = 1,  // rtmForward step (s and r, taper, 1e-6 coupling)
  kModeAdjoint = 2,  // rtmAdjoint step (r with taper, s rebuilt, image)
  kModeModel = 3,    // nonlinear modelling step with taper (+ A s output)
  kModeBornLin = 4,  // exact linearised Born step: r += m * (A s) inside taper
  kModeBornAdj = 5,  // its exact adjoint: w step, image += g * w
};

// Device view of a set of points (sources or receivers) on the grid.
// Points are sorted by cell, then by their original index; plane_off[z] is
// the offset of plane z's n1*n2 head map in cell_head, or -1 when the plane
// holds no point.  cell_head gives the first slot of a cell or -1.
struct PointSet {
  const int *plane_off;
  const int *cell_head;
  const int *slot_cell;   // linear cell index of each slot
  const int *slot_index;  // original point index (trace row) of each slot
  float *traces;          // [npts][nt_trace]
  int npts;
  int nt_trace;
  int zlo, zhi;           // planes holding points (skip the lookup elsewhere)
  int id;                 // first trace sample used this step
  int active;             // reference guard: id + 7 < nt_trace
  float scale;            // dir / jt for injection, unused for extraction
  float tab[8];           // sinc row for this step
  // 16-bit storage: bound of |trace| (device word, float bits) and the most
  // points sharing one cell, for the amplitude bound of an injection
  const unsigned int *absmax;
  int mult;
};

// Storage of the propagated wavefield levels (and the arithmetic that goes
// with it).  Velocities, image and reflectivity stay FP32.  kStoreF32 keeps
// the reference's operation order (bit-identical results); kStoreF32Fused
// keeps FP32 levels but forms the stencil and leapfrog with fused
// multiply-adds; with 16-bit storage the stencil still accumulates in FP32
// (fused) and every stored level carries its own power-of-two scale.
enum Storage : int { kStoreF32 = 0, kStoreBF16 = 1, kStoreF16 = 2,
                     kStoreF32Fused = 3, kStoreF32Exact = 4,
                     kNumStorages = 5 };
inline bool storage_16bit(int st) {
  return st == kStoreBF16 || st == kStoreF16;
}
inline int storage_esize(int st) { return storage_16bit(st) ? 2 : 4; }

// Per-level scale records (16-bit storage).  Each level buffer has two
// record slots, used alternately by its successive writes, so that a step
// reads the records of its current and previous levels while it fills the
// record of the level it writes.  A slot is two words: [0] = (tag << 32) |
// bits of max|value| (accumulated with atomicMax, the tag increasing with
// every write within a time loop, so a stale maximum never survives), [1] =
// bits of the level's scale (stored value = true value / scale).
struct LevelRefs {
  int cur, old, out;  // record slots; -1 when the level is not read/written
  unsigned int tag;
};

// Centre-tile slots (TMA maps cm[slot] in the launch)
enum CentreSlot : int { kOldA = 0, kOldB = 1, kVelA = 2, kVelB = 3, kImg = 4 };
constexpr int kNumCentre = 5;

struct StepParams {
  int n1, n2, n3;
  int tiles_x, tiles_y, zseg;
  float c[13];             // stencil coefficients, slots as cpu_prop.cc:6-18
  float bound[kNBound];
  // outputs (in-place over the previous level; element type per storage)
  void *a_out;             // field A: source p / forward s / adjoint r / w
  void *b_out;             // field B: forward r / adjoint s
  float *img_out;          // adjoint image (read through the centre ring)
  float *g_out;            // kModeModel: A s of the current level, or null
  PointSet pa;             // injection into the new level of A
  PointSet pb;             // forward / linearised: extraction from B;
                           // adjoint: injection owed to B's previous level;
                           // model: extraction from A
  unsigned int *err;       // device error word (bit 0: mbarrier wait gave up)
  // 16-bit storage only
  unsigned long long *lv;  // level records [slot][2]
  LevelRefs la, lb;        // records of fields A and B this step
  float csum;              // |c0| + 2 sum |ci|: stencil gain per unit v^2 dt^2
  const unsigned int *vmax_a, *vmax_b;  // max v^2 dt^2 seen by A / B
  const unsigned int *imgmax;           // max |reflectivity| (Born coupling)
  // host side only: launch with programmatic stream serialization (the
  // kernel waits for the previous grid itself, griddepcontrol.wait)
  int overlap;
  int pad_;
};

constexpr unsigned int kErrWaitTimeout = 1u;
constexpr int kZStages = 3;  // largest z-window ring depth (planes ahead)
// z-ring depth of a mode (at most kZStages)
constexpr int z_stages(int mode) {
  (void)mode;
  return kZStages;
}
constexpr int kOStages = 3;  // largest output ring depth (planes 2 ahead)
// output ring depth of a mode (at most kOStages).  The forward step ran
// with two stages, so that a 64x8 tile fits four CTAs per SM (shared
// memory) instead of three; once its z segments were refined in the loop
// and the step launches overlapped, three stages at three CTAs per SM were
// faster (368^3 grid: 529.8 against 537.0 ms per 2000 steps).
constexpr int out_stages(int mode) {
  (void)mode;
  return kOStages;
}

struct StepMaps {
  CUtensorMap box_a, box_b;       // halo boxes of the current levels
  CUtensorMap zc_a, zc_b;         // centre tiles of the current levels
  CUtensorMap cm[kNumCentre];     // centre tiles, by CentreSlot
};

// One shot of a batched launch (device memory).  `params` holds the shot's
// static step parameters (grid, tiling, coefficients, image/g outputs, point
// set arrays); the outputs and descriptors follow the parity of the level
// rotation.
struct BatchShot {
  StepParams params;
  void *a_out[2], *b_out[2];
  StepMaps maps[2];
};

// Scalars that change from step to step, shared by every shot.
struct StepVar {
  int parity;
  int pa_id, pa_active;
  float pa_scale;
  float pa_tab[8];
  int pb_id, pb_active;
  float pb_scale;
  float pb_tab[8];
  LevelRefs la, lb;  // 16-bit storage: the same rotation for every shot
};

// Batched launch over nshots shots; block_start[s] is the first CTA of shot
// s and block_start[nshots] the total.  total_blocks == 0 only prepares the
// kernel (its shared-memory attribute), so that a later launch can be
// recorded into a graph.
cudaError_t launch_step_batched(int storage, int mode, bool prop_a,
                                bool prop_b, int tile_cfg,
                                const BatchShot *shots, const int *block_start,
                                int nshots, int total_blocks,
                                const StepVar &var, cudaStream_t stream);

// Host-side launch entry (defined in born_step.cu).  prop_a / prop_b say
// which fields are propagated this step (adjoint first/last steps).  The
// 16-bit and fused FP32 storages support the source, forward and adjoint
// modes.
cudaError_t launch_step(int storage, int mode, bool prop_a, bool prop_b,
                        int tile_cfg, const StepMaps &maps,
                        const StepParams &p, cudaStream_t stream);

// Which centre slots a mode reads (bit mask over CentreSlot).
unsigned centre_mask(int mode, bool prop_a, bool prop_b);
// Centre slots holding levels of the propagated fields (stored with the
// field storage; the others are FP32).
inline bool field_slot(int mode, int slot) {
  return slot == kOldA || (slot == kOldB && mode != kModeBornAdj);
}

// Tile configurations (index -> TX, TY).
int tile_cfg_count();
void tile_cfg_dims(int cfg, int *tx, int *ty);
size_t step_smem_bytes(int storage, int tile_cfg, int mode, bool prop_a,
                       bool prop_b);

// Small kernels.
// Adds the injection of `ps` into `field` at its points (one thread, point
// order).  16-bit storage: decoded and re-encoded with the scale of record
// slot `rec` of `lv`.
cudaError_t launch_point_inject(const PointSet &ps, int npts, void *field,
                                int storage, unsigned long long *lv, int rec,
                                cudaStream_t stream);
// Level records: reset both slots of buffer `buf` (zero level, scale 1), or
// copy slot `src` into slot `dst` with a new tag.
cudaError_t launch_level_reset(unsigned long long *lv, int buf,
                               cudaStream_t stream);
cudaError_t launch_level_copy(unsigned long long *lv, int dst, int src,
                              unsigned int tag, cudaStream_t stream);
// *out = max(*out, max |x[i]|) as float bits (out zeroed by the caller).
cudaError_t launch_absmax(const float *x, long long n, unsigned int *out,
                          cudaStream_t stream);
// Checkpoints of the exact adjoint in FP16: snapshot writes v = x (or
// x - y when y is not null; n floats) as FP16 values with the power-of-two
// scale 2^(ceil(log2 max|v|) - 15) stored in *scale (maxw: a device word the
// call uses to find max|v|); restore writes the FP16 values times *scale
// (plus base[i] when base is not null) back as FP32.  No host
// synchronisation.
cudaError_t launch_snapshot_f16(const float *x, const float *y, long long n,
                                unsigned int *maxw, void *out, float *scale,
                                cudaStream_t stream);
cudaError_t launch_restore_f16(const void *in, long long n,
                               const float *scale, const float *base,
                               float *x, cudaStream_t stream);
// out[i] = a[i] / v[i] over the whole grid (image of the exact adjoint).
cudaError_t launch_divide(const float *a, const float *v, float *out,
                          long long n, cudaStream_t stream);
// One bounded wait that runs out (about 2 s) and sets kErrWaitTimeout in
// *err: the failure-detection self-test.
cudaError_t launch_wait_timeout_probe(unsigned int *err, cudaStream_t stream);

}  // namespace born
