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
//   * output ring (kOStages): for the plane being written, the
//     (TX+8) x (TY+8) halo box of every propagated field (x/y neighbours) and
//     the per-cell inputs (previous levels, velocities, image or
//     reflectivity), one TX x TY tile each.
// A plane's centre is thus read twice (z ring, then inside its box four
// planes later, from L2), which keeps the shared memory per CTA small enough
// for three 128-thread CTAs per SM.
// The new level (and the image) are written once with float4 stores, so HBM
// sees the compulsory bytes only.
//
// Reference semantics fused into the pass (base/cpu_prop.cc):
//   prop (224-253)       stencil, same left-to-right sum, no FMA contraction
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
};

// Centre-tile slots (TMA maps cm[slot] in the launch)
enum CentreSlot : int { kOldA = 0, kOldB = 1, kVelA = 2, kVelB = 3, kImg = 4 };
constexpr int kNumCentre = 5;

struct StepParams {
  int n1, n2, n3;
  int tiles_x, tiles_y, zseg;
  float c[13];             // stencil coefficients, slots as cpu_prop.cc:6-18
  float bound[kNBound];
  // outputs (in-place over the previous level)
  float *a_out;            // field A: source p / forward s / adjoint r / w
  float *b_out;            // field B: forward r / adjoint s
  float *img_out;          // adjoint image (read through the centre ring)
  float *g_out;            // kModeModel: A s of the current level, or null
  PointSet pa;             // injection into the new level of A
  PointSet pb;             // forward / linearised: extraction from B;
                           // adjoint: injection owed to B's previous level;
                           // model: extraction from A
  unsigned int *err;       // device error word (bit 0: mbarrier wait gave up)
};

constexpr unsigned int kErrWaitTimeout = 1u;
constexpr int kZStages = 3;  // z-window ring depth (new planes, 2 ahead)
constexpr int kOStages = 3;  // output ring depth (output planes, 2 ahead)

struct StepMaps {
  CUtensorMap box_a, box_b;       // halo boxes of the current levels
  CUtensorMap zc_a, zc_b;         // centre tiles of the current levels
  CUtensorMap cm[kNumCentre];     // centre tiles, by CentreSlot
};

// Host-side launch entry (defined in born_step.cu).  prop_a / prop_b say
// which fields are propagated this step (adjoint first/last steps).
cudaError_t launch_step(int mode, bool prop_a, bool prop_b, int tile_cfg,
                        const StepMaps &maps, const StepParams &p,
                        cudaStream_t stream);

// Which centre slots a mode reads (bit mask over CentreSlot).
unsigned centre_mask(int mode, bool prop_a, bool prop_b);

// Tile configurations (index -> TX, TY).
int tile_cfg_count();
void tile_cfg_dims(int cfg, int *tx, int *ty);
size_t step_smem_bytes(int tile_cfg, int mode, bool prop_a, bool prop_b);

// Small kernels.
cudaError_t launch_point_inject(const PointSet &ps, int npts, float *field,
                                cudaStream_t stream);
// out[i] = a[i] / v[i] over the whole grid (image of the exact adjoint).
cudaError_t launch_divide(const float *a, const float *v, float *out,
                          long long n, cudaStream_t stream);

}  // namespace born
