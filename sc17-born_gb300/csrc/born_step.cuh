// Fused 2.5D time-step kernels for the Born / RTM hot path on sm_103a.
//
// One launch advances one FD time step of one or two coupled wavefields over
// the interior [4, n-4)^3 of a [n3][n2][n1] float grid (n1 fastest).  Work is
// split into xy tiles (TX x TY cells) and z segments; each CTA marches its
// segment plane by plane.  The current wavefield of every propagated field is
// brought in by TMA (cp.async.bulk.tensor.3d) as a (TX+8) x (TY+8) box per
// plane into an S-stage shared-memory ring guarded by mbarriers; the x/y
// neighbours come from that box, the 9-plane z window lives in registers.
// The previous level, velocity and image are read once per cell with float4
// loads and the new level is written once, so HBM sees the compulsory bytes.
//
// What is fused into the pass (reference base/cpu_prop.cc):
//   prop (224-253)       stencil, same left-to-right sum, no FMA contraction
//   damp (141-165)       the new level is scaled by b(edge); the scaling that
//                        the reference applies in place to the current level
//                        is applied when that level is read back as "old"
//   injectSource (166-179) / injectReceivers (180-197)
//                        at the cell that owns each point, in point order
//   imageAdd (216-223)   Born coupling r += 1e-6 s img
//   dataExtract (198-215) receiver traces accumulate in place
//   imageCondition (97-105) img += s r
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace born {

constexpr int kRadius = 4;
constexpr int kNBound = 40;  // taper table length (cpu_prop.cc:329-332)

enum StepMode : int { kModeSource = 0, kModeForward = 1, kModeAdjoint = 2 };

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
  int id;                 // first trace sample used this step
  int active;             // reference guard: id + 7 < nt_trace
  float scale;            // dir / jt for injection, unused for extraction
  float tab[8];           // sinc row for this step
};

struct StepParams {
  int n1, n2, n3;
  int tiles_x, tiles_y, zseg;
  float c[13];             // stencil coefficients, slots as cpu_prop.cc:6-18
  float bound[kNBound];
  // field A: source mode p, forward s, adjoint r
  const float *a_cur;
  float *a_old;            // previous level in, new level out
  const float *a_vel;
  // field B: forward r, adjoint s
  const float *b_cur;
  float *b_old;
  const float *b_vel;
  float *img;              // forward: reflectivity (read); adjoint: image
  PointSet pa;             // injection into the new level of A
  PointSet pb;             // forward: extraction from B; adjoint: injection
                           // still owed to B's previous level
  unsigned int *err;       // device error word (bit 0: mbarrier wait gave up)
};

constexpr unsigned int kErrWaitTimeout = 1u;

template <int TX, int TY>
struct TileShape {
  static constexpr int kTX = TX, kTY = TY;
  static constexpr int kBX = TX + 2 * kRadius, kBY = TY + 2 * kRadius;
  static constexpr int kBoxFloats = kBX * kBY;
  // stage pitch rounded to 128 B (TMA destination alignment)
  static constexpr int kBoxPitch = ((kBoxFloats * 4 + 127) / 128) * 32;
  static constexpr int kThreads = (TX / 4) * TY;
};

constexpr int kStages = 8;

// Host-side launch entry (defined in born_step.cu).  tm_a / tm_b are the
// tensor maps of the current level of field A / B (unused ones may be any
// valid map).  pa/pb flags say which fields are propagated this step.
cudaError_t launch_step(int mode, bool prop_a, bool prop_b, int tile_cfg,
                        const CUtensorMap &tm_a, const CUtensorMap &tm_b,
                        const StepParams &p, cudaStream_t stream);

// Tile configurations (index -> TX, TY).
int tile_cfg_count();
void tile_cfg_dims(int cfg, int *tx, int *ty);
size_t step_smem_bytes(int tile_cfg, int nfields);

// Small kernel: add a pending injection into a buffer at the points of a set
// (used once at the end of the adjoint so the source level left in memory
// matches the reference's in-place injection).
cudaError_t launch_point_inject(const PointSet &ps, int npts, float *field,
                                cudaStream_t stream);

}  // namespace born
