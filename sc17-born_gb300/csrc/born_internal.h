// Internal definitions shared by the C ABI translation units (not part of
// the public interface).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/born_gb300.h"
#include "born_step.cuh"

// Level buffers of a handle (index of their level records) and the device
// words holding the maxima that 16-bit storage bounds amplitudes with.
enum LevelBuf : int { kBufS0 = 0, kBufS1, kBufR0, kBufR1, kBufF0, kBufF1,
                      kNumLevelBufs };
enum StatWord : int { kStatVel1 = 0, kStatVel2, kStatRefl, kStatSrc, kStatRec,
                      kNumStats };

// Tags of the level records written by each time loop (16-bit storage):
// every loop writes increasing tags above those of the loops whose levels it
// reads, and clears the records of the levels it starts from zero, so the
// tags of a replayed loop are the same as those of its first run.
constexpr unsigned int kTagSource = 1u;
constexpr unsigned int kTagAdjoint = 1u << 30;
constexpr unsigned int kTagForward = 2u << 30;

// Device copy of one point set (sources or receivers).
struct DevPoints {
  int npts = 0, nt = 0;
  int mult = 1;                          // most points sharing one cell
  const unsigned int *absmax = nullptr;  // max |trace| word (16-bit storage)
  int zlo = 1 << 30, zhi = -1;  // planes holding points
  int *plane_off = nullptr, *cell_head = nullptr, *slot_cell = nullptr,
      *slot_index = nullptr;
  float *traces = nullptr;
  size_t traces_cap = 0;
  std::vector<int> host_locs;  // cells as given, to recognise a repeat upload
  void release() {
    cudaFree(plane_off);
    cudaFree(cell_head);
    cudaFree(slot_cell);
    cudaFree(slot_index);
    cudaFree(traces);
    *this = DevPoints();
  }
};

struct born_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // grid
  bool have_space = false;
  int n1 = 0, n2 = 0, n3 = 0;
  long long n123 = 0;
  float coeffs[13] = {};
  float bound[born::kNBound] = {};
  // sinc tables (rows x 8)
  int jt_s = 0, jt_d = 0;
  std::vector<float> tab_s, tab_d;
  int jt = 1;  // the reference's _jt: last jt given to a time loop
  // device fields
  float *vel1 = nullptr, *vel2 = nullptr;
  float *s0 = nullptr, *s1 = nullptr;  // source levels (p0, p1 of source_prop)
  float *r0 = nullptr, *r1 = nullptr;  // receiver / scattered levels
  float *f0 = nullptr, *f1 = nullptr;  // forward background levels
  float *img = nullptr, *refl = nullptr;
  unsigned int *err_dev = nullptr;
  bool have_vel1 = false, have_vel2 = false, have_refl = false;
  DevPoints src, rec;
  bool src_levels_valid = false;
  // host arrays the last source_prop wrote the levels to (s0 -> host_p0,
  // s1 -> host_p1), the host-level policy of rtm_adjoint and, under
  // BORN_HOST_LEVELS_VERIFY, checksums of the contents written
  const float *host_p0 = nullptr, *host_p1 = nullptr;
  int host_levels = BORN_HOST_LEVELS_RESIDENT;
  bool host_sums_valid = false;
  unsigned long long host_sum0 = 0, host_sum1 = 0;
  int tile_cfg = -1, zseg = 0;
  // step launches overlap the previous step's tail (programmatic dependent
  // launch); born_set_launch_overlap
  bool overlap = true;
  // closing device-to-host copies of a time loop into page-locked host
  // arrays: a first copy into the same array on `side` while the loop runs
  // (born_set_host_prewarm); `prewarm_pending` while the closing copy has
  // not been ordered after it
  bool prewarm = true;
  bool prewarm_pending = false;
  long long prewarm_copies = 0;
  cudaStream_t side = nullptr;
  cudaEvent_t side_go = nullptr, side_done = nullptr;
  // bumped whenever device buffers or point sets are reallocated, so that
  // cached descriptors and graphs built over them can notice
  unsigned long long generation = 0;
  // autotuner: best tile configuration per storage and step mode (-1: not
  // tuned yet)
  bool autotune = true;
  static constexpr int kNS = born::kNumStorages;
  int tuned_cfg[kNS][6] = {{-1, -1, -1, -1, -1, -1},
                           {-1, -1, -1, -1, -1, -1},
                           {-1, -1, -1, -1, -1, -1},
                           {-1, -1, -1, -1, -1, -1},
                           {-1, -1, -1, -1, -1, -1}};
  float tuned_ms[kNS][6] = {};
  // tile choice refined on a time loop's own steps (LoopTuner in
  // born_api.cu), per storage and step mode
  bool loop_tuned[kNS][6] = {};
  // ms per launch of every tile (its best z segmentation) as the last
  // refinement measured it (0: not measured)
  static constexpr int kMaxTileCfgs = 8;
  float loop_ms[kNS][6][kMaxTileCfgs] = {};
  // z segments per column of tiles chosen with the tile (0: the sizing rule
  // of pick_tiling)
  int tuned_nseg[kNS][6] = {};
  // refinement progress, kept across time loops so that loops shorter than
  // the whole candidate sweep continue it: groups timed so far and the best
  // group time (ms, -1 none) of every (tile, z segments) candidate
  static constexpr int kMaxLoopCands = 64, kLoopTop = 8;
  int lt_next[kNS][6] = {};
  float lt_best[kNS][6][kMaxLoopCands];
  // the candidates timed again after the first round (its fastest ones)
  int lt_top[kNS][6][kLoopTop];
  void reset_tuning() {
    for (int st = 0; st < kNS; ++st)
      for (int m = 0; m < 6; ++m) {
        tuned_cfg[st][m] = -1;
        tuned_ms[st][m] = 0.f;
        tuned_nseg[st][m] = 0;
        loop_tuned[st][m] = false;
        lt_next[st][m] = 0;
        for (int c = 0; c < kMaxTileCfgs; ++c) loop_ms[st][m][c] = 0.f;
        for (int c = 0; c < kMaxLoopCands; ++c) lt_best[st][m][c] = -1.f;
      }
  }
  // wavefield level storage (born::Storage) and, for 16-bit storage, the
  // level records [kNumLevelBufs][2 slots][2 words], the number of writes of
  // each level buffer since its last reset (its record slot is the parity)
  // and the maxima words
  int storage = 0;
  unsigned long long *lv_dev = nullptr;
  unsigned int *stat_dev = nullptr;
  int wr[kNumLevelBufs] = {};
  size_t level_bytes() const {
    return (size_t)n123 * born::storage_esize(storage);
  }
  int level_esize() const { return born::storage_esize(storage); }
  bool lp() const { return born::storage_16bit(storage); }
  // storage a step mode runs with (and the slot of its tile choices): the
  // fused FP32 arithmetic covers the source, forward and adjoint steps, the
  // exact Born coupling the forward step; the other modes keep the
  // reference order
  int storage_for(int mode) const {
    if (storage == born::kStoreF32Fused && mode > born::kModeAdjoint)
      return born::kStoreF32;
    if (storage == born::kStoreF32Exact && mode != born::kModeForward)
      return born::kStoreF32;
    return storage;
  }
  long long launches = 0;
  int ntblock = 0;
  // TMA descriptors by (buffer, tile config * 2 + kind); kind 0 = halo box,
  // 1 = centre tile
  std::map<std::pair<const void *, int>, CUtensorMap> maps;
  // exact linearised adjoint: checkpoints (ckpt_bytes allocated; levels of
  // n123 FP32 values, or FP16 values with one power-of-two scale per level
  // in ckpt_scale) and the per-segment A s buffer
  float *ckpt = nullptr, *gbuf = nullptr;
  size_t ckpt_levels = 0, gbuf_levels = 0;
  size_t ckpt_bytes = 0;
  int ckpt_storage = 0;          // BORN_CKPT_F32 or BORN_CKPT_F16
  float *ckpt_scale = nullptr;   // device, one scale per level (FP16)
  size_t ckpt_scale_levels = 0;
  unsigned int *ckpt_maxw = nullptr;  // device word for the level maxima
  // The background s of the exact pair depends only on vel2, the source
  // (points, traces, source sinc table) and the grid: bg_gen counts changes
  // of those, and the checkpoints in ckpt are reusable while (bg_gen, jt,
  // nt, interval) equal ckpt_key.  born_lin_forward stores them every
  // ckpt_every steps (0: never) as it computes the background.
  unsigned long long bg_gen = 1;
  bool ckpt_valid = false;
  unsigned long long ckpt_gen = 0;
  int ckpt_jt = 0, ckpt_nt = 0, ckpt_interval = 0, ckpt_kind = 0;
  int ckpt_every = 50;
  bool ckpt_reused = false;  // the last born_lin_adjoint skipped its sweep
  // phase times (ms) of the last born_lin_adjoint when timing is enabled:
  // forward sweep with checkpoint stores, segment restores and recompute,
  // reverse adjoint steps, final division (born_phase_times)
  bool time_phases = false;
  float phase_ms[4] = {};
};


// Shared helpers (born_api.cu)
born::PointSet born_point_view(const DevPoints &dp, int id, int ii,
                               const std::vector<float> &tab, float scale,
                               bool use);
void born_base_params(born_handle *h, born::StepParams &p);
int born_get_map(born_handle *h, const void *buf, int cfg, int kind,
                 int esize, CUtensorMap *out);
void born_pick_tiling(born_handle *h, int mode, bool pa, bool pb, int *cfg,
                      int *zseg, int *tiles_x, int *tiles_y);
int born_ensure_tuned(born_handle *h, int mode);

// 16-bit storage bookkeeping (born_api.cu).  Record slots of a step that
// reads `cur` (null: not read) and `old` and, when `write`, writes its new
// level over `old`; born_level_written() counts that write afterwards.
int born_level_id(const born_handle *h, const void *buf);
born::LevelRefs born_level_refs(const born_handle *h, const void *cur,
                                const void *old, bool write, unsigned int tag);
void born_level_written(born_handle *h, const void *buf);
// Before a time loop with 16-bit storage: the maxima words (velocities,
// reflectivity, traces) and a reset of the records of the buffers the loop
// clears.  No-op with FP32 storage.
int born_lp_prologue(born_handle *h, cudaStream_t s, const void *const *reset,
                     int nreset);
// dst <- src for a level buffer (data and record).
int born_copy_level(born_handle *h, void *dst, const void *src,
                    unsigned int tag, cudaStream_t s);
// Step parameters that depend on the storage: maxima words of the fields'
// velocities (and the reflectivity for the Born coupling).
void born_set_lp_words(born_handle *h, born::StepParams &p, int mode);

// Error helpers (born_api.cu)
int born_fail(born_handle *h, int code, const char *fmt, ...);
int born_check_ready(born_handle *h);
int born_check_device_error(born_handle *h);
