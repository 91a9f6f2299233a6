// Batched multi-shot time loops: one launch per time step for all shots.
//
// Shots are independent (the reference runs them one after another in its
// operator, rtm_zero_op_3d.cc:137,240, or in separate processes,
// scripts/run.py:51-93).  A batch groups N shot handles that are fully set
// up (each with its own compute grid, which may differ in size, sinc tables,
// points, velocities and traces) and advances all of them together: every
// step is one launch of step_kernel_batched whose CTAs are the CTAs of every
// shot in turn.  Per shot the kernel reads its grid, buffers and TMA
// descriptors (one set per parity of the level rotation) from device memory;
// the step-varying scalars (injection sample, sinc row, scale) are kernel
// arguments shared by all shots, so all shots must use the same time axis
// (nt, jt, trace length).  The time loops follow the single-shot loops in
// born_api.cu step for step, so every shot's results are bit-identical to
// running it alone.  Optionally each whole time loop is recorded once into
// a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "born_internal.h"

using born::BatchShot;
using born::StepVar;

struct BatchTuner;

struct born_batch {
  std::vector<born_handle *> shots;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool use_graph = true;
  std::string err;
  // per (mode, pa, pb, loop kind): device shot table and block prefix
  struct Table {
    BatchShot *d_shots = nullptr;
    int *d_start = nullptr;
    int total = 0, cfg = 0;
  };
  std::map<std::tuple<int, int, int, int, int, int>, Table> tables;
  // tiling of the batched steps per step mode: tile configuration and z
  // segment depth in planes (-1 / 0: the first shot's tuned tile at every
  // shot's sizing rule), refined on the first run of each loop (tuned[m])
  int cur_cfg[6] = {-1, -1, -1, -1, -1, -1}, cur_zseg[6] = {};
  bool tuned[6] = {};
  struct BatchTuner *tuner = nullptr;
  int tuner_k = 0;
  // recorded loops by (loop kind, nt, jt, parities of the source levels'
  // record slots); wr_after: the level write counts the loop leaves behind
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int wr_after[kNumLevelBufs] = {};
    // kernels one replay runs: in the batch and on each shot
    long long kernels = 0;
    std::vector<long long> shot_kernels;
  };
  std::map<std::tuple<int, int, int, int>, Graph> graphs;
  std::vector<unsigned long long> generations;
  long long launches = 0;        // kernels run on the batch stream
  long long graph_launches = 0;  // replays of recorded time loops
};


// In-loop tiling refinement of a batched time loop, the batch's counterpart
// of the single-shot loops' refinement: one tile for every shot's CTAs and
// one z-segment depth in planes for every shot (0: each shot's sizing
// rule).  The first shot's own tuned tile had run the c4 batch (48 shots,
// 600 steps) at 165.8 Gcell-updates/s; 32x16 tiles with 48-plane segments
// ran it at 179.4.  On the first run of a loop the candidates take turns
// from its second step, in groups of one untimed step (which builds the
// candidate's shot table) and kBatchGroup timed steps between CUDA events:
// one group each, then kBatchRounds - 1 rounds over the kBatchTop fastest;
// the loop goes on with the fastest and later runs (recorded graphs) use
// it.  Every tiling gives bit-identical results.
constexpr int kBatchGroup = 4, kBatchRounds = 3, kBatchTop = 6;
constexpr int kBatchZsegs[] = {0, 32, 48, 64, 96};

struct BatchTuner {
  born_batch *b;
  int mode;
  std::vector<std::pair<int, int>> cand;  // (tile configuration, planes)
  std::vector<float> best;                // best group time, -1 none
  std::vector<int> top;
  std::vector<cudaEvent_t> ev;
  int ntop = 0, total = 0, folded = 0;
  bool on = false;

  BatchTuner(born_batch *b_, int mode_, int nsteps) : b(b_), mode(mode_) {
    for (int c = 0; c < born::tile_cfg_count(); ++c)
      for (int z : kBatchZsegs) cand.push_back({c, z});
    best.assign(cand.size(), -1.f);
    ntop = std::min((int)cand.size(), kBatchTop);
    total = (int)cand.size() + ntop * (kBatchRounds - 1);
    if ((nsteps - 2) / (kBatchGroup + 1) < total) return;  // keep the default
    ev.assign(2 * total, nullptr);
    for (cudaEvent_t &e : ev)
      if (cudaEventCreate(&e) != cudaSuccess) {
        release();
        return;
      }
    on = true;
  }
  ~BatchTuner() { release(); }
  BatchTuner(const BatchTuner &) = delete;
  BatchTuner &operator=(const BatchTuner &) = delete;

  void release() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    ev.clear();
    on = false;
  }
  int cand_of(int g) const {
    const int n = (int)cand.size();
    return g < n ? g : top[(g - n) % ntop];
  }
  void use(int i) {
    b->cur_cfg[mode] = cand[i].first;
    b->cur_zseg[mode] = cand[i].second;
  }
  cudaError_t fold(int upto) {
    if (upto <= folded) return cudaSuccess;
    cudaError_t e = cudaEventSynchronize(ev[2 * upto - 1]);
    for (int i = folded; i < upto && e == cudaSuccess; ++i) {
      float ms = 0.f;
      e = cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
      float &t = best[cand_of(i)];
      if (e == cudaSuccess && (t < 0.f || ms < t)) t = ms;
    }
    folded = upto;
    return e;
  }
  // before launching the loop's step k (k = 0 for its first step)
  cudaError_t before(int k) {
    if (!on || k < 1) return cudaSuccess;
    const int g = (k - 1) / (kBatchGroup + 1), r = (k - 1) % (kBatchGroup + 1);
    if (r == 1 && g < total) return cudaEventRecord(ev[2 * g], b->stream);
    if (r != 0) return cudaSuccess;
    if (g > 0) {
      cudaError_t e = cudaEventRecord(ev[2 * g - 1], b->stream);
      if (e != cudaSuccess) return e;
    }
    if (g < total) {
      if (g == (int)cand.size()) {  // first round done: keep its fastest
        cudaError_t e = fold(g);
        if (e != cudaSuccess) return e;
        std::vector<int> order(cand.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
          const float tx = best[x] < 0.f ? 3e38f : best[x];
          const float ty = best[y] < 0.f ? 3e38f : best[y];
          return tx < ty;
        });
        top.assign(order.begin(), order.begin() + ntop);
      }
      use(cand_of(g));
      return cudaSuccess;
    }
    return finish();
  }
  cudaError_t finish() {
    if (!on) return cudaSuccess;
    cudaError_t e = fold(total);
    int pick = -1;
    for (size_t i = 0; i < cand.size(); ++i)
      if (best[i] >= 0.f && (pick < 0 || best[i] < best[pick])) pick = (int)i;
    if (pick >= 0) use(pick);
    release();
    return e;
  }
};

namespace {

enum LoopKind { kLoopSource = 0, kLoopAdjoint = 1, kLoopForward = 2 };

int bfail(born_batch *b, int code, const char *msg) {
  b->err = msg;
  return code;
}

void drop_cache(born_batch *b) {
  for (auto &kv : b->tables) {
    cudaFree(kv.second.d_shots);
    cudaFree(kv.second.d_start);
  }
  b->tables.clear();
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second.exec);
  b->graphs.clear();
  for (int m = 0; m < 6; ++m) {  // tilings depend on the shots' grids
    b->cur_cfg[m] = -1;
    b->cur_zseg[m] = 0;
    b->tuned[m] = false;
  }
}

bool stale(born_batch *b) {
  for (size_t i = 0; i < b->shots.size(); ++i)
    if (b->shots[i]->generation != b->generations[i]) return true;
  return false;
}

// The buffers of one shot for a loop kind and parity (the level rotation of
// the single-shot loops in born_api.cu).
struct Levels {
  float *a_cur, *a_out, *b_cur, *b_out;
  const void *cen[born::kNumCentre];
};

Levels levels_for(born_handle *h, int kind, int parity) {
  Levels L{};
  if (kind == kLoopSource) {  // p0 <- f(p1, p0); rotation starts (s0, s1)
    float *p0 = parity ? h->s1 : h->s0, *p1 = parity ? h->s0 : h->s1;
    L.a_cur = p1;
    L.a_out = p0;
    const void *c[born::kNumCentre] = {p0, nullptr, h->vel1, nullptr,
                                        nullptr};
    std::memcpy(L.cen, c, sizeof(c));
  } else if (kind == kLoopAdjoint) {  // swap = 1 convention
    float *sp0 = parity ? h->s0 : h->s1, *sp1 = parity ? h->s1 : h->s0;
    float *rp0 = parity ? h->r1 : h->r0, *rp1 = parity ? h->r0 : h->r1;
    L.a_cur = rp1;
    L.a_out = rp0;
    L.b_cur = sp1;
    L.b_out = sp0;
    const void *c[born::kNumCentre] = {rp0, sp0, h->vel2, h->vel1, h->img};
    std::memcpy(L.cen, c, sizeof(c));
  } else {
    float *sp0 = parity ? h->f1 : h->f0, *sp1 = parity ? h->f0 : h->f1;
    float *rp0 = parity ? h->r1 : h->r0, *rp1 = parity ? h->r0 : h->r1;
    L.a_cur = sp1;
    L.a_out = sp0;
    L.b_cur = rp1;
    L.b_out = rp0;
    const void *c[born::kNumCentre] = {sp0, rp0, h->vel2, nullptr, h->refl};
    std::memcpy(L.cen, c, sizeof(c));
  }
  return L;
}

int build_table(born_batch *b, int mode, bool pa, bool pb, int kind,
                born_batch::Table **out) {
  const int want_cfg = b->cur_cfg[mode], want_zseg = b->cur_zseg[mode];
  auto key = std::make_tuple(mode, (int)pa, (int)pb, kind, want_cfg, want_zseg);
  auto it = b->tables.find(key);
  if (it != b->tables.end()) {
    *out = &it->second;
    return BORN_OK;
  }
  born_handle *h0 = b->shots[0];
  int cfg0 = want_cfg;
  if (cfg0 < 0) {
    int rc = born_ensure_tuned(h0, mode);
    if (rc) return bfail(b, rc, "autotune failed");
    int zs, tx, ty;
    born_pick_tiling(h0, mode, pa, pb, &cfg0, &zs, &tx, &ty);
  }
  int rc = BORN_OK;
  std::vector<BatchShot> host(b->shots.size());
  std::vector<int> start(b->shots.size() + 1, 0);
  for (size_t s = 0; s < b->shots.size(); ++s) {
    born_handle *h = b->shots[s];
    const int saved = h->tile_cfg, saved_zseg = h->zseg;
    h->tile_cfg = cfg0;  // one tile shape for the whole launch
    if (want_zseg > 0) h->zseg = want_zseg;
    int cfg, zseg, tiles_x, tiles_y;
    born_pick_tiling(h, mode, pa, pb, &cfg, &zseg, &tiles_x, &tiles_y);
    h->tile_cfg = saved;
    h->zseg = saved_zseg;
    BatchShot &bs = host[s];
    std::memset(&bs, 0, sizeof(bs));
    born_base_params(h, bs.params);
    born_set_lp_words(h, bs.params, mode);
    bs.params.tiles_x = tiles_x;
    bs.params.tiles_y = tiles_y;
    bs.params.zseg = zseg;
    bs.params.img_out = kind == kLoopAdjoint ? h->img : nullptr;
    const DevPoints &pa_set = kind == kLoopAdjoint ? h->rec : h->src;
    const DevPoints &pb_set = kind == kLoopForward ? h->rec : h->src;
    const std::vector<float> none;
    bs.params.pa = born_point_view(pa_set, 0, 0, none, 0.f, false);
    bs.params.pb = born_point_view(pb_set, 0, 0, none, 0.f, false);
    for (int par = 0; par < 2; ++par) {
      Levels L = levels_for(h, kind, par);
      bs.a_out[par] = L.a_out;
      bs.b_out[par] = L.b_out;
      born::StepMaps &m = bs.maps[par];
      const int fe = h->level_esize();
      const void *any = h->vel2, *anyf = fe == 4 ? any : (const void *)h->f0;
      rc = born_get_map(h, L.a_cur ? L.a_cur : anyf, cfg, 0, fe, &m.box_a);
      if (!rc)
        rc = born_get_map(h, L.b_cur ? L.b_cur : anyf, cfg, 0, fe, &m.box_b);
      if (!rc)
        rc = born_get_map(h, L.a_cur ? L.a_cur : anyf, cfg, 1, fe, &m.zc_a);
      if (!rc)
        rc = born_get_map(h, L.b_cur ? L.b_cur : anyf, cfg, 1, fe, &m.zc_b);
      for (int sl = 0; sl < born::kNumCentre && !rc; ++sl) {
        const int es = born::field_slot(mode, sl) ? fe : 4;
        const void *fb = es == 4 ? any : anyf;
        rc = born_get_map(h, L.cen[sl] ? L.cen[sl] : fb, cfg, 1, es,
                          &m.cm[sl]);
      }
      if (rc) return bfail(b, rc, "tensor map creation failed");
    }
    const int nseg = (h->n3 - 8 + zseg - 1) / zseg;
    start[s + 1] = start[s] + tiles_x * tiles_y * nseg;
  }
  born_batch::Table t;
  t.total = start.back();
  t.cfg = cfg0;
  if (cudaMalloc(&t.d_shots, host.size() * sizeof(BatchShot)) != cudaSuccess ||
      cudaMalloc(&t.d_start, start.size() * sizeof(int)) != cudaSuccess ||
      cudaMemcpy(t.d_shots, host.data(), host.size() * sizeof(BatchShot),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(t.d_start, start.data(), start.size() * sizeof(int),
                 cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(t.d_shots);
    cudaFree(t.d_start);
    return bfail(b, BORN_ENOMEM, "batch table allocation failed");
  }
  auto ins = b->tables.emplace(key, t);
  *out = &ins.first->second;
  return BORN_OK;
}

StepVar make_var(int parity, const born::PointSet &pa,
                 const born::PointSet &pb) {
  StepVar v;
  std::memset(&v, 0, sizeof(v));
  v.parity = parity;
  v.pa_id = pa.id;
  v.pa_active = pa.active;
  v.pa_scale = pa.scale;
  v.pb_id = pb.id;
  v.pb_active = pb.active;
  v.pb_scale = pb.scale;
  for (int k = 0; k < 8; ++k) {
    v.pa_tab[k] = pa.tab[k];
    v.pb_tab[k] = pb.tab[k];
  }
  return v;
}

// Tables and kernel attributes for a step variant, before any recording.
int prepare(born_batch *b, int mode, bool pa, bool pb, int kind) {
  born_batch::Table *t = nullptr;
  int rc = build_table(b, mode, pa, pb, kind, &t);
  if (rc) return rc;
  StepVar none;
  std::memset(&none, 0, sizeof(none));
  cudaError_t e = born::launch_step_batched(
      b->shots[0]->storage, mode, pa, pb, t->cfg, t->d_shots, t->d_start,
      (int)b->shots.size(), 0, none, b->stream);
  return e == cudaSuccess ? BORN_OK
                          : bfail(b, BORN_ECUDA, cudaGetErrorString(e));
}

// One batched step.  The level records follow shot 0's bookkeeping (every
// shot has the same rotation); afterwards every shot counts the writes of
// its own buffers (write_a / write_b: the step writes field A / B).
int launch_batched(born_batch *b, int mode, bool pa, bool pb, int kind,
                   StepVar var, bool write_a, bool write_b) {
  if (b->tuner && b->tuner->mode == mode &&
      b->tuner->before(b->tuner_k++) != cudaSuccess)
    return bfail(b, BORN_ECUDA, "batch tiling refinement failed");
  born_batch::Table *t = nullptr;
  int rc = build_table(b, mode, pa, pb, kind, &t);
  if (rc) return rc;
  born_handle *h0 = b->shots[0];
  const Levels L0 = levels_for(h0, kind, var.parity);
  const unsigned int tag = var.la.tag;
  var.la = born_level_refs(h0, pa ? L0.a_cur : nullptr, L0.a_out, write_a,
                           tag);
  var.lb = born_level_refs(h0, pb ? L0.b_cur : nullptr, L0.b_out, write_b,
                           tag + 1u);
  cudaError_t e = born::launch_step_batched(
      h0->storage, mode, pa, pb, t->cfg, t->d_shots, t->d_start,
      (int)b->shots.size(), t->total, var, b->stream);
  if (e != cudaSuccess) return bfail(b, BORN_ECUDA, cudaGetErrorString(e));
  b->launches++;
  for (born_handle *h : b->shots) {
    h->launches++;
    const Levels L = levels_for(h, kind, var.parity);
    if (write_a) born_level_written(h, L.a_out);
    if (write_b) born_level_written(h, L.b_out);
  }
  return BORN_OK;
}

// Every shot must share the time axis the step scalars describe.
int check_shared_axis(born_batch *b, bool need_rec) {
  born_handle *h0 = b->shots[0];
  for (born_handle *h : b->shots) {
    if (!h->have_space || !h->have_vel1 || !h->have_vel2)
      return bfail(b, BORN_ESTATE, "a shot is not fully set up");
    if (h->jt_s != h0->jt_s || h->jt_d != h0->jt_d ||
        h->tab_s != h0->tab_s || h->tab_d != h0->tab_d ||
        h->src.nt != h0->src.nt || (need_rec && h->rec.nt != h0->rec.nt) ||
        std::memcmp(h->coeffs, h0->coeffs, sizeof(h->coeffs)) != 0)
      return bfail(b, BORN_EINVAL,
                   "shots differ in sinc tables, trace length or spacing");
    if (h->storage != h0->storage)
      return bfail(b, BORN_EINVAL, "shots differ in level storage");
    if (std::memcmp(h->wr, h0->wr, sizeof(h->wr)) != 0)
      return bfail(b, BORN_ESTATE,
                   "shots' levels are out of step (run their loops together)");
  }
  return BORN_OK;
}

// Records (or replays) the loop body.  body(b) enqueues the whole loop on
// b->stream; with graphs on it is captured once per (kind, nt, jt).
// The batch waits for work already queued on the shots' own streams
// (transfers, clears), outside any recording.
int order_from_shots(born_batch *b) {
  for (born_handle *h : b->shots) {
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
      return bfail(b, BORN_ECUDA, "event creation failed");
    cudaError_t e = cudaEventRecord(ev, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, ev, 0);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return bfail(b, BORN_ECUDA, "ordering failed");
  }
  return BORN_OK;
}

template <class F>
int run_loop(born_batch *b, int kind, int nt, int jt, F body) {
  int orc = order_from_shots(b);
  if (orc) return orc;
  if (stale(b)) {
    drop_cache(b);
    for (size_t i = 0; i < b->shots.size(); ++i)
      b->generations[i] = b->shots[i]->generation;
  }
  // the first run of a loop refines its tiling on its own steps, uncaptured
  // (tables for every candidate are built on the way); later runs record
  // and replay it with the chosen tiling
  const int mode = kind == kLoopSource    ? born::kModeSource
                   : kind == kLoopAdjoint ? born::kModeAdjoint
                                          : born::kModeForward;
  if (!b->tuned[mode]) {
    b->tuned[mode] = true;
    born_handle *s0 = b->shots[0];
    if (s0->autotune && s0->tile_cfg < 0 && s0->zseg == 0) {
      BatchTuner t(b, mode, kind == kLoopSource ? nt + 1 : nt);
      if (t.on) {
        b->tuner = &t;
        b->tuner_k = 0;
        int rc = body(b);
        b->tuner = nullptr;
        if (rc) return rc;
        if (t.finish() != cudaSuccess)
          return bfail(b, BORN_ECUDA, "batch tiling refinement failed");
        return BORN_OK;
      }
    }
  }
  if (!b->use_graph) return body(b);
  born_handle *h0 = b->shots[0];
  auto key = std::make_tuple(kind, nt, jt,
                             (h0->wr[kBufS0] & 1) | ((h0->wr[kBufS1] & 1) << 1));
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    // tables, tuning and kernel attributes first: none of that may happen
    // while the stream is capturing
    int rc = body(nullptr);
    if (rc) return rc;
    cudaGraph_t g = nullptr;
    // recording runs no kernel: the counters advance on each replay instead
    const long long k0 = b->launches;
    std::vector<long long> s0;
    for (born_handle *h : b->shots) s0.push_back(h->launches);
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess)
      return bfail(b, BORN_ECUDA, "stream capture failed to begin");
    rc = body(b);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    const long long kernels = b->launches - k0;
    b->launches = k0;
    std::vector<long long> sk;
    for (size_t i = 0; i < b->shots.size(); ++i) {
      sk.push_back(b->shots[i]->launches - s0[i]);
      b->shots[i]->launches = s0[i];
    }
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return bfail(b, BORN_ECUDA, "stream capture failed");
    born_batch::Graph gr;
    e = cudaGraphInstantiate(&gr.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      return bfail(b, BORN_ECUDA, "graph instantiation failed");
    // recording ran the loop's bookkeeping once; a replay repeats its effect
    std::memcpy(gr.wr_after, h0->wr, sizeof(gr.wr_after));
    gr.kernels = kernels;
    gr.shot_kernels = sk;
    it = b->graphs.emplace(key, gr).first;
  }
  if (cudaGraphLaunch(it->second.exec, b->stream) != cudaSuccess)
    return bfail(b, BORN_ECUDA, "graph launch failed");
  for (size_t i = 0; i < b->shots.size(); ++i) {
    std::memcpy(b->shots[i]->wr, it->second.wr_after, sizeof(b->shots[i]->wr));
    b->shots[i]->launches += it->second.shot_kernels[i];
  }
  b->launches += it->second.kernels;
  b->graph_launches++;
  return BORN_OK;
}

// Work later queued on a shot's own stream (result copies, transfers) waits
// for the batch.
int order_shot_streams(born_batch *b) {
  cudaEvent_t ev;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
    return bfail(b, BORN_ECUDA, "event creation failed");
  cudaError_t e = cudaEventRecord(ev, b->stream);
  for (born_handle *h : b->shots)
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, ev, 0);
  cudaEventDestroy(ev);
  return e == cudaSuccess ? BORN_OK : bfail(b, BORN_ECUDA, "ordering failed");
}

}  // namespace

extern "C" {

int born_batch_create(born_handle *const *shots, int nshots,
                      born_batch **out) {
  if (!shots || nshots < 1 || !out) return BORN_EINVAL;
  *out = nullptr;
  for (int i = 0; i < nshots; ++i)
    if (!shots[i] || shots[i]->device != shots[0]->device) return BORN_EINVAL;
  born_batch *b = new born_batch();
  b->shots.assign(shots, shots + nshots);
  b->generations.assign(nshots, ~0ull);
  b->device = shots[0]->device;
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) !=
          cudaSuccess) {
    delete b;
    return BORN_ECUDA;
  }
  *out = b;
  return BORN_OK;
}

int born_batch_destroy(born_batch *b) {
  if (!b) return BORN_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  drop_cache(b);
  cudaStreamDestroy(b->stream);
  delete b;
  return BORN_OK;
}

const char *born_batch_error(const born_batch *b) {
  return b ? b->err.c_str() : "null batch";
}

int born_batch_set_graph(born_batch *b, int use_graph) {
  if (!b) return BORN_EINVAL;
  b->use_graph = use_graph != 0;
  return BORN_OK;
}

void *born_batch_stream(born_batch *b) { return b ? (void *)b->stream : nullptr; }

long long born_batch_launches(const born_batch *b) {
  return b ? b->launches : 0;
}

long long born_batch_graph_launches(const born_batch *b) {
  return b ? b->graph_launches : 0;
}

// cpuProp::sourceProp for every shot (cpu_prop.cc:106-129)
int born_batch_source_prop(born_batch *b, int jts, int nt) {
  if (!b) return BORN_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return BORN_ECUDA;
  if (nt < 0 || jts < 1) return bfail(b, BORN_EINVAL, "nt < 0 or jts < 1");
  int rc = check_shared_axis(b, false);
  if (rc) return rc;
  born_handle *h0 = b->shots[0];
  rc = run_loop(b, kLoopSource, nt, jts, [&](born_batch *rec) -> int {
    if (!rec)  // preparation pass: tables and kernel attributes
      return prepare(b, born::kModeSource, true, false, kLoopSource);
    for (born_handle *h : b->shots) {
      const size_t bytes = h->level_bytes();
      if (cudaMemsetAsync(h->s0, 0, bytes, b->stream) != cudaSuccess ||
          cudaMemsetAsync(h->s1, 0, bytes, b->stream) != cudaSuccess)
        return bfail(b, BORN_ECUDA, "memset failed");
      const void *reset[] = {h->s0, h->s1};
      if (born_lp_prologue(h, b->stream, reset, 2))
        return bfail(b, BORN_ECUDA, h->err.c_str());
    }
    const float scale = 1 / (float)jts;
    const std::vector<float> none;
    for (int it = 0; it <= nt; ++it) {
      const int id = it / h0->jt_s, ii = it - id * h0->jt_s;
      born::PointSet pa = born_point_view(h0->src, id, ii, h0->tab_s, scale,
                                          true);
      born::PointSet pb = born_point_view(h0->src, 0, 0, none, 0.f, false);
      StepVar var = make_var(it & 1, pa, pb);
      var.la.tag = kTagSource + (unsigned int)it;
      int r = launch_batched(b, born::kModeSource, true, false, kLoopSource,
                             var, true, false);
      if (r) return r;
    }
    if (nt % 2 == 1)  // after nt+1 rotations (p0, p1) = (s0, s1): p1 <- p0
      for (born_handle *h : b->shots)
        if (born_copy_level(h, h->s1, h->s0, kTagSource + nt + 1, b->stream))
          return bfail(b, BORN_ECUDA, h->err.c_str());
    return BORN_OK;
  });
  if (!rc) rc = order_shot_streams(b);
  if (rc) return rc;
  for (born_handle *h : b->shots) {
    h->jt = jts;
    h->src_levels_valid = true;
  }
  return BORN_OK;
}

// cpuProp::rtmAdjoint for every shot (cpu_prop.cc:56-96), with the source
// levels in the order rtm_zero_op passes them (swap = 1)
int born_batch_rtm_adjoint(born_batch *b, int jtd, int nt) {
  (void)jtd;
  if (!b) return BORN_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return BORN_ECUDA;
  if (nt < 1) return bfail(b, BORN_EINVAL, "nt < 1");
  int rc = check_shared_axis(b, true);
  if (rc) return rc;
  for (born_handle *h : b->shots)
    if (!h->src_levels_valid || h->jt != b->shots[0]->jt)
      return bfail(b, BORN_ESTATE, "source levels missing (run source_prop)");
  born_handle *h0 = b->shots[0];
  rc = run_loop(b, kLoopAdjoint, nt, h0->jt, [&](born_batch *rec) -> int {
    if (!rec) {
      const bool v[4][2] = {{1, 1}, {1, 0}, {0, 1}, {0, 0}};
      for (auto &pv : v) {
        int r = prepare(b, born::kModeAdjoint, pv[0], pv[1], kLoopAdjoint);
        if (r) return r;
      }
      return BORN_OK;
    }
    for (born_handle *h : b->shots) {
      const size_t lbytes = h->level_bytes();
      if (cudaMemsetAsync(h->r0, 0, lbytes, b->stream) != cudaSuccess ||
          cudaMemsetAsync(h->r1, 0, lbytes, b->stream) != cudaSuccess ||
          cudaMemsetAsync(h->img, 0, (size_t)h->n123 * 4, b->stream) !=
              cudaSuccess)
        return bfail(b, BORN_ECUDA, "memset failed");
      const void *reset[] = {h->r0, h->r1};
      if (born_lp_prologue(h, b->stream, reset, 2))
        return bfail(b, BORN_ECUDA, h->err.c_str());
    }
    const float scale = -1 / (float)h0->jt;
    const std::vector<float> none;
    born::PointSet pending = born_point_view(h0->src, 0, 0, none, 0.f, false);
    for (int it = nt - 1; it >= 0; --it) {
      const int id_s = (it + 1) / h0->jt_s, i_s = it + 1 - id_s * h0->jt_s;
      const int id = it / h0->jt_d, ii = it - id * h0->jt_d;
      const bool pa = it > 0, pb = it < nt - 1;
      born::PointSet ra = born_point_view(h0->rec, id, ii, h0->tab_d, scale,
                                          true);
      StepVar var = make_var((nt - 1 - it) & 1, ra, pending);
      var.la.tag = kTagAdjoint + 2u * (unsigned int)(nt - 1 - it);
      int r = launch_batched(b, born::kModeAdjoint, pa, pb, kLoopAdjoint,
                             var, true, pb);
      if (r) return r;
      pending = born_point_view(h0->src, id_s, i_s, h0->tab_s, scale, pb);
    }
    if (pending.active)  // final source injection, as the single-shot loop
      for (born_handle *h : b->shots) {
        born::PointSet ps = born_point_view(h->src, pending.id, 0, none,
                                            pending.scale, false);
        ps.active = 1;
        for (int k = 0; k < 8; ++k) ps.tab[k] = pending.tab[k];
        float *sp0 = ((nt & 1) == 0) ? h->s1 : h->s0;
        const int id = born_level_id(h, sp0);
        if (born::launch_point_inject(ps, h->src.npts, sp0, h->storage,
                                      h->lv_dev, 2 * id + (h->wr[id] & 1),
                                      b->stream) != cudaSuccess)
          return bfail(b, BORN_ECUDA, "inject failed");
        h->launches++;
      }
    return BORN_OK;
  });
  return rc ? rc : order_shot_streams(b);
}

// cpuProp::rtmForward for every shot (cpu_prop.cc:22-54)
int born_batch_rtm_forward(born_batch *b, int jt, int nt) {
  if (!b) return BORN_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return BORN_ECUDA;
  if (nt < 0 || jt < 1) return bfail(b, BORN_EINVAL, "nt < 0 or jt < 1");
  int rc = check_shared_axis(b, true);
  if (rc) return rc;
  born_handle *h0 = b->shots[0];
  for (born_handle *h : b->shots)
    if (!h->have_refl || jt > h->jt_s || jt > h->jt_d)
      return bfail(b, BORN_ESTATE, "reflectivity missing or jt too large");
  rc = run_loop(b, kLoopForward, nt, jt, [&](born_batch *rec) -> int {
    if (!rec)
      return prepare(b, born::kModeForward, true, true, kLoopForward);
    for (born_handle *h : b->shots) {
      const size_t bytes = h->level_bytes();
      float *bufs[] = {h->f0, h->f1, h->r0, h->r1};
      for (float *p : bufs)
        if (cudaMemsetAsync(p, 0, bytes, b->stream) != cudaSuccess)
          return bfail(b, BORN_ECUDA, "memset failed");
      const void *reset[] = {h->f0, h->f1, h->r0, h->r1};
      if (born_lp_prologue(h, b->stream, reset, 4))
        return bfail(b, BORN_ECUDA, h->err.c_str());
    }
    const float scale = 1 / (float)jt;
    for (int it = 0; it < nt; ++it) {
      const int id = it / jt, ii = it - id * jt;
      born::PointSet pa = born_point_view(h0->src, id, ii, h0->tab_s, scale,
                                          true);
      born::PointSet pb = born_point_view(h0->rec, id, ii, h0->tab_d, 0.f,
                                          true);
      StepVar var = make_var(it & 1, pa, pb);
      var.la.tag = kTagForward + 2u * (unsigned int)it;
      int r = launch_batched(b, born::kModeForward, true, true, kLoopForward,
                             var, true, true);
      if (r) return r;
    }
    return BORN_OK;
  });
  if (!rc)
    for (born_handle *h : b->shots) h->jt = jt;
  return rc ? rc : order_shot_streams(b);
}

int born_batch_synchronize(born_batch *b) {
  if (!b) return BORN_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return bfail(b, BORN_ECUDA, "batch stream failed");
  for (born_handle *h : b->shots) {
    int rc = born_check_device_error(h);
    if (rc) return bfail(b, rc, h->err.c_str());
  }
  return BORN_OK;
}

}  // extern "C"
