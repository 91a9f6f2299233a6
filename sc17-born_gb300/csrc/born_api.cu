// C ABI of the Born / RTM propagator (include/born_gb300.h).
//
// Host side of the hot path: per-handle device state, host->device
// transfers, point maps for injection/extraction, TMA descriptors and the
// three time loops.  The loops mirror the reference CPU propagator's pointer
// rotation step for step (base/cpu_prop.cc:22-129) so that every kernel sees
// the same levels the reference would; the arithmetic itself is in
// born_step_impl.cuh.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "born_internal.h"

using born::kModeAdjoint;
using born::kModeForward;
using born::kModeSource;
using born::PointSet;
using born::StepParams;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                  void *, const cuuint64_t *, const cuuint64_t *,
                                  const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

}  // namespace

namespace {

int fail(born_handle *h, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  return code;
}

#define CK(h, call)                                                          \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return fail(h, e_ == cudaErrorMemoryAllocation ? BORN_ENOMEM           \
                                                     : BORN_ECUDA,           \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                 \
  } while (0)

void free_fields(born_handle *h) {
  float **bufs[] = {&h->vel1, &h->vel2, &h->s0, &h->s1, &h->r0,
                    &h->r1,   &h->f0,   &h->f1, &h->img, &h->refl};
  for (float **b : bufs) {
    cudaFree(*b);
    *b = nullptr;
  }
  cudaFree(h->ckpt);
  cudaFree(h->gbuf);
  cudaFree(h->ckpt_scale);
  cudaFree(h->ckpt_maxw);
  h->ckpt = h->gbuf = nullptr;
  h->ckpt_scale = nullptr;
  h->ckpt_maxw = nullptr;
  h->ckpt_levels = h->gbuf_levels = h->ckpt_bytes = h->ckpt_scale_levels = 0;
  h->ckpt_valid = false;
  h->maps.clear();
  h->have_space = h->have_vel1 = h->have_vel2 = h->have_refl = false;
  h->src_levels_valid = false;
}

int set_device(born_handle *h) {
  CK(h, cudaSetDevice(h->device));
  return BORN_OK;
}

// Coefficients of cpuProp::createSpace (cpu_prop.cc:314-326): formed in
// double, stored as float.  Slot 1/4/7/10 use d1, 2/5/8/11 d2, 3/6/9/12 d3.
void make_coeffs(float *c, float d1, float d2, float d3) {
  auto c00 = [](float d) { return 8.0 / (5.0 * (double)d * (double)d); };
  c[0] = (float)(-1025.0 / 576.0 * (c00(d1) + c00(d2) + c00(d3)));
  const double div[4] = {1.0, -8.0, 63.0, -896.0};
  const float ds[3] = {d1, d2, d3};
  for (int o = 0; o < 4; ++o)
    for (int a = 0; a < 3; ++a) c[1 + 3 * o + a] = (float)(c00(ds[a]) / div[o]);
}

// Taper of cpu_prop.cc:329-332: b[i] = expf(-0.0005f (40 - i)), fixed table.
void make_bound(float *b) {
  const float bcb = .0005f, bca = 40.f;
  for (int i = 0; i < born::kNBound; ++i) b[i] = expf(-bcb * (bca - i));
}

bool interior(const born_handle *h, long long loc) {
  if (loc < 0 || loc >= h->n123) return false;
  const long long n12 = (long long)h->n1 * h->n2;
  const int z = (int)(loc / n12), y = (int)((loc % n12) / h->n1),
            x = (int)(loc % h->n1);
  return x >= 4 && x < h->n1 - 4 && y >= 4 && y < h->n2 - 4 && z >= 4 &&
         z < h->n3 - 4;
}

// Builds the sorted slot list and per-plane head maps of a point set.
int upload_points(born_handle *h, DevPoints &dp, int npts, int nt,
                  const int *locs, const float *traces) {
  if (npts < 0 || nt < 0 || (npts > 0 && (!locs || !traces)))
    return fail(h, BORN_EINVAL, "bad point set (npts=%d nt=%d)", npts, nt);
  for (int i = 0; i < npts; ++i)
    if (!interior(h, locs[i]))
      return fail(h, BORN_EINVAL,
                  "point %d at cell %d is outside the interior [4, n-4)", i,
                  locs[i]);
  const size_t tbytes = (size_t)npts * nt * sizeof(float);
  if (dp.plane_off && dp.npts == npts && dp.nt == nt &&
      std::equal(dp.host_locs.begin(), dp.host_locs.end(), locs)) {
    // same points and trace length (the next shot's data over the same
    // geometry): only the trace values change, so the buffers, descriptors
    // and recorded graphs that use them stay valid
    int rc = set_device(h);
    if (rc) return rc;
    if (tbytes)
      CK(h, cudaMemcpyAsync(dp.traces, traces, tbytes, cudaMemcpyHostToDevice,
                            h->stream));
    return BORN_OK;
  }
  std::vector<int> order(npts);
  for (int i = 0; i < npts; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return locs[a] < locs[b]; });
  const long long n12 = (long long)h->n1 * h->n2;
  std::vector<int> plane_off(h->n3, -1), slot_cell(npts), slot_index(npts);
  std::vector<int> planes;
  for (int s = 0; s < npts; ++s) {
    slot_cell[s] = locs[order[s]];
    slot_index[s] = order[s];
    const int z = (int)(slot_cell[s] / n12);
    if (plane_off[z] < 0) {
      plane_off[z] = (int)(planes.size() * n12);
      planes.push_back(z);
    }
  }
  if ((long long)planes.size() * n12 >= (1ll << 31))
    return fail(h, BORN_EINVAL, "points span too many planes");
  std::vector<int> head(std::max<size_t>(1, planes.size() * n12), -1);
  int mult = 1;
  for (int s = 1, run = 1; s < npts; ++s) {
    run = slot_cell[s] == slot_cell[s - 1] ? run + 1 : 1;
    mult = std::max(mult, run);
  }
  for (int s = npts - 1; s >= 0; --s) {
    const int z = (int)(slot_cell[s] / n12);
    head[plane_off[z] + (slot_cell[s] % n12)] = s;
  }
  int rc = set_device(h);
  if (rc) return rc;
  cudaStreamSynchronize(h->stream);
  DevPoints nd;
  nd.npts = npts;
  nd.nt = nt;
  nd.host_locs.assign(locs, locs + npts);
  nd.mult = mult;
  nd.absmax = h->stat_dev + (&dp == &h->src ? kStatSrc : kStatRec);
  for (int z : planes) {
    nd.zlo = std::min(nd.zlo, z);
    nd.zhi = std::max(nd.zhi, z);
  }
  CK(h, cudaMalloc(&nd.plane_off, sizeof(int) * h->n3));
  CK(h, cudaMalloc(&nd.cell_head, sizeof(int) * head.size()));
  CK(h, cudaMalloc(&nd.slot_cell, sizeof(int) * std::max(1, npts)));
  CK(h, cudaMalloc(&nd.slot_index, sizeof(int) * std::max(1, npts)));
  CK(h, cudaMalloc(&nd.traces, std::max<size_t>(4, tbytes)));
  nd.traces_cap = tbytes;
  CK(h, cudaMemcpy(nd.plane_off, plane_off.data(), sizeof(int) * h->n3,
                   cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(nd.cell_head, head.data(), sizeof(int) * head.size(),
                   cudaMemcpyHostToDevice));
  if (npts) {
    CK(h, cudaMemcpy(nd.slot_cell, slot_cell.data(), sizeof(int) * npts,
                     cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(nd.slot_index, slot_index.data(), sizeof(int) * npts,
                     cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(nd.traces, traces, tbytes, cudaMemcpyHostToDevice));
  }
  dp.release();
  dp = nd;
  h->generation++;
  return BORN_OK;
}

// TMA descriptor of a grid buffer: kind 0 = halo box (TX+8) x (TY+8),
// kind 1 = centre tile (TX x TY for FP32, (TX+8) x TY for 16-bit elements,
// whose copies must start at x multiples of 8).
int get_map(born_handle *h, const void *buf, int cfg, int kind, int esize,
            CUtensorMap *out) {
  auto key = std::make_pair(buf, (cfg * 2 + kind) * 8 + esize);
  auto it = h->maps.find(key);
  if (it != h->maps.end()) {
    *out = it->second;
    return BORN_OK;
  }
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(h, BORN_ECUDA, "cuTensorMapEncodeTiled unavailable");
  int tx, ty;
  born::tile_cfg_dims(cfg, &tx, &ty);
  CUtensorMap m;
  const cuuint64_t dims[3] = {(cuuint64_t)h->n1, (cuuint64_t)h->n2,
                              (cuuint64_t)h->n3};
  const cuuint64_t strides[2] = {(cuuint64_t)h->n1 * esize,
                                 (cuuint64_t)h->n1 * h->n2 * esize};
  const int halo = kind == 0 ? 2 * born::kRadius : 0;
  const int xhalo = (kind == 0 || esize == 2) ? 2 * born::kRadius : 0;
  const cuuint32_t box[3] = {(cuuint32_t)(tx + xhalo), (cuuint32_t)(ty + halo),
                             1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&m,
                   esize == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                              : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                   3, (void *)buf, dims,
                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(h, BORN_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  h->maps[key] = m;
  *out = m;
  return BORN_OK;
}

// z-segment depth of the sizing rule: segments sized so that the grid
// covers every SM about twice, at least 16 planes deep.
int rule_zseg(born_handle *h, int mode, bool pa, bool pb, int cfg,
              long long tiles) {
  const int nzi = h->n3 - 8;
  int tx, ty;
  born::tile_cfg_dims(cfg, &tx, &ty);
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const size_t smem =
      born::step_smem_bytes(h->storage_for(mode), cfg, mode, pa, pb);
  int per_sm = (int)std::max<size_t>(1, (227 * 1024) / (smem + 1024));
  per_sm = std::min(per_sm, 2048 / ((tx / 4) * ty));
  const long long target = 2ll * sms * per_sm;
  long long nseg = std::max<long long>(1, (target + tiles - 1) / tiles);
  nseg = std::min<long long>(nseg, std::max(1, nzi / 16));
  return (int)((nzi + nseg - 1) / nseg);
}

// Tiling: the configured one, else the autotuned one for the mode, else
// 64x16 tiles; z segments as configured, else as tuned with the tile, else
// by the sizing rule.
void pick_tiling(born_handle *h, int mode, bool pa, bool pb, int *cfg,
                 int *zseg, int *tiles_x, int *tiles_y) {
  const int slot = h->storage_for(mode);
  const int tuned = h->tuned_cfg[slot][mode];
  const int c = h->tile_cfg >= 0 ? h->tile_cfg : tuned >= 0 ? tuned : 0;
  int tx, ty;
  born::tile_cfg_dims(c, &tx, &ty);
  *cfg = c;
  *tiles_x = (h->n1 - 8 + tx - 1) / tx;
  *tiles_y = (h->n2 - 8 + ty - 1) / ty;
  const int nzi = h->n3 - 8;
  if (h->zseg > 0) {
    *zseg = std::min(h->zseg, nzi);
    return;
  }
  const int nseg = h->tuned_nseg[slot][mode];
  if (h->tile_cfg < 0 && tuned >= 0 && nseg > 0) {
    *zseg = (nzi + nseg - 1) / nseg;
    return;
  }
  *zseg = rule_zseg(h, mode, pa, pb, c, (long long)(*tiles_x) * (*tiles_y));
}

// Tilings a mode is tuned over: (tile configuration, z segments per column
// of tiles; 0 = the sizing rule) pairs, each tile with the rule's segments
// and with 3 to 16 segments (at least 8 planes each), without repeating a
// segment depth within a tile.
constexpr int kTuneSegs[] = {3, 4, 5, 6, 8, 10, 12, 16};

std::vector<std::pair<int, int>> tiling_candidates(born_handle *h, int mode,
                                                   bool pb) {
  std::vector<std::pair<int, int>> cand;
  const int ncfg = std::min(born::tile_cfg_count(), born_handle::kMaxTileCfgs);
  const int nzi = h->n3 - 8;
  for (int c = 0; c < ncfg; ++c) {
    int tx, ty;
    born::tile_cfg_dims(c, &tx, &ty);
    const long long tiles = (long long)((h->n1 - 8 + tx - 1) / tx) *
                            ((h->n2 - 8 + ty - 1) / ty);
    std::vector<int> seen{rule_zseg(h, mode, true, pb, c, tiles)};
    cand.push_back({c, 0});
    for (int ns : kTuneSegs) {
      if (nzi / ns < 8) break;
      const int zs = (nzi + ns - 1) / ns;
      if (std::find(seen.begin(), seen.end(), zs) != seen.end()) continue;
      seen.push_back(zs);
      cand.push_back({c, ns});
    }
  }
  if ((int)cand.size() > born_handle::kMaxLoopCands)
    cand.resize(born_handle::kMaxLoopCands);
  return cand;
}

PointSet point_view(const DevPoints &dp, int id, int ii,
                    const std::vector<float> &tab, float scale, bool use) {
  PointSet ps;
  memset(&ps, 0, sizeof(ps));
  ps.plane_off = dp.plane_off;
  ps.cell_head = dp.cell_head;
  ps.slot_cell = dp.slot_cell;
  ps.slot_index = dp.slot_index;
  ps.traces = dp.traces;
  ps.npts = dp.npts;
  ps.nt_trace = dp.nt;
  ps.zlo = dp.zlo;
  ps.zhi = dp.zhi;
  ps.id = id;
  ps.scale = scale;
  ps.absmax = dp.absmax;
  ps.mult = dp.mult;
  ps.active = use && dp.npts > 0 && (id + 7 < dp.nt) ? 1 : 0;
  if (ps.active)
    for (int k = 0; k < 8; ++k) ps.tab[k] = tab[(size_t)ii * 8 + k];
  return ps;
}

void base_params(born_handle *h, StepParams &p) {
  memset(&p, 0, sizeof(p));
  p.n1 = h->n1;
  p.n2 = h->n2;
  p.n3 = h->n3;
  memcpy(p.c, h->coeffs, sizeof(p.c));
  memcpy(p.bound, h->bound, sizeof(p.bound));
  p.err = h->err_dev;
  p.lv = h->lv_dev;
  float cs = std::fabs(h->coeffs[0]);
  for (int i = 1; i < 13; ++i) cs += 2.f * std::fabs(h->coeffs[i]);
  p.csum = cs;
  p.la = p.lb = born::LevelRefs{-1, -1, -1, 0u};
  p.vmax_a = p.vmax_b = p.imgmax = h->stat_dev;  // set per mode when used
  p.overlap = h->overlap ? 1 : 0;
}

// One step launch.  a_cur / b_cur: current levels of the propagated fields
// (halo boxes); centre[slot]: the per-cell inputs by born::CentreSlot.  With
// 16-bit storage the field levels (a_cur, b_cur and the previous-level
// slots) are 16-bit buffers.
int launch(born_handle *h, int mode, bool pa, bool pb, const void *a_cur,
           const void *b_cur, const void *const centre[born::kNumCentre],
           StepParams &p) {
  int cfg, zseg, tx, ty;
  pick_tiling(h, mode, pa, pb, &cfg, &zseg, &tx, &ty);
  p.tiles_x = tx;
  p.tiles_y = ty;
  p.zseg = zseg;
  born::StepMaps maps;
  const int fe = h->level_esize();
  const float *any = h->vel2;  // any valid grid buffer for unused slots
  // unused field maps still need a valid descriptor: any buffer of the
  // field's element size (a level buffer with 16-bit storage)
  const void *anyf = fe == 4 ? (const void *)any : (const void *)h->f0;
  int rc = get_map(h, a_cur ? a_cur : anyf, cfg, 0, fe, &maps.box_a);
  if (!rc) rc = get_map(h, b_cur ? b_cur : anyf, cfg, 0, fe, &maps.box_b);
  if (!rc) rc = get_map(h, a_cur ? a_cur : anyf, cfg, 1, fe, &maps.zc_a);
  if (!rc) rc = get_map(h, b_cur ? b_cur : anyf, cfg, 1, fe, &maps.zc_b);
  const unsigned mask = born::centre_mask(mode, pa, pb);
  for (int sl = 0; sl < born::kNumCentre && !rc; ++sl) {
    const bool used = mask & (1u << sl);
    if (used && !centre[sl])
      return fail(h, BORN_ESTATE, "step input %d missing", sl);
    const int es = born::field_slot(mode, sl) ? fe : 4;
    rc = get_map(h, used ? centre[sl] : (es == 4 ? (const void *)any : anyf),
                 cfg, 1, es, &maps.cm[sl]);
  }
  if (rc) return rc;
  CK(h, born::launch_step(h->storage_for(mode), mode, pa, pb, cfg, maps, p,
                          h->stream));
  h->launches++;
  return BORN_OK;
}

int check_device_error(born_handle *h);

// Autotuner: times every tile configuration of one step mode on the
// current grid (three sweeps of two warm-up and eight timed launches, CUDA
// events on the handle's stream) and keeps the fastest, per storage type.  It runs on the
// scratch levels f0/f1/r0/r1 and a temporary image with every point set
// inactive, so it never touches the source levels kept for rtm_adjoint nor
// an image a caller has yet to read, and clears the levels it used.
int tune_mode(born_handle *h, int mode) {
  const bool pb = mode == kModeForward || mode == kModeAdjoint ||
                  mode == born::kModeBornLin;
  if (!h->have_vel1 || !h->have_vel2) return BORN_OK;  // nothing to time yet
  float *timg = nullptr;
  CK(h, cudaMalloc(&timg, (size_t)h->n123 * 4));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMemsetAsync(timg, 0, (size_t)h->n123 * 4, h->stream) !=
          cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    cudaStreamSynchronize(h->stream);
    cudaFree(timg);
    return fail(h, BORN_ECUDA, "autotuner setup failed");
  }
  const int saved = h->tile_cfg, saved_zseg = h->zseg;
  int best = -1;
  float best_ms = 0.f;
  int rc = BORN_OK;
  const bool lp = h->lp();
  if (lp) {
    const void *reset[] = {h->f0, h->f1, h->r0, h->r1};
    rc = born_lp_prologue(h, h->stream, reset, 4);
  }
  // interleaved sweeps over the tilings, best sweep average per tiling:
  // tiles 3-4 % apart in the time loop were confused by two sweeps of four
  // timed launches (about 1.3 ms each on a 368^3 grid).  The source, rtm
  // adjoint and rtm forward loops refine tile and z segments on their own
  // steps, so they start from the tiles at the sizing rule's segments; the
  // exact pair's modes have no such refinement and take every candidate
  // tiling here.
  constexpr int kSweeps = 3, kWarm = 2, kTimed = 8;
  auto cand = tiling_candidates(h, mode, pb);
  if (mode <= kModeAdjoint)
    cand.erase(std::remove_if(cand.begin(), cand.end(),
                              [](const std::pair<int, int> &c) {
                                return c.second != 0;
                              }),
               cand.end());
  const int ncand = (int)cand.size(), nzi = h->n3 - 8;
  std::vector<float> cand_ms(ncand, -1.f);
  for (int sweep = 0; sweep < kSweeps * ncand && !rc; ++sweep) {
    const int ci = sweep % ncand, ns = cand[ci].second;
    h->tile_cfg = cand[ci].first;
    h->zseg = ns > 0 ? (nzi + ns - 1) / ns : 0;
    StepParams p;
    base_params(h, p);
    p.a_out = h->f1;
    p.b_out = h->r1;
    p.img_out = timg;
    if (lp) {
      born_set_lp_words(h, p, mode);
      // fixed record slots: the levels stay zero with every point inactive
      p.la = born_level_refs(h, h->f0, h->f1, true, 1u);
      p.lb = born_level_refs(h, h->r0, h->r1, true, 1u);
    }
    const void *cen[born::kNumCentre] = {h->f1, h->r1, h->vel2, h->vel1,
                                         mode == kModeForward ? h->refl : timg};
    for (int it = 0; it < kWarm + kTimed && !rc; ++it) {
      if (it == kWarm) cudaEventRecord(e0, h->stream);
      rc = launch(h, mode, true, pb, h->f0, h->r0, cen, p);
    }
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)kTimed;
    if (!rc && (cand_ms[ci] < 0.f || ms < cand_ms[ci])) cand_ms[ci] = ms;
  }
  for (int ci = 0; ci < ncand; ++ci)
    if (cand_ms[ci] >= 0.f && (best < 0 || cand_ms[ci] < best_ms)) {
      best = ci;
      best_ms = cand_ms[ci];
    }
  h->tile_cfg = saved;
  h->zseg = saved_zseg;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(h->stream);
  cudaFree(timg);
  if (rc) return rc;
  const int slot = h->storage_for(mode);
  h->tuned_cfg[slot][mode] = best >= 0 ? cand[best].first : 0;
  h->tuned_nseg[slot][mode] = best >= 0 ? cand[best].second : 0;
  h->tuned_ms[slot][mode] = best_ms;
  const size_t bytes = h->level_bytes();
  float *scratch[] = {h->f0, h->f1, h->r0, h->r1};
  for (float *b : scratch) CK(h, cudaMemsetAsync(b, 0, bytes, h->stream));
  return check_device_error(h);
}

int ensure_tuned(born_handle *h, int mode) {
  if (!h->autotune || h->tile_cfg >= 0 ||
      h->tuned_cfg[h->storage_for(mode)][mode] >= 0)
    return BORN_OK;
  return tune_mode(h, mode);
}

// Refines a mode's tiling on the steps of its long time loops.  Every
// tiling gives bit-identical results, so the loops' own steps are timed.
// The candidates are tiling_candidates' (tile, z segments) pairs.  The
// segment count moves the grid's last partial wave of
// CTAs: on a 368^3 grid the adjoint step on 64x8 tiles took 0.341 ms per
// launch with the rule's 4 segments and 0.314 ms with 10, and the best pairs
// of all three steps were 6-8 % faster than the best tile at the rule's
// segments.  From a loop's second step (the adjoint's first step is a
// lighter variant), candidates take turns in groups of one untimed step
// (the first launch with a tiling pays for its descriptors and attributes
// on the host) and kLoopGroup timed ones between CUDA events: one group per
// candidate, then kLoopRounds - 1 more rounds over the kLoopTop fastest of
// the first round.  A loop too short for the whole sweep times what fits
// and the next loop of the same storage and mode goes on from there.  When
// every group is timed, the loop continues with the candidate of the
// smallest group time, kept for later loops.  The scratch tuner's launches
// differ from a loop's (inactive points, fixed buffers) and picked a
// forward tile that ran 3.4 % slower in the loop than the best one (368^3
// grid).
constexpr int kLoopGroup = 8, kLoopRounds = 3, kLoopMinSteps = 400;

class LoopTuner {
 public:
  LoopTuner(born_handle *h, int mode, int nsteps, bool pb)
      : h_(h), mode_(mode), st_(h->storage_for(mode)) {
    if (!h->autotune || h->tile_cfg >= 0 || h->zseg > 0 ||
        nsteps < kLoopMinSteps || h->loop_tuned[st_][mode])
      return;
    cand_ = tiling_candidates(h, mode, pb);
    ncand_ = (int)cand_.size();
    ntop_ = std::min(ncand_, (int)born_handle::kLoopTop);
    total_ = ncand_ + ntop_ * (kLoopRounds - 1);
    g0_ = h->lt_next[st_][mode];
    if (g0_ == 0)
      for (float &b : h->lt_best[st_][mode]) b = -1.f;
    nloc_ = std::min(total_ - g0_, (nsteps - 2) / (kLoopGroup + 1));
    if (nloc_ <= 0) return;
    ev_.assign(2 * nloc_, nullptr);
    for (cudaEvent_t &e : ev_)
      if (cudaEventCreate(&e) != cudaSuccess) {
        release();
        return;
      }
    on_ = true;
  }
  ~LoopTuner() { release(); }
  LoopTuner(const LoopTuner &) = delete;
  LoopTuner &operator=(const LoopTuner &) = delete;

  // before launching the loop's step k (k = 0 for its first step)
  int before(int k) {
    if (!on_ || k < 1) return BORN_OK;
    const int g = (k - 1) / (kLoopGroup + 1), r = (k - 1) % (kLoopGroup + 1);
    if (r == 1 && g < nloc_)  // the group's timed steps start here
      CK(h_, cudaEventRecord(ev_[2 * g], h_->stream));
    if (r != 0) return BORN_OK;
    if (g > 0) CK(h_, cudaEventRecord(ev_[2 * g - 1], h_->stream));
    if (g < nloc_) {
      if (g0_ + g == ncand_) {
        // first round complete: keep its fastest candidates
        int rc = fold(g);
        if (rc) return rc;
        const float *best = h_->lt_best[st_][mode_];
        std::vector<int> order(ncand_);
        for (int i = 0; i < ncand_; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
          const float ta = best[a] < 0.f ? 3e38f : best[a];
          const float tb = best[b] < 0.f ? 3e38f : best[b];
          return ta < tb;
        });
        for (int i = 0; i < ntop_; ++i) h_->lt_top[st_][mode_][i] = order[i];
      }
      use(cand_of(g0_ + g));
      return BORN_OK;
    }
    return finish();
  }

 private:
  // candidate timed by global group G
  int cand_of(int G) const {
    return G < ncand_ ? G : h_->lt_top[st_][mode_][(G - ncand_) % ntop_];
  }
  void use(int i) {
    h_->tuned_cfg[st_][mode_] = cand_[i].first;
    h_->tuned_nseg[st_][mode_] = cand_[i].second;
  }
  // fold the times of this loop's groups [folded_, upto) into the handle
  int fold(int upto) {
    if (upto <= folded_) return BORN_OK;
    CK(h_, cudaEventSynchronize(ev_[2 * upto - 1]));
    float *best = h_->lt_best[st_][mode_];
    for (int i = folded_; i < upto; ++i) {
      float ms = 0.f;
      CK(h_, cudaEventElapsedTime(&ms, ev_[2 * i], ev_[2 * i + 1]));
      float &b = best[cand_of(g0_ + i)];
      if (b < 0.f || ms < b) b = ms;
    }
    folded_ = upto;
    return BORN_OK;
  }
  // every group of this loop is timed: go on with the best candidate so far
  // (the final choice when the sweep is complete)
  int finish() {
    int rc = fold(nloc_);
    if (rc) return rc;
    const float *best = h_->lt_best[st_][mode_];
    int pick = -1;
    for (int i = 0; i < ncand_; ++i)
      if (best[i] >= 0.f && (pick < 0 || best[i] < best[pick])) pick = i;
    if (pick >= 0) {
      use(pick);
      h_->tuned_ms[st_][mode_] = best[pick] / kLoopGroup;
    }
    h_->lt_next[st_][mode_] = g0_ + nloc_;
    if (g0_ + nloc_ >= total_) {
      float *tile_ms = h_->loop_ms[st_][mode_];
      for (int c = 0; c < born_handle::kMaxTileCfgs; ++c) tile_ms[c] = 0.f;
      for (int i = 0; i < ncand_; ++i) {
        float &t = tile_ms[cand_[i].first];
        const float ms = best[i] / kLoopGroup;
        if (best[i] >= 0.f && (t == 0.f || ms < t)) t = ms;
      }
      h_->loop_tuned[st_][mode_] = true;
    }
    release();
    return BORN_OK;
  }
  void release() {
    for (cudaEvent_t e : ev_)
      if (e) cudaEventDestroy(e);
    ev_.clear();
    on_ = false;
  }
  born_handle *h_;
  int mode_, st_;
  int ncand_ = 0, ntop_ = 0, total_ = 0, g0_ = 0, nloc_ = 0, folded_ = 0;
  bool on_ = false;
  std::vector<std::pair<int, int>> cand_;  // (tile configuration, segments)
  std::vector<cudaEvent_t> ev_;
};

// Every this many steps the loops look at the device error word, so that a
// kernel whose bounded wait gave up stops the loop instead of being followed
// by thousands of launches that would each exit early.
constexpr int kErrPollSteps = 256;

int poll_error(born_handle *h, int step) {
  if (step % kErrPollSteps != kErrPollSteps - 1) return BORN_OK;
  unsigned int e = 0;
  CK(h, cudaMemcpyAsync(&e, h->err_dev, sizeof(e), cudaMemcpyDeviceToHost,
                        h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (e)
    return fail(h, BORN_ETIMEOUT,
                "a device-side wait gave up (error word 0x%x)", e);
  return BORN_OK;
}

int check_ready(born_handle *h) {
  if (!h) return BORN_EINVAL;
  if (!h->have_space)
    return fail(h, BORN_ESTATE, "create_space has not been called");
  return set_device(h);
}

int check_device_error(born_handle *h) {
  unsigned int e = 0;
  CK(h, cudaMemcpyAsync(&e, h->err_dev, sizeof(e), cudaMemcpyDeviceToHost,
                        h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (e) {
    cudaMemsetAsync(h->err_dev, 0, sizeof(unsigned int), h->stream);
    return fail(h, BORN_ETIMEOUT,
                "a device-side wait gave up (error word 0x%x)", e);
  }
  return BORN_OK;
}

// Closing copies of a time loop.  On GB300 the first device-to-host copy
// into a page-locked array took from a few to tens of milliseconds (199 MB:
// 2-24 ms, against 0.96 ms for the next copy into it) once other host arrays
// had been copied since that array's last use, as between the calls of an
// RTM shot.  So a loop that ends with such a copy first copies into the same
// array on the handle's side stream while its steps run; the closing copy,
// ordered after that one, overwrites every byte.  Pageable arrays are left
// alone (a copy into them would hold the host thread).
constexpr int kPrewarmMinSteps = 100;
constexpr size_t kPrewarmMinBytes = size_t(8) << 20;

void release_side(born_handle *h) {
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->side_go) cudaEventDestroy(h->side_go);
  if (h->side_done) cudaEventDestroy(h->side_done);
  if (h->side) cudaStreamDestroy(h->side);
  h->side = nullptr;
  h->side_go = h->side_done = nullptr;
}

int prewarm_d2h(born_handle *h, void *dst, const void *src, size_t bytes,
                int nt) {
  if (!h->prewarm || !dst || nt < kPrewarmMinSteps || bytes < kPrewarmMinBytes)
    return BORN_OK;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, dst) != cudaSuccess) {
    cudaGetLastError();
    return BORN_OK;
  }
  if (a.type != cudaMemoryTypeHost) return BORN_OK;
  if (!h->side) {
    if (cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) !=
            cudaSuccess ||
        cudaEventCreateWithFlags(&h->side_go, cudaEventDisableTiming) !=
            cudaSuccess ||
        cudaEventCreateWithFlags(&h->side_done, cudaEventDisableTiming) !=
            cudaSuccess) {
      cudaGetLastError();
      release_side(h);
      return BORN_OK;  // the closing copy then runs without it
    }
  }
  // after everything the call has queued so far (an upload from the array)
  CK(h, cudaEventRecord(h->side_go, h->stream));
  CK(h, cudaStreamWaitEvent(h->side, h->side_go, 0));
  CK(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->side));
  CK(h, cudaEventRecord(h->side_done, h->side));
  h->prewarm_pending = true;
  h->prewarm_copies++;
  return BORN_OK;
}

// Orders the closing copies after the warming ones.
int prewarm_join(born_handle *h) {
  if (!h->prewarm_pending) return BORN_OK;
  h->prewarm_pending = false;
  CK(h, cudaStreamWaitEvent(h->stream, h->side_done, 0));
  return BORN_OK;
}

// A call that returns early waits for its warming copies, so that none of
// them writes into a caller's array after the call.
struct PrewarmGuard {
  born_handle *h;
  ~PrewarmGuard() {
    if (h->prewarm_pending) {
      cudaStreamSynchronize(h->side);
      h->prewarm_pending = false;
    }
  }
};

}  // namespace

int born_fail(born_handle *h, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  return code;
}
int born_check_ready(born_handle *h) { return check_ready(h); }
born::PointSet born_point_view(const DevPoints &dp, int id, int ii,
                               const std::vector<float> &tab, float scale,
                               bool use) {
  return point_view(dp, id, ii, tab, scale, use);
}
void born_base_params(born_handle *h, StepParams &p) { base_params(h, p); }
int born_get_map(born_handle *h, const void *buf, int cfg, int kind,
                 int esize, CUtensorMap *out) {
  return get_map(h, buf, cfg, kind, esize, out);
}
void born_pick_tiling(born_handle *h, int mode, bool pa, bool pb, int *cfg,
                      int *zseg, int *tiles_x, int *tiles_y) {
  pick_tiling(h, mode, pa, pb, cfg, zseg, tiles_x, tiles_y);
}
int born_ensure_tuned(born_handle *h, int mode) { return ensure_tuned(h, mode); }
int born_check_device_error(born_handle *h) { return check_device_error(h); }

int born_level_id(const born_handle *h, const void *buf) {
  const void *b[kNumLevelBufs] = {h->s0, h->s1, h->r0, h->r1, h->f0, h->f1};
  for (int i = 0; i < kNumLevelBufs; ++i)
    if (buf && b[i] == buf) return i;
  return -1;
}

born::LevelRefs born_level_refs(const born_handle *h, const void *cur,
                                const void *old, bool write, unsigned int tag) {
  born::LevelRefs r{-1, -1, -1, tag};
  const int c = born_level_id(h, cur), o = born_level_id(h, old);
  if (c >= 0) r.cur = 2 * c + (h->wr[c] & 1);
  if (o >= 0) {
    r.old = 2 * o + (h->wr[o] & 1);
    if (write) r.out = 2 * o + ((h->wr[o] + 1) & 1);
  }
  return r;
}

void born_level_written(born_handle *h, const void *buf) {
  const int i = born_level_id(h, buf);
  if (i >= 0) h->wr[i]++;
}

int born_lp_prologue(born_handle *h, cudaStream_t s, const void *const *reset,
                     int nreset) {
  if (!h->lp()) return BORN_OK;
  unsigned int *st = h->stat_dev;
  CK(h, cudaMemsetAsync(st, 0, kNumStats * sizeof(unsigned int), s));
  const float *arr[3] = {h->vel1, h->vel2, h->refl};
  for (int k = 0; k < 3; ++k) {
    CK(h, born::launch_absmax(arr[k], h->n123, st + k, s));
    h->launches++;
  }
  const DevPoints *pts[2] = {&h->src, &h->rec};
  for (int k = 0; k < 2; ++k)
    if (pts[k]->npts > 0) {
      CK(h, born::launch_absmax(pts[k]->traces,
                                (long long)pts[k]->npts * pts[k]->nt,
                                st + kStatSrc + k, s));
      h->launches++;
    }
  for (int i = 0; i < nreset; ++i) {
    const int id = born_level_id(h, reset[i]);
    if (id < 0) continue;
    CK(h, born::launch_level_reset(h->lv_dev, id, s));
    h->launches++;
    h->wr[id] = 0;
  }
  return BORN_OK;
}

int born_copy_level(born_handle *h, void *dst, const void *src,
                    unsigned int tag, cudaStream_t s) {
  CK(h, cudaMemcpyAsync(dst, src, h->level_bytes(), cudaMemcpyDeviceToDevice,
                        s));
  const int d = born_level_id(h, dst), c = born_level_id(h, src);
  if (h->lp() && d >= 0 && c >= 0) {
    CK(h, born::launch_level_copy(h->lv_dev, 2 * d + ((h->wr[d] + 1) & 1),
                                  2 * c + (h->wr[c] & 1), tag, s));
    h->launches++;
  }
  if (d >= 0) h->wr[d]++;
  return BORN_OK;
}

void born_set_lp_words(born_handle *h, StepParams &p, int mode) {
  unsigned int *st = h->stat_dev;
  if (mode == kModeSource) {
    p.vmax_a = p.vmax_b = st + kStatVel1;
  } else if (mode == kModeAdjoint) {
    p.vmax_a = st + kStatVel2;  // receiver field through vel2
    p.vmax_b = st + kStatVel1;  // source field rebuilt through vel1
  } else {
    p.vmax_a = p.vmax_b = st + kStatVel2;
  }
  p.imgmax = st + kStatRefl;
}

// Checksum of a host level array for BORN_HOST_LEVELS_VERIFY: four
// independent xor-multiply lanes over the 32-bit words (so the loop is not
// one long dependency chain), folded at the end.  It detects any change a
// caller makes to the array between source_prop and rtm_adjoint; it is not
// meant to resist deliberate collisions.
unsigned long long host_level_sum(const float *p, long long n) {
  const unsigned int *w = reinterpret_cast<const unsigned int *>(p);
  const unsigned long long K = 0x9E3779B97F4A7C15ull;
  unsigned long long a = 1, b = 2, c = 3, d = 4;
  long long i = 0;
  for (; i + 4 <= n; i += 4) {
    a = (a ^ w[i]) * K;
    b = (b ^ w[i + 1]) * K;
    c = (c ^ w[i + 2]) * K;
    d = (d ^ w[i + 3]) * K;
  }
  for (; i < n; ++i) a = (a ^ w[i]) * K;
  unsigned long long x = a ^ (b * 3) ^ (c * 5) ^ (d * 7) ^ (unsigned long long)n;
  x ^= x >> 31;
  return x * K;
}

// ===========================================================================
// Handle API
extern "C" {

int born_create(int device, born_handle **out) {
  if (!out) return BORN_EINVAL;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return BORN_ENODEV;
  if (device < 0 || device >= n) return BORN_EINVAL;
  born_handle *h = new born_handle();
  h->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaMalloc(&h->err_dev, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(h->err_dev, 0, sizeof(unsigned int)) != cudaSuccess ||
      cudaMalloc(&h->lv_dev, kNumLevelBufs * 4 * sizeof(unsigned long long)) !=
          cudaSuccess ||
      cudaMalloc(&h->stat_dev, kNumStats * sizeof(unsigned int)) !=
          cudaSuccess ||
      cudaMemset(h->stat_dev, 0, kNumStats * sizeof(unsigned int)) !=
          cudaSuccess) {
    cudaFree(h->err_dev);
    cudaFree(h->lv_dev);
    cudaFree(h->stat_dev);
    delete h;
    return BORN_ECUDA;
  }
  for (int b = 0; b < kNumLevelBufs; ++b)
    born::launch_level_reset(h->lv_dev, b, h->stream);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    born_destroy(h);
    return BORN_ECUDA;
  }
  *out = h;
  return BORN_OK;
}

int born_destroy(born_handle *h) {
  if (!h) return BORN_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  free_fields(h);
  h->src.release();
  h->rec.release();
  cudaFree(h->err_dev);
  cudaFree(h->lv_dev);
  cudaFree(h->stat_dev);
  release_side(h);
  cudaStreamDestroy(h->stream);
  delete h;
  return BORN_OK;
}

const char *born_error_string(const born_handle *h) {
  return h ? h->err.c_str() : "null handle";
}

int born_create_space(born_handle *h, float d1, float d2, float d3, float bc_a,
                      float bc_b, float bc_y, int nx, int ny, int nz) {
  (void)bc_a;
  (void)bc_b;
  (void)bc_y;  // the reference's taper ignores them (cpu_prop.cc:329-331)
  if (!h) return BORN_EINVAL;
  if (nx < 9 || ny < 9 || nz < 9 || nx % 4 != 0)
    return fail(h, BORN_EINVAL,
                "grid %d x %d x %d: need every n >= 9 and nx %% 4 == 0", nx,
                ny, nz);
  if ((long long)nx * ny * nz >= (1ll << 31))
    return fail(h, BORN_EINVAL, "grid too large (n123 >= 2^31)");
  if (!(d1 > 0 && d2 > 0 && d3 > 0))
    return fail(h, BORN_EINVAL, "spacings must be positive");
  int rc = set_device(h);
  if (rc) return rc;
  // tile choices depend on the grid only: a new space over the same grid
  // (the next operator of a job) keeps them
  const bool same_grid =
      h->have_space && nx == h->n1 && ny == h->n2 && nz == h->n3;
  cudaStreamSynchronize(h->stream);
  free_fields(h);
  h->src.release();
  h->rec.release();
  h->n1 = nx;
  h->n2 = ny;
  h->n3 = nz;
  h->n123 = (long long)nx * ny * nz;
  make_coeffs(h->coeffs, d1, d2, d3);
  make_bound(h->bound);
  const size_t bytes = (size_t)h->n123 * sizeof(float);
  float **bufs[] = {&h->vel1, &h->vel2, &h->s0, &h->s1, &h->r0,
                    &h->r1,   &h->f0,   &h->f1, &h->img, &h->refl};
  for (float **b : bufs) {
    cudaError_t e = cudaMalloc(b, bytes);
    if (e != cudaSuccess) {
      free_fields(h);
      return fail(h, BORN_ENOMEM, "cudaMalloc of %zu bytes failed: %s", bytes,
                  cudaGetErrorString(e));
    }
    CK(h, cudaMemsetAsync(*b, 0, bytes, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  h->have_space = true;
  h->generation++;
  h->bg_gen++;
  if (!same_grid) h->reset_tuning();
  return BORN_OK;
}

int born_set_sinc_table(born_handle *h, int which, int nsinc, int jt,
                        const float *table) {
  if (!h) return BORN_EINVAL;
  if (nsinc != 8 || jt < 1 || !table || (which != 0 && which != 1))
    return fail(h, BORN_EINVAL, "sinc table: need nsinc == 8, jt >= 1");
  std::vector<float> t(table, table + (size_t)jt * 8);
  h->generation++;  // table values are baked into recorded graphs
  if (which == 0) {
    h->tab_s = t;
    h->jt_s = jt;
    h->bg_gen++;
  } else {
    h->tab_d = t;
    h->jt_d = jt;
  }
  return BORN_OK;
}

int born_set_source_func(born_handle *h, int npts, int nt_big, const int *locs,
                         const float *vals) {
  int rc = check_ready(h);
  if (rc) return rc;
  h->src_levels_valid = false;
  h->bg_gen++;
  return upload_points(h, h->src, npts, nt_big, locs, vals);
}

int born_set_receiver_func(born_handle *h, int rec_nx, int rec_ny, int nt_big,
                           const int *locs, const float *traces) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (rec_nx < 0 || rec_ny < 0)
    return fail(h, BORN_EINVAL, "bad receiver grid");
  return upload_points(h, h->rec, rec_nx * rec_ny, nt_big, locs, traces);
}

int born_set_velocity(born_handle *h, int slot, int nx, int ny, int nz,
                      const float *v) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (nx != h->n1 || ny != h->n2 || nz != h->n3 || !v || (slot != 1 && slot != 2))
    return fail(h, BORN_EINVAL, "velocity: grid mismatch or bad slot");
  float *dst = slot == 1 ? h->vel1 : h->vel2;
  CK(h, cudaMemcpyAsync(dst, v, (size_t)h->n123 * 4, cudaMemcpyHostToDevice,
                        h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  (slot == 1 ? h->have_vel1 : h->have_vel2) = true;
  if (slot == 2) h->bg_gen++;
  return BORN_OK;
}

int born_set_reflectivity(born_handle *h, const float *img) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (!img) return fail(h, BORN_EINVAL, "null reflectivity");
  CK(h, cudaMemcpyAsync(h->refl, img, (size_t)h->n123 * 4,
                        cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->have_refl = true;
  return BORN_OK;
}

// cpuProp::sourceProp, cpu_prop.cc:106-129
int born_source_prop(born_handle *h, int jts, int nt, float *p0_out,
                     float *p1_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (nt < 0 || jts < 1) return fail(h, BORN_EINVAL, "nt < 0 or jts < 1");
  if (!h->have_vel1) return fail(h, BORN_ESTATE, "vel1 not transferred");
  if (h->jt_s < 1) return fail(h, BORN_ESTATE, "source sinc table missing");
  if ((p0_out || p1_out) && h->lp())
    return fail(h, BORN_ESTATE, "host copies of the levels need FP32 storage");
  h->jt = jts;
  rc = ensure_tuned(h, kModeSource);
  if (rc) return rc;
  const size_t lbytes = h->level_bytes(), bytes = (size_t)h->n123 * 4;
  CK(h, cudaMemsetAsync(h->s0, 0, lbytes, h->stream));
  CK(h, cudaMemsetAsync(h->s1, 0, lbytes, h->stream));
  {
    const void *reset[] = {h->s0, h->s1};
    rc = born_lp_prologue(h, h->stream, reset, 2);
    if (rc) return rc;
  }
  PrewarmGuard pw{h};
  rc = prewarm_d2h(h, p0_out, h->s0, bytes, nt);
  if (!rc) rc = prewarm_d2h(h, p1_out, h->s1, bytes, nt);
  if (rc) return rc;
  float *p0 = h->s0, *p1 = h->s1;
  const float scale = 1 / (float)jts;
  LoopTuner tuner(h, kModeSource, nt + 1, false);
  for (int it = 0; it <= nt; ++it) {
    rc = tuner.before(it);
    if (rc) return rc;
    const int id = it / h->jt_s, ii = it - id * h->jt_s;
    StepParams p;
    base_params(h, p);
    p.a_out = p0;
    p.pa = point_view(h->src, id, ii, h->tab_s, scale, true);
    p.pb = point_view(h->src, 0, 0, h->tab_s, 0.f, false);
    born_set_lp_words(h, p, kModeSource);
    p.la = born_level_refs(h, p1, p0, true, kTagSource + it);
    const void *cen[born::kNumCentre] = {p0, nullptr, h->vel1, nullptr,
                                         nullptr};
    rc = launch(h, kModeSource, true, false, p1, nullptr, cen, p);
    if (!rc) rc = poll_error(h, it);
    if (rc) return rc;
    born_level_written(h, p0);
    std::swap(p0, p1);
  }
  if (nt % 2 == 1) {
    rc = born_copy_level(h, p1, p0, kTagSource + nt + 1, h->stream);
    if (rc) return rc;
  }
  h->src_levels_valid = true;
  h->host_p0 = p0_out;
  h->host_p1 = p1_out;
  h->host_sums_valid = false;
  rc = prewarm_join(h);
  if (rc) return rc;
  if (p0_out) CK(h, cudaMemcpyAsync(p0_out, h->s0, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (p1_out) CK(h, cudaMemcpyAsync(p1_out, h->s1, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (p0_out || p1_out) {
    rc = check_device_error(h);
    if (rc) return rc;
    if (h->host_levels == BORN_HOST_LEVELS_VERIFY && p0_out && p1_out) {
      h->host_sum0 = host_level_sum(p0_out, h->n123);
      h->host_sum1 = host_level_sum(p1_out, h->n123);
      h->host_sums_valid = true;
    }
  }
  return BORN_OK;
}

// cpuProp::rtmAdjoint, cpu_prop.cc:56-96
int born_rtm_adjoint(born_handle *h, int jtd, int nt, int swap,
                     float *img_out) {
  (void)jtd;  // the data table's own jt indexes the traces (cpu_prop.cc:75)
  int rc = check_ready(h);
  if (rc) return rc;
  if (nt < 1) return fail(h, BORN_EINVAL, "nt < 1");
  if (!h->have_vel1 || !h->have_vel2)
    return fail(h, BORN_ESTATE, "velocities not transferred");
  if (h->jt_s < 1 || h->jt_d < 1)
    return fail(h, BORN_ESTATE, "sinc tables missing");
  if (!h->src_levels_valid)
    return fail(h, BORN_ESTATE, "no source levels (run source_prop first)");
  rc = ensure_tuned(h, kModeAdjoint);
  if (rc) return rc;
  const size_t lbytes = h->level_bytes(), bytes = (size_t)h->n123 * 4;
  CK(h, cudaMemsetAsync(h->r0, 0, lbytes, h->stream));
  CK(h, cudaMemsetAsync(h->r1, 0, lbytes, h->stream));
  {
    const void *reset[] = {h->r0, h->r1};
    rc = born_lp_prologue(h, h->stream, reset, 2);
    if (rc) return rc;
  }
  // cpuProp accumulates into the caller's image (cpu_prop.cc:101)
  if (img_out)
    CK(h, cudaMemcpyAsync(h->img, img_out, bytes, cudaMemcpyHostToDevice,
                          h->stream));
  else
    CK(h, cudaMemsetAsync(h->img, 0, bytes, h->stream));
  PrewarmGuard pw{h};
  rc = prewarm_d2h(h, img_out, h->img, bytes, nt);
  if (rc) return rc;
  float *sp0 = swap ? h->s1 : h->s0, *sp1 = swap ? h->s0 : h->s1;
  float *rp0 = h->r0, *rp1 = h->r1;
  const float scale = -1 / (float)h->jt;
  PointSet pending = point_view(h->src, 0, 0, h->tab_s, 0.f, false);
  LoopTuner tuner(h, kModeAdjoint, nt, true);
  for (int it = nt - 1; it >= 0; --it) {
    rc = tuner.before(nt - 1 - it);
    if (rc) return rc;
    const int id_s = (it + 1) / h->jt_s, i_s = it + 1 - id_s * h->jt_s;
    const int id = it / h->jt_d, ii = it - id * h->jt_d;
    const bool pa = it > 0, pb = it < nt - 1;
    StepParams p;
    base_params(h, p);
    p.a_out = rp0;
    p.b_out = sp0;
    p.img_out = h->img;
    p.pa = point_view(h->rec, id, ii, h->tab_d, scale, true);
    p.pb = pending;
    born_set_lp_words(h, p, kModeAdjoint);
    const unsigned int tag = kTagAdjoint + 2u * (unsigned int)(nt - 1 - it);
    p.la = born_level_refs(h, pa ? rp1 : nullptr, rp0, true, tag);
    p.lb = born_level_refs(h, pb ? sp1 : nullptr, sp0, pb, tag + 1u);
    const void *cen[born::kNumCentre] = {rp0, sp0, h->vel2, h->vel1, h->img};
    rc = launch(h, kModeAdjoint, pa, pb, pa ? rp1 : nullptr,
                pb ? sp1 : nullptr, cen, p);
    if (!rc) rc = poll_error(h, nt - 1 - it);
    if (rc) return rc;
    born_level_written(h, rp0);
    if (pb) born_level_written(h, sp0);
    // the source injection of this step goes into the current level, which
    // the next step reads as its previous level (cpu_prop.cc:79-82)
    pending = point_view(h->src, id_s, i_s, h->tab_s, scale, pb);
    std::swap(sp0, sp1);
    std::swap(rp0, rp1);
  }
  if (pending.active) {
    const int id = born_level_id(h, sp0);
    CK(h, born::launch_point_inject(pending, h->src.npts, sp0, h->storage,
                                    h->lv_dev, 2 * id + (h->wr[id] & 1),
                                    h->stream));
    h->launches++;
  }
  if (img_out) {
    rc = prewarm_join(h);
    if (rc) return rc;
    CK(h, cudaMemcpyAsync(img_out, h->img, bytes, cudaMemcpyDeviceToHost,
                          h->stream));
    return check_device_error(h);
  }
  return BORN_OK;
}

int born_set_host_levels(born_handle *h, int policy) {
  if (!h) return BORN_EINVAL;
  if (policy != BORN_HOST_LEVELS_RESIDENT &&
      policy != BORN_HOST_LEVELS_VERIFY && policy != BORN_HOST_LEVELS_UPLOAD)
    return fail(h, BORN_EINVAL, "unknown host-level policy %d", policy);
  h->host_levels = policy;
  // checksums are only taken while verifying: a later source_prop makes them
  h->host_sums_valid = false;
  return BORN_OK;
}

// baseProp::rtmAdjoint on host arrays of the source levels (base_prop.h:57-62)
int born_rtm_adjoint_host(born_handle *h, int jtd, int nt, const float *p0,
                          const float *p1, float *img) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (!p0 || !p1) return fail(h, BORN_EINVAL, "null source level array");
  int swap = -1;  // -1: upload p0/p1
  if (h->host_levels != BORN_HOST_LEVELS_UPLOAD && h->src_levels_valid &&
      h->host_p0 && h->host_p1) {
    if (p0 == h->host_p1 && p1 == h->host_p0)
      swap = 1;
    else if (p0 == h->host_p0 && p1 == h->host_p1)
      swap = 0;
    if (swap >= 0 && h->host_levels == BORN_HOST_LEVELS_VERIFY) {
      // the arrays still hold what source_prop wrote into them?
      const bool same =
          h->host_sums_valid &&
          host_level_sum(h->host_p0, h->n123) == h->host_sum0 &&
          host_level_sum(h->host_p1, h->n123) == h->host_sum1;
      if (!same) swap = -1;
    }
  }
  if (swap < 0) {
    rc = born_set_source_levels(h, p0, p1);
    if (rc) return rc;
    // the device levels now mirror these arrays (s0 <- p0, s1 <- p1)
    h->host_p0 = p0;
    h->host_p1 = p1;
    h->host_sums_valid = false;
    if (h->host_levels == BORN_HOST_LEVELS_VERIFY) {
      h->host_sum0 = host_level_sum(p0, h->n123);
      h->host_sum1 = host_level_sum(p1, h->n123);
      h->host_sums_valid = true;
    }
    swap = 0;
  }
  return born_rtm_adjoint(h, jtd, nt, swap, img);
}

// cpuProp::rtmForward, cpu_prop.cc:22-54
int born_rtm_forward(born_handle *h, int jt, int nt, float *traces_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (nt < 0 || jt < 1) return fail(h, BORN_EINVAL, "nt < 0 or jt < 1");
  if (!h->have_vel2 || !h->have_refl)
    return fail(h, BORN_ESTATE, "vel2 or reflectivity not transferred");
  if (jt > h->jt_s || jt > h->jt_d)
    return fail(h, BORN_EINVAL, "jt %d exceeds the sinc tables' rows", jt);
  h->jt = jt;
  rc = ensure_tuned(h, kModeForward);
  if (rc) return rc;
  const size_t lbytes = h->level_bytes();
  CK(h, cudaMemsetAsync(h->f0, 0, lbytes, h->stream));
  CK(h, cudaMemsetAsync(h->f1, 0, lbytes, h->stream));
  CK(h, cudaMemsetAsync(h->r0, 0, lbytes, h->stream));
  CK(h, cudaMemsetAsync(h->r1, 0, lbytes, h->stream));
  {
    const void *reset[] = {h->f0, h->f1, h->r0, h->r1};
    rc = born_lp_prologue(h, h->stream, reset, 4);
    if (rc) return rc;
  }
  PrewarmGuard pw{h};
  rc = prewarm_d2h(h, traces_out, h->rec.traces,
                   (size_t)h->rec.npts * h->rec.nt * 4, nt);
  if (rc) return rc;
  float *sp0 = h->f0, *sp1 = h->f1, *rp0 = h->r0, *rp1 = h->r1;
  const float scale = 1 / (float)jt;
  LoopTuner tuner(h, kModeForward, nt, true);
  for (int it = 0; it < nt; ++it) {
    rc = tuner.before(it);
    if (rc) return rc;
    const int id = it / jt, ii = it - id * jt;
    StepParams p;
    base_params(h, p);
    p.a_out = sp0;
    p.b_out = rp0;
    p.pa = point_view(h->src, id, ii, h->tab_s, scale, true);
    p.pb = point_view(h->rec, id, ii, h->tab_d, 0.f, true);
    born_set_lp_words(h, p, kModeForward);
    const unsigned int tag = kTagForward + 2u * (unsigned int)it;
    p.la = born_level_refs(h, sp1, sp0, true, tag);
    p.lb = born_level_refs(h, rp1, rp0, true, tag + 1u);
    const void *cen[born::kNumCentre] = {sp0, rp0, h->vel2, nullptr,
                                         h->refl};
    rc = launch(h, kModeForward, true, true, sp1, rp1, cen, p);
    if (!rc) rc = poll_error(h, it);
    if (rc) return rc;
    born_level_written(h, sp0);
    born_level_written(h, rp0);
    std::swap(sp0, sp1);
    std::swap(rp0, rp1);
  }
  if (traces_out) {
    rc = prewarm_join(h);
    if (rc) return rc;
    CK(h, cudaMemcpyAsync(traces_out, h->rec.traces,
                          (size_t)h->rec.npts * h->rec.nt * 4,
                          cudaMemcpyDeviceToHost, h->stream));
    return check_device_error(h);
  }
  return BORN_OK;
}

// ---------------------------------------------------------------------------
// Nonlinear modelling and the exact linearised Born pair.
//
// Modelling (the background of cpuProp::rtmForward with its own traces):
//   s_{t+1} = B (V A s_t + 2 s_t - B s_{t-1}) + Q_t,   d_t = E_t s_{t+1}
// with V = vel2 (v^2 dt^2), B the taper, Q_t the source injection and E_t
// the sinc extraction of step t.  Its derivative with respect to V along m:
//   r_{t+1} = B (V A r_t + 2 r_t - B r_{t-1} + m (A s_t)),   δd_t = E_t r_{t+1}
// and the exact transpose of that map, in the variable w = V μ:
//   w_{t+1} = B (V A w_{t+2} + 2 w_{t+2} - B w_{t+3} + V E_t^T δd),
//   m̄ = (1/V) Σ_t (A s_t) w_{t+1}
// (A is the symmetric interior stencil, V and B are diagonal).  The adjoint
// needs A s_t in reverse order: s is checkpointed every `interval` steps and
// each segment is recomputed forward, storing A s_t, before the reverse
// sweep over it.

int born_model(born_handle *h, int jt, int nt, float *traces_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->lp())
    return fail(h, BORN_ESTATE, "%s needs FP32 storage", __func__);
  if (nt < 0 || jt < 1) return fail(h, BORN_EINVAL, "nt < 0 or jt < 1");
  if (!h->have_vel2) return fail(h, BORN_ESTATE, "vel2 not transferred");
  if (jt > h->jt_s || jt > h->jt_d)
    return fail(h, BORN_EINVAL, "jt %d exceeds the sinc tables' rows", jt);
  rc = ensure_tuned(h, born::kModeModel);
  if (rc) return rc;
  const size_t bytes = (size_t)h->n123 * 4;
  CK(h, cudaMemsetAsync(h->f0, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->f1, 0, bytes, h->stream));
  float *sp0 = h->f0, *sp1 = h->f1;
  const float scale = 1 / (float)jt;
  for (int it = 0; it < nt; ++it) {
    const int id = it / jt, ii = it - id * jt;
    StepParams p;
    base_params(h, p);
    p.a_out = sp0;
    p.pa = point_view(h->src, id, ii, h->tab_s, scale, true);
    p.pb = point_view(h->rec, id, ii, h->tab_d, 0.f, true);
    const void *cen[born::kNumCentre] = {sp0, nullptr, h->vel2, nullptr,
                                          nullptr};
    rc = launch(h, born::kModeModel, true, false, sp1, nullptr, cen, p);
    if (!rc) rc = poll_error(h, it);
    if (rc) return rc;
    std::swap(sp0, sp1);
  }
  if (traces_out) {
    CK(h, cudaMemcpyAsync(traces_out, h->rec.traces,
                          (size_t)h->rec.npts * h->rec.nt * 4,
                          cudaMemcpyDeviceToHost, h->stream));
    return check_device_error(h);
  }
  return BORN_OK;
}

namespace {
// CUDA events recorded one after another on the handle's stream (none when
// count is 0); elapsed() waits for the later event.
struct PhaseEvents {
  born_handle *h;
  std::vector<cudaEvent_t> ev;
  int next = 0;
  PhaseEvents(born_handle *hh, int count) : h(hh) {
    for (int i = 0; i < count; ++i) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) break;
      ev.push_back(e);
    }
  }
  ~PhaseEvents() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  int record() {
    if (ev.empty()) return BORN_OK;
    if (next >= (int)ev.size())
      return fail(h, BORN_ECUDA, "phase timing: out of events");
    CK(h, cudaEventRecord(ev[next++], h->stream));
    return BORN_OK;
  }
  int elapsed(int a, int b, float *ms) {
    CK(h, cudaEventSynchronize(ev[b]));
    CK(h, cudaEventElapsedTime(ms, ev[a], ev[b]));
    return BORN_OK;
  }
};

int ensure_levels(born_handle *h, float **buf, size_t *have, size_t levels) {
  if (*have >= levels) return BORN_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  CK(h, cudaMalloc(buf, levels * (size_t)h->n123 * 4));
  *have = levels;
  return BORN_OK;
}

// Room for `levels` checkpoint levels in the handle's checkpoint storage
// (FP32, or FP16 with one scale per level).  Reallocating drops the
// checkpoints held.
int ensure_ckpt(born_handle *h, size_t levels) {
  const size_t esize = h->ckpt_storage == BORN_CKPT_F16 ? 2 : 4;
  const size_t bytes = levels * (size_t)h->n123 * esize;
  if (h->ckpt_bytes < bytes) {
    cudaFree(h->ckpt);
    h->ckpt = nullptr;
    h->ckpt_bytes = 0;
    h->ckpt_valid = false;
    CK(h, cudaMalloc(&h->ckpt, bytes));
    h->ckpt_bytes = bytes;
  }
  if (h->ckpt_storage == BORN_CKPT_F16) {
    if (h->ckpt_scale_levels < levels) {
      cudaFree(h->ckpt_scale);
      h->ckpt_scale = nullptr;
      h->ckpt_scale_levels = 0;
      h->ckpt_valid = false;
      CK(h, cudaMalloc(&h->ckpt_scale, levels * sizeof(float)));
      h->ckpt_scale_levels = levels;
    }
    if (!h->ckpt_maxw) CK(h, cudaMalloc(&h->ckpt_maxw, sizeof(unsigned int)));
  }
  return BORN_OK;
}

// Checkpoint k of the background: its two levels (old, cur) = (s_{t-1},
// s_t) as stored at step t.  FP32: plain copies into levels 2k, 2k+1.
// FP16: level 2k+1 holds cur and level 2k the difference old - cur, each
// with its own power-of-two scale.  The difference is about omega dt of
// the field, so it keeps FP16's relative precision at that small size:
// the time derivative the leapfrog restarts from stays accurate, where two
// independently rounded levels would differ by their rounding noise.
int store_ckpt(born_handle *h, size_t k, const float *old, const float *cur) {
  const size_t n = (size_t)h->n123;
  if (h->ckpt_storage == BORN_CKPT_F16) {
    unsigned short *base = reinterpret_cast<unsigned short *>(h->ckpt);
    CK(h, born::launch_snapshot_f16(cur, nullptr, (long long)n, h->ckpt_maxw,
                                    base + (2 * k + 1) * n,
                                    h->ckpt_scale + 2 * k + 1, h->stream));
    CK(h, born::launch_snapshot_f16(old, cur, (long long)n, h->ckpt_maxw,
                                    base + 2 * k * n, h->ckpt_scale + 2 * k,
                                    h->stream));
    h->launches += 4;
    return BORN_OK;
  }
  CK(h, cudaMemcpyAsync(h->ckpt + 2 * k * n, old, n * 4,
                        cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->ckpt + (2 * k + 1) * n, cur, n * 4,
                        cudaMemcpyDeviceToDevice, h->stream));
  return BORN_OK;
}

// (old, cur) <- checkpoint k (FP32 values).
int load_ckpt(born_handle *h, size_t k, float *old, float *cur) {
  const size_t n = (size_t)h->n123;
  if (h->ckpt_storage == BORN_CKPT_F16) {
    const unsigned short *base =
        reinterpret_cast<const unsigned short *>(h->ckpt);
    CK(h, born::launch_restore_f16(base + (2 * k + 1) * n, (long long)n,
                                   h->ckpt_scale + 2 * k + 1, nullptr, cur,
                                   h->stream));
    CK(h, born::launch_restore_f16(base + 2 * k * n, (long long)n,
                                   h->ckpt_scale + 2 * k, cur, old,
                                   h->stream));
    h->launches += 2;
    return BORN_OK;
  }
  CK(h, cudaMemcpyAsync(old, h->ckpt + 2 * k * n, n * 4,
                        cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(cur, h->ckpt + (2 * k + 1) * n, n * 4,
                        cudaMemcpyDeviceToDevice, h->stream));
  return BORN_OK;
}
}  // namespace

int born_lin_forward(born_handle *h, int jt, int nt, float *traces_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->lp())
    return fail(h, BORN_ESTATE, "%s needs FP32 storage", __func__);
  if (nt < 0 || jt < 1) return fail(h, BORN_EINVAL, "nt < 0 or jt < 1");
  if (!h->have_vel2 || !h->have_refl)
    return fail(h, BORN_ESTATE, "vel2 or model perturbation not transferred");
  if (jt > h->jt_s || jt > h->jt_d)
    return fail(h, BORN_EINVAL, "jt %d exceeds the sinc tables' rows", jt);
  rc = ensure_tuned(h, born::kModeBornLin);
  if (rc) return rc;
  const size_t n = (size_t)h->n123, bytes = n * 4;
  // the background computed here is the one born_lin_adjoint checkpoints:
  // store its checkpoints on the way (two levels every ckpt_every steps)
  const int every = h->ckpt_every;
  h->ckpt_valid = false;
  if (every > 0) {
    rc = ensure_ckpt(h, 2 * (size_t)((nt + every - 1) / every));
    if (rc) return rc;
  }
  CK(h, cudaMemsetAsync(h->f0, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->f1, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->r0, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->r1, 0, bytes, h->stream));
  float *sp0 = h->f0, *sp1 = h->f1, *rp0 = h->r0, *rp1 = h->r1;
  const float scale = 1 / (float)jt;
  for (int it = 0; it < nt; ++it) {
    if (every > 0 && it % every == 0) {
      rc = store_ckpt(h, (size_t)(it / every), sp0, sp1);
      if (rc) return rc;
    }
    const int id = it / jt, ii = it - id * jt;
    StepParams p;
    base_params(h, p);
    p.a_out = sp0;
    p.b_out = rp0;
    p.pa = point_view(h->src, id, ii, h->tab_s, scale, true);
    p.pb = point_view(h->rec, id, ii, h->tab_d, 0.f, true);
    const void *cen[born::kNumCentre] = {sp0, rp0, h->vel2, nullptr,
                                          h->refl};
    rc = launch(h, born::kModeBornLin, true, true, sp1, rp1, cen, p);
    if (!rc) rc = poll_error(h, it);
    if (rc) return rc;
    std::swap(sp0, sp1);
    std::swap(rp0, rp1);
  }
  if (every > 0) {
    h->ckpt_valid = true;
    h->ckpt_gen = h->bg_gen;
    h->ckpt_jt = jt;
    h->ckpt_nt = nt;
    h->ckpt_interval = every;
    h->ckpt_kind = h->ckpt_storage;
  }
  if (traces_out) {
    CK(h, cudaMemcpyAsync(traces_out, h->rec.traces,
                          (size_t)h->rec.npts * h->rec.nt * 4,
                          cudaMemcpyDeviceToHost, h->stream));
    return check_device_error(h);
  }
  return BORN_OK;
}


int born_lin_adjoint(born_handle *h, int jt, int nt, int interval,
                     float *model_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->lp())
    return fail(h, BORN_ESTATE, "%s needs FP32 storage", __func__);
  if (nt < 1 || jt < 1 || interval < 1)
    return fail(h, BORN_EINVAL, "nt, jt and interval must be >= 1");
  if (!h->have_vel2) return fail(h, BORN_ESTATE, "vel2 not transferred");
  if (jt > h->jt_s || jt > h->jt_d)
    return fail(h, BORN_EINVAL, "jt %d exceeds the sinc tables' rows", jt);
  rc = ensure_tuned(h, born::kModeModel);
  if (!rc) rc = ensure_tuned(h, born::kModeBornAdj);
  if (rc) return rc;
  const size_t n = (size_t)h->n123, bytes = n * 4;
  const int nseg = (nt + interval - 1) / interval;
  rc = ensure_ckpt(h, 2 * (size_t)nseg);
  if (!rc) rc = ensure_levels(h, &h->gbuf, &h->gbuf_levels, (size_t)interval);
  if (rc) return rc;
  const float scale = 1 / (float)jt;
  // optional phase timing: one event at every phase boundary on the stream
  PhaseEvents pe(h, h->time_phases ? 2 * nseg + 3 : 0);
  rc = pe.record();
  if (rc) return rc;
  auto model_step = [&](float *sp0, float *sp1, int it, float *g) {
    const int id = it / jt, ii = it - id * jt;
    StepParams p;
    base_params(h, p);
    p.a_out = sp0;
    p.g_out = g;
    p.pa = point_view(h->src, id, ii, h->tab_s, scale, true);
    p.pb = point_view(h->rec, id, ii, h->tab_d, 0.f, false);
    const void *cen[born::kNumCentre] = {sp0, nullptr, h->vel2, nullptr,
                                          nullptr};
    return launch(h, born::kModeModel, true, false, sp1, nullptr, cen, p);
  };
  // forward sweep of the background, checkpointing (old, cur) per segment,
  // unless the checkpoints of this background are already there (left by
  // born_lin_forward or an earlier adjoint)
  const bool have_ckpt = h->ckpt_valid && h->ckpt_gen == h->bg_gen &&
                         h->ckpt_jt == jt && h->ckpt_nt == nt &&
                         h->ckpt_interval == interval &&
                         h->ckpt_kind == h->ckpt_storage;
  h->ckpt_reused = have_ckpt;
  if (!have_ckpt) {
    h->ckpt_valid = false;
    CK(h, cudaMemsetAsync(h->f0, 0, bytes, h->stream));
    CK(h, cudaMemsetAsync(h->f1, 0, bytes, h->stream));
    float *sp0 = h->f0, *sp1 = h->f1;
    for (int it = 0; it < nt; ++it) {
      if (it % interval == 0) {
        rc = store_ckpt(h, (size_t)(it / interval), sp0, sp1);
        if (rc) return rc;
      }
      rc = model_step(sp0, sp1, it, nullptr);
      if (!rc) rc = poll_error(h, it);
      if (rc) return rc;
      std::swap(sp0, sp1);
    }
    h->ckpt_valid = true;
    h->ckpt_gen = h->bg_gen;
    h->ckpt_jt = jt;
    h->ckpt_nt = nt;
    h->ckpt_interval = interval;
    h->ckpt_kind = h->ckpt_storage;
  }
  rc = pe.record();
  if (rc) return rc;
  // reverse sweep
  CK(h, cudaMemsetAsync(h->r0, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->r1, 0, bytes, h->stream));
  CK(h, cudaMemsetAsync(h->img, 0, bytes, h->stream));
  float *wp0 = h->r0, *wp1 = h->r1;
  int steps = 0;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int t0 = seg * interval, t1 = std::min(nt, t0 + interval);
    float *a0 = h->f0, *a1 = h->f1;
    rc = load_ckpt(h, (size_t)seg, a0, a1);
    if (rc) return rc;
    for (int it = t0; it < t1; ++it) {
      rc = model_step(a0, a1, it, h->gbuf + (size_t)(it - t0) * n);
      if (!rc) rc = poll_error(h, steps++);
      if (rc) return rc;
      std::swap(a0, a1);
    }
    rc = pe.record();
    if (rc) return rc;
    for (int it = t1 - 1; it >= t0; --it) {
      const int id = it / jt, ii = it - id * jt;
      StepParams p;
      base_params(h, p);
      p.a_out = wp0;
      p.img_out = h->img;
      p.pa = point_view(h->rec, id, ii, h->tab_d, 1.f, true);
      const float *g = h->gbuf + (size_t)(it - t0) * n;
      const void *cen[born::kNumCentre] = {wp0, g, h->vel2, nullptr, h->img};
      rc = launch(h, born::kModeBornAdj, true, false, wp1, nullptr, cen, p);
      if (!rc) rc = poll_error(h, steps++);
      if (rc) return rc;
      std::swap(wp0, wp1);
    }
    rc = pe.record();
    if (rc) return rc;
  }
  CK(h, born::launch_divide(h->img, h->vel2, h->img, h->n123, h->stream));
  h->launches++;
  rc = pe.record();
  if (!rc && h->time_phases) {
    // events: start, end of sweep, then (recompute end, reverse end) per
    // segment, then the end of the division
    float ms[4] = {0.f, 0.f, 0.f, 0.f};
    rc = pe.elapsed(0, 1, &ms[0]);
    for (int k = 0; !rc && k < nseg; ++k) {
      float a = 0.f, b = 0.f;
      rc = pe.elapsed(1 + 2 * k, 2 + 2 * k, &a);
      if (!rc) rc = pe.elapsed(2 + 2 * k, 3 + 2 * k, &b);
      ms[1] += a;
      ms[2] += b;
    }
    if (!rc) rc = pe.elapsed(2 * nseg + 1, 2 * nseg + 2, &ms[3]);
    for (int k = 0; k < 4; ++k) h->phase_ms[k] = ms[k];
  }
  if (rc) return rc;
  if (model_out) {
    CK(h, cudaMemcpyAsync(model_out, h->img, bytes, cudaMemcpyDeviceToHost,
                          h->stream));
    return check_device_error(h);
  }
  return BORN_OK;
}

int born_get_image(born_handle *h, float *img_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (!img_out) return fail(h, BORN_EINVAL, "null output");
  CK(h, cudaMemcpyAsync(img_out, h->img, (size_t)h->n123 * 4,
                        cudaMemcpyDeviceToHost, h->stream));
  return check_device_error(h);
}

float *born_image_device(born_handle *h) {
  return (h && h->have_space) ? h->img : nullptr;
}

int born_get_traces(born_handle *h, float *out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (!out) return fail(h, BORN_EINVAL, "null output");
  if (h->rec.npts)
    CK(h, cudaMemcpyAsync(out, h->rec.traces,
                          (size_t)h->rec.npts * h->rec.nt * 4,
                          cudaMemcpyDeviceToHost, h->stream));
  return check_device_error(h);
}

int born_get_source_levels(born_handle *h, float *p0_out, float *p1_out) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->lp())
    return fail(h, BORN_ESTATE, "%s needs FP32 storage", __func__);
  const size_t bytes = (size_t)h->n123 * 4;
  if (p0_out) CK(h, cudaMemcpyAsync(p0_out, h->s0, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (p1_out) CK(h, cudaMemcpyAsync(p1_out, h->s1, bytes, cudaMemcpyDeviceToHost, h->stream));
  return check_device_error(h);
}

int born_set_source_levels(born_handle *h, const float *p0, const float *p1) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->lp())
    return fail(h, BORN_ESTATE, "%s needs FP32 storage", __func__);
  if (!p0 || !p1) return fail(h, BORN_EINVAL, "null source level");
  const size_t bytes = (size_t)h->n123 * 4;
  CK(h, cudaMemcpyAsync(h->s0, p0, bytes, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->s1, p1, bytes, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->src_levels_valid = true;
  return BORN_OK;
}

int born_zero_traces(born_handle *h) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (h->rec.npts)
    CK(h, cudaMemsetAsync(h->rec.traces, 0, (size_t)h->rec.npts * h->rec.nt * 4,
                          h->stream));
  return BORN_OK;
}

int born_synchronize(born_handle *h) {
  if (!h) return BORN_EINVAL;
  int rc = set_device(h);
  if (rc) return rc;
  return check_device_error(h);
}

int born_selftest_wait_timeout(born_handle *h) {
  if (!h) return BORN_EINVAL;
  int rc = set_device(h);
  if (rc) return rc;
  rc = check_device_error(h);  // start from a clear error word
  if (rc) return rc;
  CK(h, born::launch_wait_timeout_probe(h->err_dev, h->stream));
  h->launches++;
  return check_device_error(h);  // BORN_ETIMEOUT, and the word is cleared
}

int born_tile_config_count(void) { return born::tile_cfg_count(); }

int born_set_host_prewarm(born_handle *h, int enable) {
  if (!h) return BORN_EINVAL;
  h->prewarm = enable != 0;
  return BORN_OK;
}

long long born_host_prewarm_count(const born_handle *h) {
  return h ? h->prewarm_copies : 0;
}

int born_autotune(born_handle *h, int enable) {
  int rc = check_ready(h);
  if (rc) return rc;
  h->autotune = enable != 0;
  h->reset_tuning();
  if (!enable) return BORN_OK;
  const int modes[] = {kModeSource, kModeForward, kModeAdjoint,
                       born::kModeModel, born::kModeBornLin,
                       born::kModeBornAdj};
  for (int m : modes) {
    if (h->lp() && m > kModeAdjoint) continue;
    rc = tune_mode(h, m);
    if (rc) return rc;
  }
  return BORN_OK;
}

int born_tuned_config(const born_handle *h, int mode, int *cfg,
                      float *ms_per_launch) {
  if (!h || mode < 0 || mode > 5) return BORN_EINVAL;
  if (cfg)
    *cfg = h->tile_cfg >= 0 ? h->tile_cfg
                            : h->tuned_cfg[h->storage_for(mode)][mode];
  if (ms_per_launch) *ms_per_launch = h->tuned_ms[h->storage_for(mode)][mode];
  return BORN_OK;
}

int born_tuned_zseg(born_handle *h, int mode) {
  if (!h || mode < 0 || mode > 5) return BORN_EINVAL;
  if (!h->have_space) return fail(h, BORN_ESTATE, "no grid");
  int cfg, zseg, tx, ty;
  const bool pb = mode == kModeForward || mode == kModeAdjoint ||
                  mode == born::kModeBornLin;
  pick_tiling(h, mode, true, pb, &cfg, &zseg, &tx, &ty);
  return zseg;
}

int born_loop_tile_ms(const born_handle *h, int mode, float *ms, int n) {
  if (!h || mode < 0 || mode > 5 || !ms || n < 0) return BORN_EINVAL;
  for (int c = 0; c < n; ++c)
    ms[c] = c < born_handle::kMaxTileCfgs ? h->loop_ms[h->storage_for(mode)][mode][c]
                                          : 0.f;
  return BORN_OK;
}

int born_set_checkpoint_storage(born_handle *h, int storage) {
  if (!h) return BORN_EINVAL;
  if (storage != BORN_CKPT_F32 && storage != BORN_CKPT_F16)
    return fail(h, BORN_EINVAL, "unknown checkpoint storage %d", storage);
  if (storage != h->ckpt_storage) {
    h->ckpt_storage = storage;
    h->ckpt_valid = false;
  }
  return BORN_OK;
}

int born_set_checkpoint_interval(born_handle *h, int interval) {
  if (!h) return BORN_EINVAL;
  if (interval < 0) return fail(h, BORN_EINVAL, "checkpoint interval < 0");
  h->ckpt_every = interval;
  return BORN_OK;
}

int born_checkpoints_reused(const born_handle *h) {
  return h ? (h->ckpt_reused ? 1 : 0) : BORN_EINVAL;
}

int born_time_phases(born_handle *h, int enable) {
  if (!h) return BORN_EINVAL;
  h->time_phases = enable != 0;
  return BORN_OK;
}

int born_phase_times(const born_handle *h, float *ms, int n) {
  if (!h || !ms || n < 0) return BORN_EINVAL;
  for (int k = 0; k < n && k < 4; ++k) ms[k] = h->phase_ms[k];
  return BORN_OK;
}

int born_set_launch_overlap(born_handle *h, int enable) {
  if (!h) return BORN_EINVAL;
  h->overlap = enable != 0;
  return BORN_OK;
}

int born_set_tiling(born_handle *h, int cfg, int zseg) {
  if (!h) return BORN_EINVAL;
  if (cfg < -1 || cfg >= born::tile_cfg_count() || zseg < 0)
    return fail(h, BORN_EINVAL, "bad tiling (%d, %d)", cfg, zseg);
  h->tile_cfg = cfg;
  h->zseg = zseg;
  return BORN_OK;
}

int born_set_storage(born_handle *h, int storage) {
  int rc = check_ready(h);
  if (rc) return rc;
  if (storage != BORN_STORE_F32 && storage != BORN_STORE_BF16 &&
      storage != BORN_STORE_F16 && storage != BORN_STORE_F32_FUSED &&
      storage != BORN_STORE_F32_EXACT)
    return fail(h, BORN_EINVAL, "unknown storage %d", storage);
  if (born::storage_16bit(storage) && h->n1 % 8 != 0)
    return fail(h, BORN_EINVAL,
                "16-bit storage needs nx %% 8 == 0 (rows of 16-byte multiples)");
  CK(h, cudaStreamSynchronize(h->stream));
  if (storage != h->storage) {
    h->storage = storage;
    h->src_levels_valid = false;  // the levels change representation
    h->generation++;
    const size_t bytes = (size_t)h->n123 * 4;
    float *lv[] = {h->s0, h->s1, h->r0, h->r1, h->f0, h->f1};
    for (float *b : lv) CK(h, cudaMemsetAsync(b, 0, bytes, h->stream));
    for (int b = 0; b < kNumLevelBufs; ++b) {
      CK(h, born::launch_level_reset(h->lv_dev, b, h->stream));
      h->wr[b] = 0;
    }
    CK(h, cudaStreamSynchronize(h->stream));
  }
  return BORN_OK;
}

int born_get_storage(const born_handle *h) {
  return h ? h->storage : BORN_STORE_F32;
}

long long born_kernel_launches(const born_handle *h) {
  return h ? h->launches : 0;
}

void *born_stream(born_handle *h) { return h ? (void *)h->stream : nullptr; }

// ===========================================================================
// Reference-compatible entry points over a default handle
namespace {
born_handle *g_default = nullptr;
int g_status = BORN_OK;
std::string g_error;
int g_ngpus = 1;

void record(int rc) {
  g_status = rc;
  if (rc == BORN_OK)
    g_error.clear();
  else
    g_error = g_default ? g_default->err : std::string("no device handle");
}

born_handle *dflt() {
  if (!g_default) {
    int dev = 0;
    cudaGetDevice(&dev);
    int rc = born_create(dev, &g_default);
    if (rc) {
      g_default = nullptr;
      record(rc);
    }
  }
  return g_default;
}
}  // namespace

int born_default_status(void) { return g_status; }
const char *born_default_error(void) { return g_error.c_str(); }
born_handle *born_default_handle(void) { return dflt(); }

void setup_cuda(int ngpus) {
  g_ngpus = ngpus;
  record(dflt() ? BORN_OK : BORN_ENODEV);
}

void create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b,
                      float bc_b_y, int nx, int ny, int nz) {
  born_handle *h = dflt();
  record(h ? born_create_space(h, d1, d2, d3, bc_a, bc_b, bc_b_y, nx, ny, nz)
           : BORN_ENODEV);
}

void transfer_sinc_table_s(int nsinc, int ns, float *tables) {
  born_handle *h = dflt();
  record(h ? born_set_sinc_table(h, 0, nsinc, ns, tables) : BORN_ENODEV);
}

void transfer_sinc_table_d(int nsinc, int ns, float *tabled) {
  born_handle *h = dflt();
  record(h ? born_set_sinc_table(h, 1, nsinc, ns, tabled) : BORN_ENODEV);
}

void transfer_source_func(int npts, int nt, int *locs, float *vals) {
  born_handle *h = dflt();
  record(h ? born_set_source_func(h, npts, nt, locs, vals) : BORN_ENODEV);
}

void load_source(int it) { (void)it; }

void transfer_receiver_func(int nx, int ny, int nt, int *locs, float *vals) {
  born_handle *h = dflt();
  record(h ? born_set_receiver_func(h, nx, ny, nt, locs, vals) : BORN_ENODEV);
}

void transfer_vel_func1(int nx, int ny, int nz, float *vel) {
  born_handle *h = dflt();
  record(h ? born_set_velocity(h, 1, nx, ny, nz, vel) : BORN_ENODEV);
}

void transfer_vel_func2(int nx, int ny, int nz, float *vel) {
  born_handle *h = dflt();
  record(h ? born_set_velocity(h, 2, nx, ny, nz, vel) : BORN_ENODEV);
}

void source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0,
                 float *p1, int jt, int npts, int nt) {
  (void)damp;
  (void)npts;
  born_handle *h = dflt();
  if (!h) return record(BORN_ENODEV);
  if (h->have_space && (n1 != h->n1 || n2 != h->n2 || n3 != h->n3))
    return record(fail(h, BORN_EINVAL, "source_prop: grid mismatch"));
  int rc = born_source_prop(h, jt, nt, get_last ? p0 : nullptr,
                            get_last ? p1 : nullptr);
  if (rc == BORN_OK && !get_last) {
    // the reference's GPU path keeps the levels on the device and ignores
    // the host arrays (gpu_funcs_3d.cu:409-427): they still name them
    h->host_p0 = p0;
    h->host_p1 = p1;
  }
  record(rc);
}

void rtm_adjoint(int n1, int n2, int n3, int j, float *p0_s_cpu,
                 float *p1_s_cpu, float *img, int npts, int nt) {
  (void)npts;
  born_handle *h = dflt();
  if (!h) return record(BORN_ENODEV);
  if (h->have_space && (n1 != h->n1 || n2 != h->n2 || n3 != h->n3))
    return record(fail(h, BORN_EINVAL, "rtm_adjoint: grid mismatch"));
  if (!p0_s_cpu || !p1_s_cpu)  // the device-resident levels as they are
    return record(born_rtm_adjoint(h, j, nt, 0, img));
  record(born_rtm_adjoint_host(h, j, nt, p0_s_cpu, p1_s_cpu, img));
}

void set_ntblock(int nt) {
  born_handle *h = dflt();
  if (h) h->ntblock = nt;
  record(h ? BORN_OK : BORN_ENODEV);
}

void rtm_forward(int n1, int n2, int n3, int jt, float *img, float *dat,
                 int npts_src, int nt, int nt_big, int nx, int ny) {
  (void)npts_src;
  born_handle *h = dflt();
  if (!h) return record(BORN_ENODEV);
  if (h->have_space && (n1 != h->n1 || n2 != h->n2 || n3 != h->n3))
    return record(fail(h, BORN_EINVAL, "rtm_forward: grid mismatch"));
  if (h->rec.npts != nx * ny || h->rec.nt != nt_big)
    return record(fail(h, BORN_EINVAL,
                       "rtm_forward: receiver geometry differs from the "
                       "transferred one"));
  if (img) {
    int rc = born_set_reflectivity(h, img);
    if (rc) return record(rc);
  }
  record(born_rtm_forward(h, jt, nt, dat));
}

}  // extern "C"
