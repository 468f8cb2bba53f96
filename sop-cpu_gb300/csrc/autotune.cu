// Autotuner of the batched step: launch shape (step-kernel block size, beads
// per work item, shared-memory stage limit) for the whole engine, and list
// parameters (skin, cell edge) per replica size bucket.
//
// Every trial is a run of real steps: the tuner opens one run window over all
// its trials for every active replica, so sop_autotune advances the replicas
// exactly as one sop_run of the same number of steps would.  Launch-shape
// knobs leave every per-bead computation unchanged (trajectories stay
// bit-identical).  Skin and cell edge apply to replicas in skin mode only;
// pair sets stay exact (the pair filter is exact at every step) but rows are
// rebuilt in another order, so float summation order, and thus rounding, can
// change.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

using namespace sop;

#define TK(call)                                      \
  do {                                                \
    cudaError_t err_ = (call);                        \
    if (err_ != cudaSuccess) return SOP_ERR_CUDA;     \
  } while (0)

namespace {

struct Shape {
  int threads, chunk, stage, slice;
};

struct Bucket {
  int lo, hi;
  std::vector<int> ids;  // skin-mode replicas of this size range
};

struct Tuner {
  sop_engine* e;
  int S;                 // steps per timed trial (each trial also runs S warm-up steps)
  int64_t left;          // steps still to run in the open window (excluding the final step)
  std::string log;

  void note(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    log += buf;
  }

  // S warm-up steps, then S timed steps: milliseconds per step
  int trial(double* ms_per_step) {
    float ms = 0;
    int rc = run_steps(e, S, nullptr);
    if (rc) return rc;
    rc = run_steps(e, S, &ms);
    if (rc) return rc;
    left -= 2 * (int64_t)S;
    *ms_per_step = ms / S;
    return SOP_OK;
  }
};

int fetch_reps(sop_engine* e, std::vector<RepDev>& out) {
  out.resize(e->cfg.max_replicas);
  TK(cudaMemcpyAsync(out.data(), e->A.rep, sizeof(RepDev) * out.size(), cudaMemcpyDeviceToHost,
                     e->stream));
  TK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

// Give the bucket's replicas a new skin and cell edge and rebuild their lists
// at once (one forced build over all of them); rows that overflow grow.
int set_lists(sop_engine* e, const std::vector<int>& ids, double skin, double edge) {
  if (ids.empty()) return SOP_OK;
  std::vector<RepDev> reps;
  int rc = fetch_reps(e, reps);
  if (rc) return rc;
  for (int r : ids) {
    RepDev& d = reps[r];
    d.skin = (float)skin;
    d.half_skin2 = (float)(0.25 * skin * skin);
    d.cell_edge = (float)edge;
    e->reps[r].params.skin = skin;
    e->reps[r].params.cell_edge = edge;
    TK(cudaMemcpyAsync(e->A.rep + r, &reps[r], sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
  }
  TK(cudaMemcpyAsync(e->d_pack_ids, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice,
                     e->stream));
  TK(launch_prologue(e->A, e->d_pack_ids, (int)ids.size(), nullptr, 1, -1,
                     2 * e->prop.multiProcessorCount, e->stream));
  e->launches += kPrologueLaunches;
  rc = fetch_reps(e, reps);
  if (rc) return rc;
  for (int r : ids) {
    if (!(reps[r].status & SOP_ST_LIST_OVERFLOW)) continue;
    rc = grow_rows(e, r, reps[r].max_row);
    if (rc) return rc;
    rc = rebuild_fit(e, r, reps[r].mode);
    if (rc) return rc;
  }
  return SOP_OK;
}

}  // namespace

extern "C" int sop_autotune_ex(sop_engine* e, int steps_per_trial, int what, char* report,
                               int report_cap) {
  if (!e || steps_per_trial <= 0 || !(what & (SOP_TUNE_SHAPE | SOP_TUNE_LISTS))) return SOP_ERR_ARG;
  TK(cudaSetDevice(e->cfg.device));
  int rc = refresh_layout(e);
  if (rc) return rc;
  if (e->active.empty()) return SOP_ERR_STATE;

  // candidates
  const int stage_max = std::min<int>(kStageMax, ((int)e->prop.sharedMemPerBlockOptin - 1024) / 32);
  std::vector<int> stages, chunks = {64, 128, 256, 512}, threads = {64, 128, 256},
                   slices = {16, 32, 64, 128};
  for (int s : {-1, 1024, 2048, 4096})
    if (s <= stage_max) stages.push_back(s);
  const std::vector<double> skins = {1.0, 1.5, 2.0, 3.0, 4.0};
  const std::vector<double> edge_pads = {0.0, 2.0, 4.0};
  std::vector<Bucket> buckets = {{1, 256, {}}, {256, 1024, {}}, {1024, 4096, {}}, {4096, 1 << 30, {}}};
  if (what & SOP_TUNE_LISTS) {
    for (int r : e->active) {
      const Replica& R = e->reps[r];
      if (R.params.list_mode != SOP_LIST_SKIN) continue;
      for (auto& b : buckets)
        if (R.n >= b.lo && R.n < b.hi) b.ids.push_back(r);
    }
  }
  buckets.erase(std::remove_if(buckets.begin(), buckets.end(), [](const Bucket& b) { return b.ids.empty(); }),
                buckets.end());

  // trials: one baseline, then every other value of each knob in turn
  int ntrials = 1;
  if (what & SOP_TUNE_SHAPE)
    ntrials += (int)(stages.size() + chunks.size() + threads.size() + slices.size());
  for (size_t b = 0; b < buckets.size(); b++) ntrials += (int)(skins.size() + edge_pads.size());
  Tuner T{e, steps_per_trial, (int64_t)ntrials * 2 * steps_per_trial, std::string()};
  const int64_t total = T.left;
  rc = begin_all(e, total);
  if (rc) return rc;

  Shape cur{e->cfg.block_threads, e->cfg.chunk_beads, e->cfg.stage_limit > 0 ? e->cfg.stage_limit : -1,
            e->cfg.build_slice_beads};
  double best = 0;
  rc = T.trial(&best);
  if (rc) return rc;
  T.note("baseline threads=%d chunk=%d stage=%d slice=%d  %.4f ms/step\n", cur.threads, cur.chunk,
         cur.stage, cur.slice, best);
  int used = 1;

  auto try_shape = [&](Shape s) -> int {
    set_launch_shape(e, s.threads, s.chunk, s.stage, s.slice);
    double ms = 0;
    int r2 = T.trial(&ms);
    if (r2) return r2;
    used++;
    T.note("shape threads=%d chunk=%d stage=%d slice=%d  %.4f ms/step\n", s.threads, s.chunk,
           s.stage, s.slice, ms);
    if (ms < best * 0.99) { best = ms; cur = s; }
    set_launch_shape(e, cur.threads, cur.chunk, cur.stage, cur.slice);
    return SOP_OK;
  };
  if (what & SOP_TUNE_SHAPE) {
    // each knob sweeps its values with the others at their best so far; a
    // knob's current value is re-timed once so the comparison is fresh
    for (int s : stages) { Shape c = cur; c.stage = s; if ((rc = try_shape(c))) return rc; }
    for (int c : chunks) { Shape x = cur; x.chunk = c; if ((rc = try_shape(x))) return rc; }
    for (int t : threads) { Shape x = cur; x.threads = t; if ((rc = try_shape(x))) return rc; }
    for (int q : slices) { Shape x = cur; x.slice = q; if ((rc = try_shape(x))) return rc; }
  }

  const FFTables& F = tables();
  const double rc_pl = 2.5 * std::max(F.sigma_rep[1][1], F.sigma_rep[2][2]);
  for (auto& b : buckets) {
    const Replica& R0 = e->reps[b.ids[0]];
    double best_skin = R0.params.skin, best_edge = R0.params.cell_edge, bms = 1e300;
    for (double s : skins) {
      rc = set_lists(e, b.ids, s, best_edge);
      if (rc == SOP_ERR_FULL) {  // longer rows than the list arena holds: not a candidate
        T.note("bucket n=[%d,%d) skin=%.1f skipped (list arena full)\n", b.lo, b.hi, s);
        if ((rc = set_lists(e, b.ids, best_skin, best_edge))) return rc;
        continue;
      }
      if (rc) return rc;
      double ms = 0;
      if ((rc = T.trial(&ms))) return rc;
      used++;
      T.note("bucket n=[%d,%d) replicas=%zu skin=%.1f edge=%.1f  %.4f ms/step\n", b.lo, b.hi,
             b.ids.size(), s, best_edge, ms);
      if (ms < bms * 0.99) { bms = ms; best_skin = s; }
    }
    for (double pad : edge_pads) {
      const double edge = pad > 0 ? rc_pl + best_skin + pad : 0.0;
      rc = set_lists(e, b.ids, best_skin, edge);
      if (rc) return rc;
      double ms = 0;
      if ((rc = T.trial(&ms))) return rc;
      used++;
      T.note("bucket n=[%d,%d) replicas=%zu skin=%.1f edge=%.1f  %.4f ms/step\n", b.lo, b.hi,
             b.ids.size(), best_skin, edge, ms);
      if (ms < bms * 0.99) { bms = ms; best_edge = edge; }
    }
    rc = set_lists(e, b.ids, best_skin, best_edge);
    if (rc) return rc;
    T.note("chosen bucket n=[%d,%d) skin=%.1f edge=%.1f\n", b.lo, b.hi, best_skin, best_edge);
  }
  // the window's remaining steps (trials that were planned but not needed) and
  // its final step (force + velocity, no move)
  float ms = 0;
  rc = run_steps(e, T.left + 1, &ms);
  if (rc) return rc;
  T.note("chosen threads=%d chunk=%d stage=%d slice=%d  %.4f ms/step; %d trials, %lld steps\n",
         cur.threads, cur.chunk, cur.stage, cur.slice, best, used, (long long)total);
  if (report && report_cap > 0) {
    std::strncpy(report, T.log.c_str(), report_cap - 1);
    report[report_cap - 1] = 0;
  }
  return SOP_OK;
}

extern "C" int sop_autotune(sop_engine* e, int steps_per_trial, char* report, int report_cap) {
  return sop_autotune_ex(e, steps_per_trial, SOP_TUNE_SHAPE | SOP_TUNE_LISTS, report, report_cap);
}
