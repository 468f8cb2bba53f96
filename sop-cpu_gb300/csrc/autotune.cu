// Autotuner of the batched step: launch shape (step strategy, stage limit,
// beads per work item, block size 64-512, lanes per bead, register budget,
// build slice, rebuild grouping) for the whole engine, and list parameters
// (skin 1-4 A, cell edge 6-12 A) per replica size bucket.
//
// Every trial is a run of real steps: the tuner opens one run window over all
// its trials for every active replica, so sop_autotune advances the replicas
// exactly as one sop_run of the same number of steps would -- bit for bit,
// whatever it chooses: every force and pair energy is an exact fixed-point
// sum of its contributions, so neither list order, build times, lane count
// nor the kernel variant moves a trajectory, and the pair filter is exact at
// every step whatever the skin or cell edge.
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

  // n warm-up steps (default S), then n timed steps: milliseconds per step
  int trial(double* ms_per_step, int n = 0) {
    NvtxRange range("autotune trial");
    if (n <= 0) n = S;
    float ms = 0;
    int rc = run_steps(e, n, nullptr);
    if (rc) return rc;
    rc = run_steps(e, n, &ms);
    if (rc) return rc;
    left -= 2 * (int64_t)n;
    *ms_per_step = ms / n;
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
  TK(launch_prologue(e->A, e->d_pack_ids, (int)ids.size(), nullptr, 1, -1, 1,
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
  std::vector<int> stages;
  for (int s : {-1, 1024, 1664, 2048, 4096})
    if (s <= stage_max) stages.push_back(s);
  struct Knob {
    const char* name;
    int LaunchShape::*field;
    std::vector<int> values;
  };
  const std::vector<Knob> knobs = {
      {"warp", &LaunchShape::strategy, {0, 1}},
      {"stage", &LaunchShape::stage, stages},
      {"chunk", &LaunchShape::chunk, {32, 64, 128, 256, 512}},
      {"threads", &LaunchShape::threads, {64, 128, 256, 512}},
      {"lanes", &LaunchShape::lanes, {1, 2, 4, 8, 16}},
      {"occ", &LaunchShape::min_blocks, {2, 3, 4}},
      {"slice", &LaunchShape::slice, {16, 32, 64, 128}},
      {"group", &LaunchShape::group_pct, {0, 30, 50, 70}},
      {"cost", &LaunchShape::item_cost, {-1, 64, 128, 256, 512}},
      {"queue", &LaunchShape::queue, {-1, 0, 2, 4, 8}},
  };
  const std::vector<double> skins = {1.0, 1.5, 2.0, 3.0, 4.0};
  // absolute cell edges (A); the build widens an edge below half the list
  // cutoff to that half, and 0 is that half exactly
  const std::vector<double> edges = {0.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0};
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

  // trials: one baseline, then every value of each knob in turn
  int ntrials = 1;
  if (what & SOP_TUNE_SHAPE)
    for (const Knob& k : knobs) ntrials += (int)k.values.size();
  // list trials span several rebuild intervals, so each lasts at least 400
  // steps; the bucket's current skin and edge are timed first, and a
  // candidate replaces them only when 2% faster
  const int SL = std::max(steps_per_trial, 400);
  int ltrials = 0;
  for (size_t b = 0; b < buckets.size(); b++) ltrials += 1 + (int)(skins.size() + edges.size());
  Tuner T{e, steps_per_trial,
          (int64_t)ntrials * 2 * steps_per_trial + (int64_t)ltrials * 2 * SL, std::string()};
  const int64_t total = T.left;
  rc = begin_all(e, total);
  if (rc) return rc;

  auto describe = [](const LaunchShape& s) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "threads=%d chunk=%d stage=%d slice=%d occ=%d warp=%d lanes=%d group=%d cost=%d queue=%d",
             s.threads, s.chunk, s.stage, s.slice, s.min_blocks, s.strategy, s.lanes, s.group_pct,
             s.item_cost, s.queue);
    return std::string(buf);
  };
  LaunchShape cur = get_launch_shape(e);
  double best = 0;
  rc = T.trial(&best);
  if (rc) return rc;
  T.note("baseline %s  %.4f ms/step\n", describe(cur).c_str(), best);
  int used = 1;
  if (what & SOP_TUNE_SHAPE) {
    // each knob sweeps its values with the others at their best so far; a
    // knob's current value is re-timed once so the comparison is fresh
    for (const Knob& k : knobs)
      for (int v : k.values) {
        LaunchShape s = cur;
        s.*(k.field) = v;
        if (!step_shape_supported(s.lanes, s.strategy, s.threads)) continue;
        set_launch_shape(e, s);
        double ms = 0;
        if ((rc = T.trial(&ms))) return rc;
        used++;
        T.note("shape %s  %.4f ms/step\n", describe(s).c_str(), ms);
        if (ms < best * 0.99) { best = ms; cur = s; }
        set_launch_shape(e, cur);
      }
  }

  for (auto& b : buckets) {
    const Replica& R0 = e->reps[b.ids[0]];
    double best_skin = R0.params.skin, best_edge = R0.params.cell_edge, bms = 1e300;
    rc = set_lists(e, b.ids, best_skin, best_edge);
    if (rc) return rc;
    if ((rc = T.trial(&bms, SL))) return rc;
    used++;
    T.note("bucket n=[%d,%d) replicas=%zu skin=%.1f edge=%.1f  %.4f ms/step (current)\n", b.lo,
           b.hi, b.ids.size(), best_skin, best_edge, bms);
    for (double s : skins) {
      if (s == best_skin) continue;
      rc = set_lists(e, b.ids, s, best_edge);
      if (rc == SOP_ERR_FULL) {  // longer rows than the list arena holds: not a candidate
        T.note("bucket n=[%d,%d) skin=%.1f skipped (list arena full)\n", b.lo, b.hi, s);
        if ((rc = set_lists(e, b.ids, best_skin, best_edge))) return rc;
        continue;
      }
      if (rc) return rc;
      double ms = 0;
      if ((rc = T.trial(&ms, SL))) return rc;
      used++;
      T.note("bucket n=[%d,%d) replicas=%zu skin=%.1f edge=%.1f  %.4f ms/step\n", b.lo, b.hi,
             b.ids.size(), s, best_edge, ms);
      if (ms < bms * 0.98) { bms = ms; best_skin = s; }
    }
    for (double edge : edges) {
      if (edge == best_edge) continue;
      rc = set_lists(e, b.ids, best_skin, edge);
      if (rc) return rc;
      double ms = 0;
      if ((rc = T.trial(&ms, SL))) return rc;
      used++;
      T.note("bucket n=[%d,%d) replicas=%zu skin=%.1f edge=%.1f  %.4f ms/step\n", b.lo, b.hi,
             b.ids.size(), best_skin, edge, ms);
      if (ms < bms * 0.98) { bms = ms; best_edge = edge; }
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
  T.note("chosen %s  %.4f ms/step; %d trials, %lld steps\n", describe(cur).c_str(), best, used,
         (long long)total);
  if (report && report_cap > 0) {
    std::strncpy(report, T.log.c_str(), report_cap - 1);
    report[report_cap - 1] = 0;
  }
  return SOP_OK;
}

extern "C" int sop_autotune(sop_engine* e, int steps_per_trial, char* report, int report_cap) {
  return sop_autotune_ex(e, steps_per_trial, SOP_TUNE_SHAPE | SOP_TUNE_LISTS, report, report_cap);
}
