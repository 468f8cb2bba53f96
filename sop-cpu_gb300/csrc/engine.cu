// Host side of the GB300 SOP engine: device memory, replica admission,
// the plain and batched step loops, reference-named operations and the C ABI
// declared in include/sop_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sop_gpu.h"
#include "engine.h"
#include "kernels.cuh"
#include "sop_common.cuh"

namespace sop {

// ---- force-field tables (global.cpp:60-92, params.cpp:281-286) ---------------

static FFTables make_tables() {
  FFTables t;
  std::memset(&t, 0, sizeof t);
  const double ca[3][3] = {{0, 0, 0}, {0, 0.7, 0.8}, {0, 0.8, 1.0}};
  const double cr[3][3] = {{0, 0, 0}, {0, 1.0, 1.0}, {0, 1.0, 1.0}};
  const double fa[3][3] = {{0, 0, 0}, {0, -12.0 * 1.0, -12.0 * 0.8}, {0, -12.0 * 0.8, -12.0 * 0.7}};
  const double fr[3][3] = {{0, 0, 0}, {0, -6.0 * 1.0, -6.0 * 1.0}, {0, -6.0 * 1.0, -6.0 * 1.0}};
  const double sr[3][3] = {{0, 0, 0}, {0, 3.8, 5.4}, {0, 5.4, 7.0}};
  const double rn[3][3] = {{0, 0, 0}, {0, 8.0, 11.0}, {0, 11.0, 14.0}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      t.coeff_att[i][j] = ca[i][j];
      t.coeff_rep[i][j] = cr[i][j];
      t.force_coeff_att[i][j] = fa[i][j];
      t.force_coeff_rep[i][j] = fr[i][j];
      t.sigma_rep[i][j] = sr[i][j];
      t.sigma_rep2[i][j] = sr[i][j] * sr[i][j];
      t.sigma_rep6[i][j] = t.sigma_rep2[i][j] * t.sigma_rep2[i][j] * t.sigma_rep2[i][j];
      t.sigma_rep12[i][j] = t.sigma_rep6[i][j] * t.sigma_rep6[i][j];
      t.rcut_nat[i][j] = rn[i][j];
      t.fca[i][j] = (float)fa[i][j];
      t.fcr[i][j] = (float)fr[i][j];
      t.s2[i][j] = (float)t.sigma_rep2[i][j];
      double rpl = 2.5 * sr[i][j];  // sop.cpp:539-540
      t.rc2_pl[i][j] = rpl * rpl;
      t.rc2_pl_f[i][j] = (float)t.rc2_pl[i][j];
      double rnl = 3.2 * sr[i][j];  // neighbor_list.cpp:97-100
      t.rc2_nl[i][j] = rnl * rnl;
    }
  return t;
}

const FFTables& tables() {
  static FFTables t = make_tables();
  return t;
}

// ---- first-fit range allocator ----------------------------------------------

bool RangeAlloc::alloc(long long n, long long align, long long* out) {
  if (n <= 0) { *out = 0; return true; }
  for (auto it = free_.begin(); it != free_.end(); ++it) {
    long long s = (it->first + align - 1) / align * align;
    long long e = it->first + it->second;
    if (s + n <= e) {
      long long fs = it->first, fe = e;
      free_.erase(it);
      if (s > fs) free_[fs] = s - fs;
      if (fe > s + n) free_[s + n] = fe - (s + n);
      *out = s;
      used_ += n;
      return true;
    }
  }
  return false;
}

void RangeAlloc::release(long long s, long long n) {
  if (n <= 0) return;
  used_ -= n;
  auto it = free_.emplace(s, n).first;
  auto nx = std::next(it);
  if (nx != free_.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    free_.erase(nx);
  }
  if (it != free_.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      free_.erase(it);
    }
  }
}

long long RangeAlloc::largest() const {
  long long m = 0;
  for (auto& kv : free_) m = std::max(m, kv.second);
  return m;
}

}  // namespace sop

using namespace sop;

#define CK(call)                                                     \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) {                                         \
      std::snprintf(g_last_error, sizeof g_last_error, "%s: %s", #call, \
                    cudaGetErrorString(e_));                         \
      return SOP_ERR_CUDA;                                           \
    }                                                                \
  } while (0)

static char g_last_error[512];

// ---- defaults -------------------------------------------------------------------

extern "C" const char* sop_version(void) { return "sop-gb300 1.0 (sm_103a)"; }

extern "C" int sop_struct_size(const char* name) {
  if (!name) return -1;
  const std::string n(name);
  if (n == "sop_params") return (int)sizeof(sop_params);
  if (n == "sop_system_desc") return (int)sizeof(sop_system_desc);
  if (n == "sop_engine_config") return (int)sizeof(sop_engine_config);
  if (n == "sop_server_config") return (int)sizeof(sop_server_config);
  if (n == "sop_request_result") return (int)sizeof(sop_request_result);
  return -1;
}

extern "C" const char* sop_status_string(int s) {
  switch (s) {
    case SOP_OK: return "ok";
    case SOP_ERR_ARG: return "bad argument";
    case SOP_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA error";
    case SOP_ERR_NOMEM: return "out of memory";
    case SOP_ERR_STATE: return "invalid state";
    case SOP_ERR_OVERFLOW: return "list or buffer overflow";
    case SOP_ERR_UNSUPPORTED: return "unsupported input";
    case SOP_ERR_NODEV: return "no CUDA device";
    case SOP_ERR_REPLICA: return "replica error status";
    case SOP_ERR_FULL: return "engine full";
    case SOP_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    case SOP_ERR_INDEX: return "an index outside its replica (checked build)";
    default: return "unknown";
  }
}

static void set_integrator(sop_params* p, double h) {
  // params.cpp:22-27 / 84-90 (set t_step)
  p->h = h;
  double halfh = h / 2.0;
  p->a1 = h * (1.0 - p->zeta * halfh);
  p->a2 = h * halfh;
  p->a3 = (1.0 - h * p->zeta / 2.0 + (h * p->zeta) * (h * p->zeta) / 4.0) / h;
  p->a4 = halfh * (1.0 - h * p->zeta / 2.0);
}

extern "C" void sop_params_default(sop_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  // params.cpp:262-400
  p->T = 0.6;
  p->zeta = 5.0e-2;
  set_integrator(p, 2.5e-3);
  p->boxl = 500.0;
  p->ncell = 55.0;
  p->lcell = p->boxl / p->ncell;
  p->k_bnd = 20.0;
  p->R0 = 2.0;
  p->sigma_ss = 3.5;
  p->epsilon_ss = 1.0;
  p->skin = 2.0;
  p->cell_edge = 0.0;
  p->pull_force = 0.0;
  p->seed = (uint64_t)(int64_t)(-101);  // set_seed(-100-run), run = 1
  p->nnlup = 50;
  p->nup = 1000;
  p->list_mode = SOP_LIST_NEIGHBOR;
  p->force_terms = SOP_TERM_ALL;
  p->precision = SOP_PREC_MIXED;
  p->pull_i = 0;
  p->pull_j = -1;
  p->dynamics = SOP_DYN_UNDERDAMPED;
  p->a5 = p->h / p->zeta;  // params.cpp:392
}

extern "C" void sop_engine_config_default(sop_engine_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof *c);
  c->device = 0;
  c->max_beads = 1 << 21;
  c->max_replicas = 4096;
  c->max_list_entries = (int64_t)(1 << 21) * 64;
  c->block_threads = 256;
  c->lanes_per_bead = 2;
  c->graph_steps = 20;
  c->stage_limit = 1664;  // 52 KB of staging: four step CTAs per SM
  c->chunk_beads = 128;
  c->build_slice_beads = kSliceBeads;
  c->step_min_blocks = 4;
  c->group_rebuild_pct = 50;
  c->queue_wait_ns = kDefaultWaitNs;
  c->stage_wait_ns = kDefaultWaitNs;
  c->item_cost_beads = 512;  // measured on the 512-replica mix: 71.6 -> 68.5 us per k_step
}

// ---- engine lifetime ------------------------------------------------------------

template <class T>
static cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

// Device and host resources of a new engine (e->cfg already validated).  On
// failure the caller destroys the partly built engine, which frees what was
// made (every pointer starts null).
static int engine_init(sop_engine* e) {
  const sop_engine_config& cfg = e->cfg;
  CK(cudaSetDevice(cfg.device));
  CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  CK(cudaGetDeviceProperties(&e->prop, cfg.device));
  const long long cap = cfg.max_beads;
  const long long lcap = cfg.max_list_entries;
  const long long ecap = cap * 24;  // native / bond / angle / exclusion entries
  e->cap = cap;
  DevArrays& A = e->A;
  std::memset(&A, 0, sizeof A);
  A.cap = cap;
  for (int b = 0; b < 2; b++) {
    CK(dalloc(&A.X[b], 3 * cap));
    CK(dalloc(&A.stage[b], 2 * cap));
  }
  CK(dalloc(&A.incr, 3 * cap));
  CK(dalloc(&A.incr64, 3 * cap));
  CK(cudaMemsetAsync(A.incr64, 0, 3 * cap * sizeof(double), e->stream));
  CK(dalloc(&A.vel, 3 * cap));
  CK(dalloc(&A.force, 3 * cap));
  CK(dalloc(&A.xb, cap));
  CK(dalloc(&A.topo, cap));
  CK(dalloc(&A.exc_rng, cap));
  CK(dalloc(&A.nl_cnt, cap));
  CK(dalloc(&A.nl_near, cap));
  CK(dalloc(&A.nl, lcap));
  CK(dalloc(&A.nat, ecap));
  CK(dalloc(&A.nat_r0, ecap));
  CK(dalloc(&A.bnd, cap * 4));
  CK(dalloc(&A.bnd_r0, cap * 4));
  CK(dalloc(&A.ang, cap * 4));
  CK(dalloc(&A.exc, ecap));
  CK(dalloc(&A.rep, cfg.max_replicas));
  e->pairs_cap = 1 << 22;
  CK(dalloc(&A.pairs_out, e->pairs_cap));
  CK(dalloc(&A.pairs_cnt, 1));
  CK(dalloc(&A.err, 1));
  // {next item, finished warps, any_rebuild, prep flags (3)}
  CK(dalloc(&A.step_ctr, 6));
  CK(cudaMemsetAsync(A.step_ctr, 0, 6 * sizeof(int), e->stream));
  A.any_rebuild = A.step_ctr + 2;
  A.prep_flag = A.step_ctr + 3;
  // grouped skin rebuilds: replicas past this fraction of their trigger
  // distance rebuild together with one that must (0 = off)
  A.group_frac2 = cfg.group_rebuild_pct > 0
                      ? (float)(0.01 * cfg.group_rebuild_pct * 0.01 * cfg.group_rebuild_pct)
                      : 4.0f;
  CK(cudaMemsetAsync(A.err, 0, sizeof(int), e->stream));
  A.queue_wait_ns = cfg.queue_wait_ns;
  A.row_bands = cfg.row_bands >= 0 ? 1 : 0;
  A.stage_wait_ns = cfg.stage_wait_ns;
  A.publish_delay_ns = 0;
  A.skip_stage_copy = 0;
  // unit queue: every replica may queue all its build slices plus two units
  A.slice_beads = cfg.build_slice_beads;
  // every replica may queue all its build slices (at the smallest slice size)
  // plus an energy and an observables unit
  A.unit_cap = (int)std::min<long long>(cap / kMinSliceBeads + 3LL * cfg.max_replicas + 64, 1LL << 30);
  CK(dalloc(&A.units, A.unit_cap));
  CK(cudaMemsetAsync(A.units, 0xFF, sizeof(int4) * A.unit_cap, e->stream));  // every slot free (x = -1)
  // {queued, exited, next ticket, producers done}
  CK(dalloc(&A.unit_cnt, 4));
  A.unit_exit = A.unit_cnt + 1;
  A.unit_take = A.unit_cnt + 2;
  A.pro_done = A.unit_cnt + 3;
  CK(dalloc(&A.slice_done, cfg.max_replicas));
  CK(cudaMemsetAsync(A.unit_cnt, 0, 4 * sizeof(int), e->stream));
  A.done_cap = cfg.max_replicas;
  CK(dalloc(&A.done_list, A.done_cap));
  CK(dalloc(&A.done_cnt, 1));
  CK(cudaMemsetAsync(A.done_cnt, 0, sizeof(int), e->stream));
  CK(cudaMemsetAsync(A.slice_done, 0, sizeof(int) * cfg.max_replicas, e->stream));
  CK(cudaMemsetAsync(A.rep, 0, sizeof(RepDev) * cfg.max_replicas, e->stream));
  // cell bins of the list builds: per bead, and a cell range per replica
  const long long cellcap = 4 * cap + 4104LL * cfg.max_replicas;
  CK(dalloc(&A.bin_p, cap));
  CK(dalloc(&A.bin_sorted, cap));
  CK(dalloc(&A.bin_cell, cap));
  CK(dalloc(&A.cstart, cellcap));
  CK(dalloc(&A.ccur, cellcap));
  CK(dalloc(&A.bin_hdr, cfg.max_replicas));
  e->cells.init(cellcap);
  CK(dalloc(&e->d_ids, cfg.max_replicas + 4));
  CK(dalloc(&e->d_items, cap / 32 + cfg.max_replicas + 16));
  e->items_cap = cap / 32 + cfg.max_replicas + 16;
  CK(cudaMallocHost((void**)&e->h_rep, sizeof(RepDev)));
  CK(cudaMallocHost((void**)&e->h_reps, sizeof(RepDev) * cfg.max_replicas));
  CK(cudaMallocHost((void**)&e->h_done, sizeof(int)));
  e->beads.init(cap);
  e->lists.init(lcap);
  e->nats.init(ecap);
  e->bnds.init(cap * 4);
  e->angs.init(cap * 4);
  e->excs.init(ecap);
  e->reps.resize(cfg.max_replicas);
  upload_tables(tables(), e->stream);
  CK(cudaGetLastError());
  CK(init_kernels((int)e->prop.sharedMemPerBlockOptin, (int)e->prop.sharedMemPerMultiprocessor));
  CK(dalloc(&e->d_counts, 3));
  e->cta_first_cap = 32 * e->prop.multiProcessorCount + 1;  // any resident grid + 1
  CK(dalloc(&e->d_cta_first, e->cta_first_cap));
  // the CTA queue: up to kMaxQueueBlocks blocks per resident CTA
  e->blk_cap = kMaxQueueBlocks * (e->cta_first_cap - 1);
  CK(dalloc(&A.blk, e->blk_cap));
  CK(dalloc(&A.blk_q, 4));
  CK(cudaMemsetAsync(A.blk_q, 0, 4 * sizeof(int), e->stream));
  CK(cudaMemsetAsync(e->d_counts, 0, 3 * sizeof(int), e->stream));
  e->items64_cap = cap / 256 + cfg.max_replicas + 16;
  CK(dalloc(&e->d_items64, e->items64_cap));
  CK(dalloc(&e->d_pack_xyz, 3 * cap));
  CK(dalloc(&e->d_pack_vel, 3 * cap));
  CK(dalloc(&e->d_pack_ids, cfg.max_replicas));
  CK(dalloc(&e->d_reps_pack, cfg.max_replicas));
  // energy slices: every replica's beads in kEnergySlice slices, plus one
  // partial slice each
  e->en_part_cap = cap / kEnergySlice + cfg.max_replicas + 16;
  CK(dalloc(&A.en_part, 4 * e->en_part_cap));
  CK(dalloc(&A.en_done, cfg.max_replicas + 4));
  CK(cudaMemsetAsync(A.en_done, 0, sizeof(int) * (cfg.max_replicas + 4), e->stream));
  CK(dalloc(&e->d_en_base, cfg.max_replicas + 4));
  CK(dalloc(&e->d_pack_off, cfg.max_replicas));
  // fixed launch shapes of the batched step (so captured graphs stay valid):
  // persistent step CTAs as many as fit, staging sized by the stage limit
  e->max_staged = cfg.stage_limit > 0 ? cfg.stage_limit : 0;
  e->step_grid = step_blocks_per_sm(cfg.lanes_per_bead, cfg.step_min_blocks, cfg.step_strategy, cfg.block_threads,
                                    e->max_staged) *
                 e->prop.multiProcessorCount;
  e->pro_grid = 2 * e->prop.multiProcessorCount;  // k_prep CTAs (two per SM, all resident)
  for (int k = 0; k < 4; k++) CK(cudaEventCreate(&e->ev[k]));
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

extern "C" int sop_engine_create(const sop_engine_config* cfg_in, sop_engine** out) {
  if (!out) return SOP_ERR_ARG;
  *out = nullptr;
  sop_engine_config cfg;
  sop_engine_config_default(&cfg);
  if (cfg_in) {
    cfg.device = cfg_in->device;
    if (cfg_in->max_beads > 0) cfg.max_beads = cfg_in->max_beads;
    if (cfg_in->max_replicas > 0) cfg.max_replicas = cfg_in->max_replicas;
    if (cfg_in->max_list_entries > 0) cfg.max_list_entries = cfg_in->max_list_entries;
    if (cfg_in->block_threads > 0) cfg.block_threads = cfg_in->block_threads;
    if (cfg_in->lanes_per_bead > 0) cfg.lanes_per_bead = cfg_in->lanes_per_bead;
    if (cfg_in->graph_steps > 0) cfg.graph_steps = cfg_in->graph_steps;
    if (cfg_in->stage_limit != 0) cfg.stage_limit = cfg_in->stage_limit;
    if (cfg_in->chunk_beads > 0) cfg.chunk_beads = cfg_in->chunk_beads;
    if (cfg_in->build_slice_beads > 0) cfg.build_slice_beads = cfg_in->build_slice_beads;
    if (cfg_in->step_min_blocks > 0) cfg.step_min_blocks = cfg_in->step_min_blocks;
    if (cfg_in->step_strategy > 0) cfg.step_strategy = cfg_in->step_strategy;
    if (cfg_in->group_rebuild_pct != 0) cfg.group_rebuild_pct = cfg_in->group_rebuild_pct;
    cfg.lean_prep = cfg_in->lean_prep < 0 ? -1 : 0;
    if (cfg_in->queue_wait_ns > 0) cfg.queue_wait_ns = std::min<int64_t>(cfg_in->queue_wait_ns, kMaxWaitNs);
    if (cfg_in->stage_wait_ns > 0) cfg.stage_wait_ns = std::min<int64_t>(cfg_in->stage_wait_ns, kMaxWaitNs);
    cfg.row_bands = cfg_in->row_bands < 0 ? -1 : 0;
    if (cfg_in->item_cost_beads != 0) cfg.item_cost_beads = std::min(cfg_in->item_cost_beads, 1 << 20);
    if (cfg_in->queue_blocks != 0) cfg.queue_blocks = cfg_in->queue_blocks < 0 ? -1 : std::min(cfg_in->queue_blocks, kMaxQueueBlocks);
  }
  if (cfg.group_rebuild_pct < 0 || cfg.group_rebuild_pct >= 100) cfg.group_rebuild_pct = 0;
  if (cfg.step_strategy != 1) cfg.step_strategy = 0;
  if (cfg.step_min_blocks < 2 || cfg.step_min_blocks > 4) cfg.step_min_blocks = 3;
  if (cfg.step_strategy == 1 && cfg.step_min_blocks == 4) cfg.step_min_blocks = 3;
  if (cfg.stage_limit > kStageMax) cfg.stage_limit = kStageMax;
  if (cfg.chunk_beads < 32) cfg.chunk_beads = 32;
  if (cfg.build_slice_beads < kMinSliceBeads) cfg.build_slice_beads = kMinSliceBeads;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return SOP_ERR_NODEV;
  }
  if (cfg.device < 0 || cfg.device >= ndev) return SOP_ERR_ARG;
  int lanes = cfg.lanes_per_bead;
  if (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16) return SOP_ERR_ARG;
  if (cfg.block_threads % 32 || cfg.block_threads < 64 || cfg.block_threads > 512) return SOP_ERR_ARG;
  if (!step_shape_supported(cfg.lanes_per_bead, cfg.step_strategy, cfg.block_threads))
    return SOP_ERR_UNSUPPORTED;
  std::unique_ptr<sop_engine> e(new (std::nothrow) sop_engine());
  if (!e) return SOP_ERR_NOMEM;
  e->cfg = cfg;
  const int rc = engine_init(e.get());
  if (rc != SOP_OK) {
    sop_engine_destroy(e.release());  // frees whatever was made before the failure
    return rc;
  }
  *out = e.release();
  return SOP_OK;
}

extern "C" int sop_engine_destroy(sop_engine* e) {
  if (!e) return SOP_ERR_ARG;
  cudaSetDevice(e->cfg.device);
  cudaStreamSynchronize(e->stream);
  if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
  DevArrays& A = e->A;
  void* ptrs[] = {A.X[0], A.X[1], A.stage[0], A.stage[1], A.incr, A.incr64, A.vel, A.force, A.xb, A.topo,
                  A.exc_rng, A.nl_cnt, A.nl_near, A.nl, A.nat, A.nat_r0, A.bnd, A.bnd_r0, A.ang, A.exc,
                  A.rep, A.pairs_out, A.pairs_cnt, A.err, A.units, A.unit_cnt, A.slice_done,
                  A.done_list, A.done_cnt, e->d_ids, e->d_items, e->d_items64, e->d_counts, e->d_cta_first,
                  A.blk, A.blk_q, e->d_pack_xyz,
                  e->d_pack_vel, e->d_pack_ids, e->d_pack_off, e->d_reps_pack, e->d_en_base,
                  A.en_part, A.en_done, A.bin_p, A.bin_sorted,
                  A.bin_cell, A.cstart, A.ccur, A.bin_hdr, A.step_ctr};
  for (void* p : ptrs) cudaFree(p);
  if (e->h_rep) cudaFreeHost(e->h_rep);
  if (e->h_reps) cudaFreeHost(e->h_reps);
  if (e->h_done) cudaFreeHost(e->h_done);
  for (int k = 0; k < 4; k++) if (e->ev[k]) cudaEventDestroy(e->ev[k]);
  cudaStreamDestroy(e->stream);
  delete e;
  return SOP_OK;
}

extern "C" int sop_engine_sync(sop_engine* e) {
  if (!e) return SOP_ERR_ARG;
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

extern "C" int sop_engine_launches(const sop_engine* e, int64_t* n) {
  if (!e || !n) return SOP_ERR_ARG;
  *n = e->launches;
  return SOP_OK;
}

extern "C" int sop_engine_prep_fallbacks(sop_engine* e, int64_t* n) {
  if (!e || !n) return SOP_ERR_ARG;
  CK(cudaSetDevice(e->cfg.device));
  int v = 0;
  CK(cudaMemcpyAsync(&v, e->A.prep_flag + 2, sizeof v, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  *n = v;
  return SOP_OK;
}

// ---- replica descriptors -------------------------------------------------------

static int fill_repdev(const sop_params& p, RepDev& d) {
  d.mode = p.list_mode;
  d.terms = p.force_terms & SOP_TERM_ALL;
  d.prec = p.precision;
  d.nnlup = p.nnlup > 0 ? p.nnlup : 1;
  d.nup = p.nup;
  d.skin = (float)p.skin;
  d.cell_edge = (float)p.cell_edge;
  d.half_skin2 = (float)(0.25 * p.skin * p.skin);
  d.boxl = p.boxl;
  d.lcell = p.lcell;
  d.ncell = p.ncell;
  // the box edge as a two-float, so an image shift k boxl keeps FP32 accuracy
  d.Lh = (float)p.boxl;
  d.Ll = (float)(p.boxl - (double)d.Lh);
  d.invL = (float)(1.0 / p.boxl);
  d.a1 = (float)p.a1; d.a2 = (float)p.a2; d.a3 = (float)p.a3; d.a4 = (float)p.a4;
  d.a1d = p.a1; d.a2d = p.a2; d.a3d = p.a3; d.a4d = p.a4;
  double amp = (p.h > 0 && p.T > 0 && p.zeta > 0) ? std::sqrt(2.0 * p.T * p.zeta / p.h) : 0.0;
  d.noise_amp = (float)amp;  // random_force (energy.cpp:456)
  d.noise_amp_d = amp;
  d.pull_fd = p.pull_force;
  d.T = (float)p.T;
  if (p.T < kEpsT && p.T != 0.0) d.T = 0.0f;  // keep the sop.cpp:316 branch exact
  d.kbnd = (float)p.k_bnd;
  d.R0sq = (float)(p.R0 * p.R0);
  d.inv_R0sq = (float)(1.0 / (p.R0 * p.R0));
  d.kbnd_d = p.k_bnd;
  d.R0sq_d = p.R0 * p.R0;
  double s6 = std::pow(p.sigma_ss, 6.0);
  d.e_ang_coeff = p.epsilon_ss * s6;
  d.fang_d = 6.0 * d.e_ang_coeff;
  d.fang = (float)d.fang_d;
  d.e_bnd_coeff = p.k_bnd * (p.R0 * p.R0) / 2.0;
  d.pull_f = (float)p.pull_force;
  d.dyn = p.dynamics;
  d.a5 = (float)p.a5;
  d.a5d = p.a5;
  d.zeta_2h = (p.h > 0) ? p.zeta / (2.0 * p.h) : 0.0;
  d.seed_lo = (uint32_t)p.seed;
  d.seed_hi = (uint32_t)(p.seed >> 32);
  if (p.list_mode < SOP_LIST_NONE || p.list_mode > SOP_LIST_SKIN) return SOP_ERR_ARG;
  if (p.dynamics != SOP_DYN_UNDERDAMPED && p.dynamics != SOP_DYN_OVERDAMPED) return SOP_ERR_ARG;
  if (p.precision != SOP_PREC_MIXED && p.precision != SOP_PREC_FP64) return SOP_ERR_ARG;
  return SOP_OK;
}

// Exact count of list candidates per bead at the given positions, for sizing
// the neighbor-list rows (same predicate as the device build, FP64).
static int max_candidates(const sop_system_desc* d, const std::vector<int>& type,
                          const std::vector<int>& chain, int mode) {
  const int n = d->nbead;
  if (mode == SOP_LIST_NONE) return n;
  const double* x = d->xyz;
  const FFTables& T = tables();
  double rl = 0;
  for (int a = 1; a < 3; a++)
    for (int b = 1; b < 3; b++) {
      double r = mode == SOP_LIST_SKIN ? 2.5 * T.sigma_rep[a][b] + d->params.skin
                                       : 3.2 * T.sigma_rep[a][b];
      rl = std::max(rl, r);
    }
  double edge = mode == SOP_LIST_CELL ? d->params.lcell : rl;
  if (edge <= 0) return n;
  // flat cell grid over the bounding box (counting sort), widened if huge
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      lo[c] = std::min(lo[c], x[3 * i + c]);
      hi[c] = std::max(hi[c], x[3 * i + c]);
    }
  const double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  const double L = d->params.boxl;
  if (ext + 2.0 * rl >= 0.5 * L) {
    // minimum images apply (global.cpp:223-227): every pair, as the device
    // build of such a replica does
    auto rnd = [](double v) { return v > 0 ? std::floor(v + 0.5) : std::ceil(v - 0.5); };
    auto img = [&](double v) { return v - L * rnd(v / L); };
    const double lc = d->params.lcell, nc = d->params.ncell;
    int best = 0;
    for (int i = 0; i < n; i++) {
      int cnt = 0;
      for (int j = 0; j < n; j++) {
        if (j == i || (chain[i] == chain[j] && std::abs(i - j) <= 2)) continue;
        if (mode == SOP_LIST_CELL) {
          bool adj = true;
          for (int c = 0; c < 3; c++) {
            double cd = std::floor(x[3 * i + c] / lc) - std::floor(x[3 * j + c] / lc);
            cd -= nc * rnd(cd / nc);
            adj = adj && cd >= -1.0 && cd <= 1.0;
          }
          cnt += adj;
          continue;
        }
        const double dx = img(x[3 * j] - x[3 * i]), dy = img(x[3 * j + 1] - x[3 * i + 1]),
                     dz = img(x[3 * j + 2] - x[3 * i + 2]);
        const double r = mode == SOP_LIST_SKIN ? 2.5 * T.sigma_rep[type[i]][type[j]] + d->params.skin
                                               : 3.2 * T.sigma_rep[type[i]][type[j]];
        cnt += dx * dx + dy * dy + dz * dz < r * r * 1.01;
      }
      best = std::max(best, cnt);
    }
    return best;
  }
  long long dim[3];
  for (;;) {
    for (int c = 0; c < 3; c++) dim[c] = (long long)((hi[c] - lo[c]) / edge) + 1;
    if (dim[0] * dim[1] * dim[2] <= (1LL << 22)) break;
    edge *= 1.5;
  }
  const long long ncell = dim[0] * dim[1] * dim[2];
  std::vector<int> cx(n), cy(n), cz(n), cstart(ncell + 1, 0), sorted(n);
  for (int i = 0; i < n; i++) {
    cx[i] = std::min<long long>((long long)((x[3 * i] - lo[0]) / edge), dim[0] - 1);
    cy[i] = std::min<long long>((long long)((x[3 * i + 1] - lo[1]) / edge), dim[1] - 1);
    cz[i] = std::min<long long>((long long)((x[3 * i + 2] - lo[2]) / edge), dim[2] - 1);
    cstart[cx[i] + dim[0] * (cy[i] + dim[1] * cz[i]) + 1]++;
  }
  for (long long c = 0; c < ncell; c++) cstart[c + 1] += cstart[c];
  {
    std::vector<int> fill(cstart.begin(), cstart.end() - 1);
    for (int i = 0; i < n; i++) sorted[fill[cx[i] + dim[0] * (cy[i] + dim[1] * cz[i])]++] = i;
  }
  int best = 0;
  for (int i = 0; i < n; i++) {
    int cnt = 0;
    for (int a = -1; a <= 1; a++)
      for (int b = -1; b <= 1; b++)
        for (int c = -1; c <= 1; c++) {
          const long long xx = cx[i] + a, yy = cy[i] + b, zz = cz[i] + c;
          if (xx < 0 || yy < 0 || zz < 0 || xx >= dim[0] || yy >= dim[1] || zz >= dim[2]) continue;
          const long long cc = xx + dim[0] * (yy + dim[1] * zz);
          for (int s = cstart[cc]; s < cstart[cc + 1]; s++) {
            const int j = sorted[s];
            if (j == i) continue;
            if (chain[i] == chain[j] && std::abs(i - j) <= 2) continue;
            if (mode == SOP_LIST_CELL) { cnt++; continue; }
            double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1],
                   dz = x[3 * j + 2] - x[3 * i + 2];
            double r = mode == SOP_LIST_SKIN ? 2.5 * T.sigma_rep[type[i]][type[j]] + d->params.skin
                                             : 3.2 * T.sigma_rep[type[i]][type[j]];
            if (dx * dx + dy * dy + dz * dz < r * r) cnt++;
          }
        }
    best = std::max(best, cnt);
  }
  return best;
}

struct Topo {
  std::vector<int4> topo;
  std::vector<int2> exc_rng;
  std::vector<int4> nat;
  std::vector<double> nat_r0;
  std::vector<int4> bnd;
  std::vector<double> bnd_r0;
  std::vector<int> ang;
  std::vector<int> exc;
  std::vector<int> type, chain;
  int nnat_pairs = 0;
};

static float f32_bits_float(float f) { return f; }

static int build_topology(const sop_system_desc* d, Topo& T) {
  const int n = d->nbead;
  T.type.assign(n, 1);
  T.chain.assign(n, 0);
  for (int i = 0; i < n; i++) {
    if (d->bead_type) {
      if (d->bead_type[i] < 1 || d->bead_type[i] > 2) return SOP_ERR_UNSUPPORTED;
      T.type[i] = d->bead_type[i];
    }
    if (d->chain) {
      if (d->chain[i] < 0 || d->chain[i] >= (1 << 20)) return SOP_ERR_UNSUPPORTED;
      T.chain[i] = d->chain[i];
    }
  }
  const FFTables& F = tables();
  std::vector<std::vector<std::pair<int, double>>> nat(n), bnd(n);
  std::vector<std::vector<int>> ang(n), exc(n);
  for (int k = 0; k < d->nnat; k++) {
    int i = d->in_[k], j = d->jn[k];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) return SOP_ERR_ARG;
    // native iff r < rcut_nat (params.cpp:197); others stay non-native candidates
    if (!(d->rn[k] < F.rcut_nat[T.type[i]][T.type[j]])) continue;
    if (T.chain[i] == T.chain[j] && std::abs(i - j) <= 2) {
      // the implicit candidate set excludes |i-j|<=2 on a chain; a native there
      // is still honoured as a native pair (the vdw file may list it)
    }
    nat[i].push_back({j, d->rn[k]});
    nat[j].push_back({i, d->rn[k]});
    T.nnat_pairs++;
  }
  for (int k = 0; k < d->nbnd; k++) {
    int i = d->ib[k], j = d->jb[k];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) return SOP_ERR_ARG;
    bnd[i].push_back({j, d->r0[k]});
    bnd[j].push_back({i, d->r0[k]});
  }
  for (int k = 0; k < d->nang; k++) {
    int i = d->ia[k], j = d->ka[k];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) return SOP_ERR_ARG;
    ang[i].push_back(j);
    ang[j].push_back(i);
  }
  for (int k = 0; k < d->nexcl; k++) {
    int i = d->ie[k], j = d->je[k];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) return SOP_ERR_ARG;
    exc[i].push_back(j);
    exc[j].push_back(i);
  }
  T.topo.resize(n);
  T.exc_rng.resize(n);
  for (int i = 0; i < n; i++) {
    auto& v = nat[i];
    std::stable_sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (size_t q = 1; q < v.size(); q++)
      if (v[q].first == v[q - 1].first) return SOP_ERR_UNSUPPORTED;  // duplicate native pair
    std::sort(exc[i].begin(), exc[i].end());
    exc[i].erase(std::unique(exc[i].begin(), exc[i].end()), exc[i].end());
    if (v.size() > 0xFFFF || bnd[i].size() > 0xFF || ang[i].size() > 0xFF) return SOP_ERR_UNSUPPORTED;
    int4 t;
    t.x = (int)T.nat.size();
    t.y = (int)T.bnd.size();
    t.z = (int)T.ang.size();
    t.w = (int)v.size() | ((int)bnd[i].size() << 16) | ((int)ang[i].size() << 24);
    T.topo[i] = t;
    for (auto& pr : v) {
      // r0^2 as a two-float pair so r0^2 - d^2 keeps precision near the minimum
      double r0 = pr.second, r0sq = r0 * r0;
      float hi = (float)r0sq, lo = (float)(r0sq - (double)hi), r0f = (float)r0;
      int4 e;
      e.x = pr.first;
      std::memcpy(&e.y, &hi, 4);
      std::memcpy(&e.z, &lo, 4);
      std::memcpy(&e.w, &r0f, 4);
      T.nat.push_back(e);
      T.nat_r0.push_back(pr.second);
    }
    for (auto& pr : bnd[i]) {
      double r0 = pr.second, r0sq = r0 * r0;
      float r0f = (float)r0, hi = (float)r0sq, lo = (float)(r0sq - (double)hi);
      int4 b;
      b.x = pr.first;
      std::memcpy(&b.y, &r0f, 4);
      std::memcpy(&b.z, &hi, 4);
      std::memcpy(&b.w, &lo, 4);
      T.bnd.push_back(b);
      T.bnd_r0.push_back(r0);
    }
    for (int j : ang[i]) T.ang.push_back(j);
    T.exc_rng[i] = make_int2((int)T.exc.size(), (int)exc[i].size());
    for (int j : exc[i]) T.exc.push_back(j);
  }
  (void)f32_bits_float;
  return SOP_OK;
}

static int compute_L(const sop_system_desc* d, const Topo& T, int mode) {
  if (mode == SOP_LIST_NONE) return (d->nbead + 7) / 8 * 8 + 8;
  int m = max_candidates(d, T.type, T.chain, mode);
  int L = m + m / 2 + 32;
  return (L + 7) / 8 * 8;
}

extern "C" int sop_engine_free_bytes(const sop_engine* e, int64_t* bytes) {
  if (!e || !bytes) return SOP_ERR_ARG;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return SOP_ERR_CUDA;
  *bytes = (int64_t)fr;
  return SOP_OK;
}

template <class T>
static cudaError_t h2d(T* dst, const T* src, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  return cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

int sop::upload_positions(sop_engine* e, int r, const double* xyz, int which_bufs) {
  Replica& R = e->reps[r];
  const int n = R.n;
  const long long off = R.off, cap = e->cap;
  std::vector<double> soa(3 * (size_t)n);
  std::vector<float4> st(2 * (size_t)n);
  for (int i = 0; i < n; i++) {
    for (int c = 0; c < 3; c++) soa[(size_t)c * n + i] = xyz[3 * i + c];
    float h[3], l[3];
    for (int c = 0; c < 3; c++) split_double(xyz[3 * i + c], h[c], l[c]);
    // .w: bead type and chain id as integer bits
    st[2 * i] = make_float4(h[0], h[1], h[2], u2f((uint32_t)R.type[i]));
    st[2 * i + 1] = make_float4(l[0], l[1], l[2], u2f((uint32_t)R.chain[i]));
  }
  for (int b = 0; b < 2; b++) {
    if (!(which_bufs & (1 << b))) continue;
    for (int c = 0; c < 3; c++) CK(h2d(e->A.X[b] + c * cap + off, soa.data() + (size_t)c * n, n, e->stream));
    CK(h2d(e->A.stage[b] + 2 * off, st.data(), 2 * (size_t)n, e->stream));
  }
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

int sop::upload_velocities(sop_engine* e, int r, const double* vel) {
  Replica& R = e->reps[r];
  const int n = R.n;
  const long long off = R.off, cap = e->cap;
  std::vector<double> soa(3 * (size_t)n, 0.0);
  std::vector<float> zero(3 * (size_t)n, 0.0f);
  if (vel)
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 3; c++) soa[(size_t)c * n + i] = vel[3 * i + c];
  for (int c = 0; c < 3; c++) {
    CK(h2d(e->A.vel + c * cap + off, soa.data() + (size_t)c * n, n, e->stream));
    CK(h2d(e->A.incr + c * cap + off, zero.data() + (size_t)c * n, n, e->stream));
  }
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

// Copy the device descriptor of replica r to the host mirror and back.
int sop::get_rep(sop_engine* e, int r, RepDev* out) {
  CK(cudaMemcpyAsync(e->h_rep, e->A.rep + r, sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  *out = *e->h_rep;
  return SOP_OK;
}

int sop::put_rep(sop_engine* e, int r, const RepDev& d) {
  *e->h_rep = d;
  CK(cudaMemcpyAsync(e->A.rep + r, e->h_rep, sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

static bool live(const sop_engine* e, int r) {
  return r >= 0 && r < (int)e->reps.size() && e->reps[r].live;
}

// Build the lists of replica r from its current positions (single CTA).
int sop::build_now(sop_engine* e, int r, int mode) {
  Replica& R = e->reps[r];
  int id = r;
  CK(cudaMemcpyAsync(e->d_ids + scratch_id(e, 0), &id, sizeof(int), cudaMemcpyHostToDevice,
                     e->stream));
  const int nsl = (R.n + e->A.slice_beads - 1) / e->A.slice_beads;
  CK(launch_prologue(e->A, e->d_ids + scratch_id(e, 0), 1, nullptr, 1, mode, 1,
                     std::min(nsl, 2 * e->prop.multiProcessorCount), e->stream));
  e->launches += kPrologueLaunches;
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

// ---- admission: host preparation, then device placement -------------------------

// A system prepared on the host (topology, row length, byte count): no
// device work, so it can run while the GPU steps other replicas.
struct sop_prepared {
  Topo T;
  sop_params params{};
  int n = 0, L = 0;
  std::vector<double> xyz, vel;
  int64_t bytes = 0;
};

static int64_t replica_bytes(long long n, long long L, const Topo& T) {
  return n * (2 * 24 + 2 * 32 + 12 + 24 + 24 + 24 + 16 + 16 + 8 + 4) + n * L * 4 +
         n * (16 + 4 + 4) + (cell_capacity((int)n) + 1) * 8 + (long long)T.nat.size() * 16 +
         (long long)T.bnd.size() * 24 + (long long)T.ang.size() * 4 + (long long)T.exc.size() * 4;
}

static int prepare(const sop_system_desc* d, sop_prepared& P) {
  if (!d || d->nbead <= 0 || !d->xyz) return SOP_ERR_ARG;
  if ((d->nbnd && (!d->ib || !d->jb || !d->r0)) || (d->nang && (!d->ia || !d->ka)) ||
      (d->nnat && (!d->in_ || !d->jn || !d->rn)) || (d->nexcl && (!d->ie || !d->je)))
    return SOP_ERR_ARG;
  if (d->nbead > kMaxReplicaBeads) return SOP_ERR_UNSUPPORTED;
  for (long long q = 0; q < 3LL * d->nbead; q++)
    if (!std::isfinite(d->xyz[q])) return SOP_ERR_ARG;
  RepDev rd;
  std::memset(&rd, 0, sizeof rd);
  int rc = fill_repdev(d->params, rd);  // validates the parameters
  if (rc) return rc;
  rc = build_topology(d, P.T);
  if (rc) return rc;
  P.params = d->params;
  P.n = d->nbead;
  P.L = compute_L(d, P.T, d->params.list_mode);
  P.xyz.assign(d->xyz, d->xyz + 3 * (size_t)P.n);
  if (d->vel) P.vel.assign(d->vel, d->vel + 3 * (size_t)P.n);
  else P.vel.clear();
  P.bytes = replica_bytes(P.n, P.L, P.T);
  return SOP_OK;
}

// Queue the positions (both buffers and their staged float pairs), the
// velocities and zero increments of replica r (no synchronization: copies
// from pageable memory return once the data is staged).
static int stage_state(sop_engine* e, int r, const double* xyz, const double* vel) {
  Replica& R = e->reps[r];
  const int n = R.n;
  const long long off = R.off, cap = e->cap;
  std::vector<double> soa(3 * (size_t)n), vs(3 * (size_t)n, 0.0);
  std::vector<float> zero(3 * (size_t)n, 0.0f);
  std::vector<float4> st(2 * (size_t)n);
  for (int i = 0; i < n; i++) {
    float h[3], l[3];
    for (int c = 0; c < 3; c++) {
      soa[(size_t)c * n + i] = xyz[3 * i + c];
      if (vel) vs[(size_t)c * n + i] = vel[3 * i + c];
      split_double(xyz[3 * i + c], h[c], l[c]);
    }
    // .w: bead type and chain id as integer bits
    st[2 * i] = make_float4(h[0], h[1], h[2], u2f((uint32_t)R.type[i]));
    st[2 * i + 1] = make_float4(l[0], l[1], l[2], u2f((uint32_t)R.chain[i]));
  }
  for (int b = 0; b < 2; b++) {
    for (int c = 0; c < 3; c++) CK(h2d(e->A.X[b] + c * cap + off, soa.data() + (size_t)c * n, n, e->stream));
    CK(h2d(e->A.stage[b] + 2 * off, st.data(), 2 * (size_t)n, e->stream));
  }
  for (int c = 0; c < 3; c++) {
    CK(h2d(e->A.vel + c * cap + off, vs.data() + (size_t)c * n, n, e->stream));
    CK(h2d(e->A.incr + c * cap + off, zero.data() + (size_t)c * n, n, e->stream));
  }
  return SOP_OK;
}

// Place a prepared system into a free slot: arenas, uploads and the replica
// descriptor, all queued on the stream without a synchronization.  The
// caller builds its lists.  SOP_ERR_FULL when a slot or an arena is missing.
static int place(sop_engine* e, const sop_prepared& P, int* replica) {
  const Topo& T = P.T;
  int slot = -1;
  for (int k = 0; k < (int)e->reps.size(); k++)
    if (!e->reps[k].live) { slot = k; break; }
  if (slot < 0) return SOP_ERR_FULL;
  const int n = P.n, L = P.L;
  const long long ncell_e = cell_capacity(n) + 1;
  long long off = 0, nlb = 0, nb = 0, bb = 0, ab = 0, xb = 0, cb = 0;
  {
    // all ranges or none
    struct Want { RangeAlloc* a; long long n, align; long long* out; };
    const Want want[] = {{&e->beads, n, 8, &off},
                         {&e->lists, (long long)n * L, 8, &nlb},
                         {&e->nats, (long long)T.nat.size(), 1, &nb},
                         {&e->bnds, (long long)T.bnd.size(), 1, &bb},
                         {&e->angs, (long long)T.ang.size(), 1, &ab},
                         {&e->excs, (long long)T.exc.size(), 1, &xb},
                         {&e->cells, ncell_e, 8, &cb}};
    const int nw = (int)(sizeof want / sizeof want[0]);
    for (int k = 0; k < nw; k++) {
      if (!want[k].a->alloc(want[k].n, want[k].align, want[k].out)) {
        for (int q = 0; q < k; q++) want[q].a->release(*want[q].out, want[q].n);
        return SOP_ERR_FULL;
      }
    }
  }
  if (nb + (long long)T.nat.size() > 0x7fffffffLL) {
    e->beads.release(off, n);
    e->lists.release(nlb, (long long)n * L);
    e->nats.release(nb, (long long)T.nat.size());
    e->bnds.release(bb, (long long)T.bnd.size());
    e->angs.release(ab, (long long)T.ang.size());
    e->excs.release(xb, (long long)T.exc.size());
    e->cells.release(cb, ncell_e);
    return SOP_ERR_FULL;
  }
  Replica& R = e->reps[slot];
  R = Replica();
  R.live = true;
  R.n = n;
  R.cell_base = cb;
  R.ncell_e = ncell_e;
  R.off = off;
  R.nl_base = nlb;
  R.L = L;
  R.nat_base = nb; R.nnat_e = (long long)T.nat.size();
  R.bnd_base = bb; R.nbnd_e = (long long)T.bnd.size();
  R.ang_base = ab; R.nang_e = (long long)T.ang.size();
  R.exc_base = xb; R.nexc_e = (long long)T.exc.size();
  R.params = P.params;
  R.type = T.type;
  R.chain = T.chain;
  R.nnat_pairs = T.nnat_pairs;
  // the per-bead ranges rebased onto the arenas
  std::vector<int4> topo(T.topo);
  std::vector<int2> exc_rng(T.exc_rng);
  for (int i = 0; i < n; i++) {
    topo[i].x += (int)nb;
    topo[i].y += (int)bb;
    topo[i].z += (int)ab;
    exc_rng[i].x += (int)xb;
  }
  // host-to-device copies from pageable memory return once the data is
  // staged, so the host vectors may go out of scope right after
  CK(h2d(e->A.topo + off, topo.data(), n, e->stream));
  CK(h2d(e->A.exc_rng + off, exc_rng.data(), n, e->stream));
  CK(h2d(e->A.nat + nb, T.nat.data(), T.nat.size(), e->stream));
  CK(h2d(e->A.nat_r0 + nb, T.nat_r0.data(), T.nat_r0.size(), e->stream));
  CK(h2d(e->A.bnd + bb, T.bnd.data(), T.bnd.size(), e->stream));
  CK(h2d(e->A.bnd_r0 + bb, T.bnd_r0.data(), T.bnd_r0.size(), e->stream));
  CK(h2d(e->A.ang + ab, T.ang.data(), T.ang.size(), e->stream));
  CK(h2d(e->A.exc + xb, T.exc.data(), T.exc.size(), e->stream));
  CK(cudaMemsetAsync(e->A.nl_cnt + off, 0, sizeof(int) * n, e->stream));
  CK(cudaMemsetAsync(e->A.nl_near + off, 0, sizeof(int) * n, e->stream));
  RepDev rd;
  std::memset(&rd, 0, sizeof rd);
  fill_repdev(P.params, rd);
  rd.off = (int)off;
  rd.n = n;
  rd.type_mask = 0;
  for (int t : T.type) rd.type_mask |= 1 << t;
  rd.nl_base = nlb;
  rd.L = L;
  rd.nat_base = (int)nb; rd.bnd_base = (int)bb; rd.ang_base = (int)ab; rd.exc_base = (int)xb;
  rd.cell_base = cb;
  rd.cell_cap = (int)cell_capacity(n);
  int pi = P.params.pull_i, pj = P.params.pull_j;
  rd.pull_i = (pi >= 0 && pi < n) ? pi : 0;
  rd.pull_j = (pj >= 0 && pj < n) ? pj : n - 1;
  rd.t = 0;
  rd.cur = 0;
  rd.inlup = 1;
  rd.active = 1;
  rd.dmax2 = 3.0e38f;  // no band split of the rows until their first build
  CK(cudaMemcpyAsync(e->A.rep + slot, &rd, sizeof rd, cudaMemcpyHostToDevice, e->stream));
  int rc = stage_state(e, slot, P.xyz.data(), P.vel.empty() ? nullptr : P.vel.data());
  if (rc) return rc;
  e->layout_dirty = true;
  *replica = slot;
  return SOP_OK;
}

// Energy terms of replicas ids[0..n) (ids also on the device at d_ids): their
// slice bases, then one launch of the sliced energy kernel.
static int enqueue_energy(sop_engine* e, const int* ids, const int* d_ids, int n) {
  std::vector<int> base(n);
  long long tot = 0;
  int mx = 0;
  for (int k = 0; k < n; k++) {
    const int ns = (e->reps[ids[k]].n + kEnergySlice - 1) / kEnergySlice;
    base[k] = (int)tot;
    tot += ns;
    mx = std::max(mx, ns);
  }
  if (tot > e->en_part_cap) return SOP_ERR_STATE;  // sized for the bead capacity: never
  CK(cudaMemcpyAsync(e->d_en_base, base.data(), n * sizeof(int), cudaMemcpyHostToDevice, e->stream));
  CK(launch_energy(e->A, d_ids, e->d_en_base, n, mx, e->stream));
  e->launches++;
  return SOP_OK;
}

// Descriptors of replicas ids[0..n) packed into out[0..n) (one CTA each), so a
// batch reads back n descriptors instead of the whole table; with `clear`, each
// descriptor is zeroed after it is copied (removal).
__global__ void k_pack_reps(RepDev* rep, const int* ids, int n, RepDev* out, int clear) {
  static_assert(sizeof(RepDev) % sizeof(int) == 0, "descriptor copied as ints");
  constexpr int kWords = (int)(sizeof(RepDev) / sizeof(int));
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    int* src = reinterpret_cast<int*>(rep + ids[k]);
    int* dst = reinterpret_cast<int*>(out + k);
    for (int w = threadIdx.x; w < kWords; w += blockDim.x) dst[w] = src[w];
    if (clear) {
      __syncthreads();
      for (int w = threadIdx.x; w < kWords; w += blockDim.x) src[w] = 0;
    }
    __syncthreads();
  }
}

// Read back the descriptors of ids[0..n) (ids already in d_pack_ids) into
// h_reps[0..n); `clear` also zeroes them on the device.  Synchronizes.
static int read_packed_reps(sop_engine* e, int n, int clear, int* err) {
  k_pack_reps<<<std::min(n, 1024), 128, 0, e->stream>>>(e->A.rep, e->d_pack_ids, n, e->d_reps_pack,
                                                        clear);
  e->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(e->h_reps, e->d_reps_pack, sizeof(RepDev) * n, cudaMemcpyDeviceToHost,
                     e->stream));
  if (err) CK(cudaMemcpyAsync(err, e->A.err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

__global__ void k_begin_many(RepDev* rep, const int* ids, const long long* nsteps, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || nsteps[k] <= 0) return;
  RepDev* R = &rep[ids[k]];
  if (!R->active) return;
  R->t_end = R->t + nsteps[k];
  R->first_pending = 1;
  R->running = 1;
}

extern "C" int sop_prepare(const sop_system_desc* d, sop_prepared** out) {
  if (!out) return SOP_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<sop_prepared> P(new (std::nothrow) sop_prepared());
  if (!P) return SOP_ERR_NOMEM;
  int rc = prepare(d, *P);
  if (rc) return rc;
  *out = P.release();
  return SOP_OK;
}

extern "C" int sop_prepared_bytes(const sop_prepared* p, int64_t* bytes) {
  if (!p || !bytes) return SOP_ERR_ARG;
  *bytes = p->bytes;
  return SOP_OK;
}

extern "C" void sop_prepared_free(sop_prepared* p) { delete p; }

extern "C" int sop_system_bytes(const sop_engine* e, const sop_system_desc* d, int64_t* bytes) {
  if (!e || !d || !bytes) return SOP_ERR_ARG;
  sop_prepared P;
  int rc = prepare(d, P);
  if (rc) return rc;
  *bytes = P.bytes;
  return SOP_OK;
}

extern "C" int sop_replicas_admit(sop_engine* e, sop_prepared* const* p, const int64_t* nsteps, int n,
                                  int* ids, int* admitted) {
  NvtxRange range("admit replicas");
  if (!e || (n > 0 && (!p || !ids)) || !admitted || n < 0) return SOP_ERR_ARG;
  *admitted = 0;
  if (n == 0) return SOP_OK;
  if (e->chunk_open) return SOP_ERR_STATE;
  CK(cudaSetDevice(e->cfg.device));
  CK(cudaStreamSynchronize(e->stream));  // the id / step scratch below is reused
  // 1. places, in order, until a slot or an arena is missing
  int k = 0;
  for (; k < n; k++) {
    if (!p[k]) return SOP_ERR_ARG;
    const int rc = place(e, *p[k], &ids[k]);
    if (rc == SOP_ERR_FULL) break;
    if (rc) {  // nothing of this batch is admitted
      for (int w = 0; w < k; w++) sop_replica_remove(e, ids[w]);
      return rc;
    }
  }
  const int m = k;
  if (m == 0) return SOP_ERR_FULL;
  // 2. one list build for all of them (sop.cpp:117-125: lists at the initial positions)
  CK(cudaMemcpyAsync(e->d_pack_ids, ids, m * sizeof(int), cudaMemcpyHostToDevice, e->stream));
  CK(launch_prologue(e->A, e->d_pack_ids, m, nullptr, 1, -1, 1, e->pro_grid, e->stream));
  e->launches += kPrologueLaunches;
  int rc0 = read_packed_reps(e, m, 0, nullptr);
  if (rc0) return rc0;
  // 3. rows longer than estimated grow (rare), then the run windows open
  std::vector<int> grow_row(m, -1);  // h_reps is reused by the calls below
  for (int q = 0; q < m; q++)
    if (e->h_reps[q].status & SOP_ST_LIST_OVERFLOW) grow_row[q] = e->h_reps[q].max_row;
  for (int q = 0; q < m; q++) {
    if (grow_row[q] < 0) continue;
    int rc = grow_rows(e, ids[q], grow_row[q]);
    if (rc == SOP_OK) rc = rebuild_fit(e, ids[q], e->reps[ids[q]].params.list_mode);
    if (rc) {  // no room for its rows: nothing of this batch is admitted
      for (int w = 0; w < m; w++) sop_replica_remove(e, ids[w]);
      return rc;
    }
  }
  if (nsteps) {
    std::vector<long long> ns(nsteps, nsteps + m);
    CK(cudaMemcpyAsync(e->d_pack_off, ns.data(), m * sizeof(long long), cudaMemcpyHostToDevice,
                       e->stream));
    k_begin_many<<<(m + 127) / 128, 128, 0, e->stream>>>(e->A.rep, e->d_pack_ids, e->d_pack_off, m);
    e->launches++;
    CK(cudaGetLastError());
  }
  *admitted = m;
  return SOP_OK;
}

extern "C" int sop_replica_add(sop_engine* e, const sop_system_desc* d, int* replica) {
  NvtxRange range("add replica");
  if (!e || !replica) return SOP_ERR_ARG;
  sop_prepared P;
  int rc = prepare(d, P);
  if (rc) return rc;
  sop_prepared* pp = &P;
  int got = 0;
  rc = sop_replicas_admit(e, &pp, nullptr, 1, replica, &got);
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->stream));
  return got == 1 ? SOP_OK : SOP_ERR_FULL;
}


// Move replica r's list rows to a range of row length >= need (+50% and 32
// spare), releasing the old range; the caller rebuilds.  Clears the overflow
// status.  SOP_ERR_FULL (old range kept) when the list arena has no room.
int sop::grow_rows(sop_engine* e, int r, int need) {
  Replica& R = e->reps[r];
  const int L2 = ((need + need / 2 + 32) + 7) / 8 * 8;
  long long nlb2;
  if (!e->lists.alloc((long long)R.n * L2, 8, &nlb2)) return SOP_ERR_FULL;
  RepDev got;
  int rc = get_rep(e, r, &got);
  if (rc) return rc;
  e->lists.release(R.nl_base, (long long)R.n * R.L);
  R.nl_base = nlb2;
  R.L = L2;
  got.nl_base = nlb2;
  got.L = L2;
  got.status &= ~SOP_ST_LIST_OVERFLOW;
  return put_rep(e, r, got);
}

// Build replica r's lists now; rows sized from a host estimate grow (up to
// three times) when the build finds a longer row.
int sop::rebuild_fit(sop_engine* e, int r, int mode) {
  int rc = build_now(e, r, mode);
  for (int attempt = 0; rc == SOP_OK && attempt < 3; attempt++) {
    RepDev got;
    rc = get_rep(e, r, &got);
    if (rc) return rc;
    if (!(got.status & SOP_ST_LIST_OVERFLOW)) return SOP_OK;
    rc = grow_rows(e, r, got.max_row);
    if (rc) return rc;
    rc = build_now(e, r, mode);
  }
  if (rc) return rc;
  RepDev got;
  rc = get_rep(e, r, &got);
  if (rc) return rc;
  return (got.status & SOP_ST_LIST_OVERFLOW) ? SOP_ERR_OVERFLOW : SOP_OK;
}

extern "C" int sop_replica_remove(sop_engine* e, int r) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  CK(cudaStreamSynchronize(e->stream));
  Replica& R = e->reps[r];
  RepDev d;
  std::memset(&d, 0, sizeof d);
  int rc = put_rep(e, r, d);
  if (rc) return rc;
  e->beads.release(R.off, R.n);
  e->lists.release(R.nl_base, (long long)R.n * R.L);
  e->nats.release(R.nat_base, R.nnat_e);
  e->bnds.release(R.bnd_base, R.nbnd_e);
  e->angs.release(R.ang_base, R.nang_e);
  e->excs.release(R.exc_base, R.nexc_e);
  e->cells.release(R.cell_base, R.ncell_e);
  R = Replica();
  e->layout_dirty = true;
  return SOP_OK;
}

extern "C" int sop_replica_count(const sop_engine* e, int* n) {
  if (!e || !n) return SOP_ERR_ARG;
  int c = 0;
  for (auto& R : e->reps) c += R.live;
  *n = c;
  return SOP_OK;
}

extern "C" int sop_replica_set_params(sop_engine* e, int r, const sop_params* p) {
  if (!e || !p || !live(e, r)) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  RepDev cfg = d;
  rc = fill_repdev(*p, cfg);
  if (rc) return rc;
  Replica& R = e->reps[r];
  // a new list mode or skin, or a new box or cell grid (minimum images are
  // decided at every build), rebuilds the lists now
  bool mode_changed = cfg.mode != d.mode || p->skin != R.params.skin || p->boxl != R.params.boxl ||
                      p->lcell != R.params.lcell || p->ncell != R.params.ncell;
  // another precision moves the replica to the other step kernel's items (the
  // next run restarts from the stored velocities, so no increment carries over)
  if (cfg.prec != d.prec) e->layout_dirty = true;
  // configuration fields only; run state and layout stay
  d.mode = cfg.mode; d.terms = cfg.terms; d.prec = cfg.prec; d.nnlup = cfg.nnlup; d.nup = cfg.nup;
  d.skin = cfg.skin; d.cell_edge = cfg.cell_edge; d.half_skin2 = cfg.half_skin2;
  d.boxl = cfg.boxl; d.lcell = cfg.lcell; d.ncell = cfg.ncell;
  d.Lh = cfg.Lh; d.Ll = cfg.Ll; d.invL = cfg.invL;
  d.a1 = cfg.a1; d.a2 = cfg.a2; d.a3 = cfg.a3; d.a4 = cfg.a4;
  d.a1d = cfg.a1d; d.a2d = cfg.a2d; d.a3d = cfg.a3d; d.a4d = cfg.a4d;
  d.noise_amp = cfg.noise_amp; d.T = cfg.T; d.kbnd = cfg.kbnd; d.R0sq = cfg.R0sq;
  d.noise_amp_d = cfg.noise_amp_d; d.pull_fd = cfg.pull_fd;
  d.inv_R0sq = cfg.inv_R0sq;
  d.kbnd_d = cfg.kbnd_d; d.R0sq_d = cfg.R0sq_d; d.fang = cfg.fang; d.fang_d = cfg.fang_d;
  d.e_bnd_coeff = cfg.e_bnd_coeff; d.e_ang_coeff = cfg.e_ang_coeff; d.pull_f = cfg.pull_f;
  d.dyn = cfg.dyn; d.a5 = cfg.a5; d.a5d = cfg.a5d; d.zeta_2h = cfg.zeta_2h;
  d.seed_lo = cfg.seed_lo; d.seed_hi = cfg.seed_hi;
  int pi = p->pull_i, pj = p->pull_j;
  d.pull_i = (pi >= 0 && pi < R.n) ? pi : 0;
  d.pull_j = (pj >= 0 && pj < R.n) ? pj : R.n - 1;
  R.params = *p;
  rc = put_rep(e, r, d);
  if (rc) return rc;
  if (mode_changed) {
    // a new list mode or skin may need longer rows than the replica holds
    if (p->list_mode == SOP_LIST_NONE && R.L < R.n) return SOP_ERR_UNSUPPORTED;
    rc = rebuild_fit(e, r, p->list_mode);
  }
  e->graph_valid = false;
  return rc;
}

extern "C" int sop_replica_get_params(sop_engine* e, int r, sop_params* p) {
  if (!e || !p || !live(e, r)) return SOP_ERR_ARG;
  *p = e->reps[r].params;
  return SOP_OK;
}

extern "C" int sop_replica_get_state(sop_engine* e, int r, double* pos, double* unc_pos,
                                     double* vel) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  Replica& R = e->reps[r];
  const int n = R.n;
  const long long off = R.off, cap = e->cap;
  std::vector<double> soa(3 * (size_t)n);
  if (pos || unc_pos) {
    for (int c = 0; c < 3; c++)
      CK(cudaMemcpyAsync(soa.data() + (size_t)c * n, e->A.X[d.cur] + c * cap + off,
                         n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 3; c++) {
        double u = soa[(size_t)c * n + i];
        if (unc_pos) unc_pos[3 * i + c] = u;
        if (pos) {
          // wrapped coordinate (sop.cpp:300-302); equal to unc_pos inside the box
          double b = d.boxl;
          double t = u / b;
          double rn = (t > 0) ? std::floor(t + 0.5) : std::ceil(t - 0.5);
          pos[3 * i + c] = u - b * rn;
        }
      }
  }
  if (vel) {
    for (int c = 0; c < 3; c++)
      CK(cudaMemcpyAsync(soa.data() + (size_t)c * n, e->A.vel + c * cap + off, n * sizeof(double),
                         cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 3; c++) vel[3 * i + c] = soa[(size_t)c * n + i];
  }
  return SOP_OK;
}

extern "C" int sop_replica_set_state(sop_engine* e, int r, const double* unc_pos, const double* vel) {
  if (!e || !live(e, r) || !unc_pos) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  if (d.running) return SOP_ERR_STATE;
  rc = upload_positions(e, r, unc_pos, 3);
  if (rc) return rc;
  rc = upload_velocities(e, r, vel);
  if (rc) return rc;
  // lists for the new positions (the reference builds them before loading a
  // restart, sop.cpp:119-136, and runs on stale lists until the next rebuild)
  return rebuild_fit(e, r, e->reps[r].params.list_mode);
}

extern "C" int sop_replica_status(sop_engine* e, int r, int* status, int64_t* steps) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  int err = 0;
  CK(cudaMemcpy(&err, e->A.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (status) *status = d.status | (err ? 0x100 : 0);
  if (steps) *steps = d.t;
  return SOP_OK;
}

extern "C" int sop_replica_info(sop_engine* e, int r, int64_t* out) {
  if (!e || !out || !live(e, r)) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  const Replica& R = e->reps[r];
  out[0] = R.n;
  out[1] = R.L;
  out[2] = d.max_row;
  out[3] = d.builds;
  out[4] = d.t;
  out[5] = d.status;
  out[6] = R.nnat_pairs;
  out[7] = R.off;
  return SOP_OK;
}

// ---- layout of the batched step -------------------------------------------------

// Contiguous blocks of work items for `grid` step CTAs with about equal
// estimated cost: an item costs its beads plus a fixed `item_cost` (the
// context load, staging wait and row latency every item pays, in bead
// equivalents).  first[b] is CTA b's first item, first[grid] = items.size().
static void split_items(const std::vector<StepItem>& items, int grid, int item_cost,
                        std::vector<int>& first) {
  double total = 0;
  for (const StepItem& w : items) total += item_cost + (w.b1 - w.b0);
  first.assign(grid + 1, (int)items.size());
  first[0] = 0;
  double acc = 0;
  int b = 1;
  for (size_t k = 0; k < items.size() && b < grid; k++) {
    // item k opens CTA b's block once the items before it fill b shares
    while (b < grid && acc >= total * b / grid) first[b++] = (int)k;
    acc += item_cost + (items[k].b1 - items[k].b0);
  }
}

// Step-kernel work items of one replica: chunks of cfg.chunk_beads beads,
// staged through shared memory when the replica fits the stage limit.
// FP64-precision replicas: chunks of 256 beads for k_step64 (never staged).
static std::vector<StepItem> replica_items(const sop_engine* e, int r) {
  const Replica& R = e->reps[r];
  const bool fp64 = R.params.precision == SOP_PREC_FP64;
  const int chunk = fp64 ? 256 : e->cfg.chunk_beads;
  const int staged = !fp64 && e->cfg.stage_limit > 0 && R.n <= e->cfg.stage_limit;
  std::vector<StepItem> items;
  for (int b = 0; b < R.n; b += chunk) items.push_back(StepItem{r, b, std::min(R.n, b + chunk), staged});
  return items;
}

int sop::refresh_layout(sop_engine* e) {
  if (!e->layout_dirty) return SOP_OK;
  std::vector<int> ids;
  for (int r = 0; r < (int)e->reps.size(); r++)
    if (e->reps[r].live) ids.push_back(r);
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return e->reps[a].n > e->reps[b].n; });
  e->active = ids;
  e->max_n = 0;
  e->items.clear();
  e->items64.clear();
  for (int r : ids) {
    const Replica& R = e->reps[r];
    e->max_n = std::max(e->max_n, R.n);
    std::vector<StepItem> it = replica_items(e, r);
    auto& dst = R.params.precision == SOP_PREC_FP64 ? e->items64 : e->items;
    dst.insert(dst.end(), it.begin(), it.end());
  }
  if ((long long)e->items.size() + 64 > e->items_cap) return SOP_ERR_FULL;
  if ((long long)e->items64.size() > e->items64_cap) return SOP_ERR_FULL;
  // the CTA queue: on request, or (automatic) while some replica steps
  // without staging; a captured graph launched the other way is recaptured
  bool unstaged = false;
  for (const StepItem& w : e->items) unstaged = unstaged || !w.staged;
  const bool queue = e->cfg.item_cost_beads >= 0 && e->step_grid <= e->cta_first_cap - 1 &&
                     (e->cfg.queue_blocks > 0 || (e->cfg.queue_blocks == 0 && unstaged));
  if (queue != e->step_queue) e->graph_valid = false;
  e->step_queue = queue;
  if (e->cfg.item_cost_beads >= 0 && e->step_grid <= e->cta_first_cap - 1) {
    if (queue) {
      // blocks {first, end} in item order, none empty
      const int per_cta = e->cfg.queue_blocks > 0 ? e->cfg.queue_blocks : kMaxQueueBlocks;
      const int nb = std::min<long long>(e->blk_cap, (long long)per_cta * e->step_grid);
      std::vector<int> first;
      split_items(e->items, nb, e->cfg.item_cost_beads, first);
      e->h_blk.clear();
      for (int b = 0; b < nb; b++)
        if (first[b] < first[b + 1]) {
          e->h_blk.push_back(first[b]);
          e->h_blk.push_back(first[b + 1]);
        }
      const int q[4] = {0, 0, (int)(e->h_blk.size() / 2), 0};
      if (!e->h_blk.empty())
        CK(h2d(reinterpret_cast<int*>(e->A.blk), e->h_blk.data(), e->h_blk.size(), e->stream));
      CK(h2d(e->A.blk_q, q, 4, e->stream));
    } else {
      split_items(e->items, e->step_grid, e->cfg.item_cost_beads, e->h_cta_first);
      CK(h2d(e->d_cta_first, e->h_cta_first.data(), e->h_cta_first.size(), e->stream));
    }
  }

  // the kernels read the counts from device memory, so a captured graph stays
  // valid; only the first FP64 replica (one more kernel per step) needs a recapture
  const int counts[3] = {(int)ids.size(), (int)e->items.size(), (int)e->items64.size()};
  if (!ids.empty()) CK(h2d(e->d_ids, ids.data(), ids.size(), e->stream));
  if (!e->items.empty()) CK(h2d(e->d_items, e->items.data(), e->items.size(), e->stream));
  if (!e->items64.empty()) CK(h2d(e->d_items64, e->items64.data(), e->items64.size(), e->stream));
  CK(h2d(e->d_counts, counts, 3, e->stream));
  const bool has64 = !e->items64.empty();
  if (has64 && !e->has64) e->graph_valid = false;
  e->has64 = e->has64 || has64;
  e->layout_dirty = false;
  return SOP_OK;
}

// Item boundaries of the batched step's CTAs, or null for equal item counts.
static const int* cta_first(const sop_engine* e) {
  return (e->cfg.item_cost_beads >= 0 && !e->step_queue && e->step_grid <= e->cta_first_cap - 1)
             ? e->d_cta_first : nullptr;
}
// Whether the batched step's CTAs take their item blocks from the CTA queue
// (decided by the last layout).
static int step_queue(const sop_engine* e) { return e->step_queue ? 1 : 0; }

// One step over given ids / items with host counts (single-replica paths).
int sop::enqueue_step(sop_engine* e, const int* d_ids, int nrep, const StepItem* d_items,
                      int nitems, int max_staged, int step_grid, int pro_grid, bool fp64) {
  NvtxRange range("plain step: k_prep + k_step");
  CK(launch_prologue(e->A, d_ids, nrep, nullptr, 0, 0, 1, pro_grid, e->stream));
  if (fp64)
    CK(launch_step64(e->A, d_items, nitems, nullptr, step_grid, e->stream));
  else
    CK(launch_step(e->A, d_items, nitems, nullptr, nullptr, 0, max_staged, e->cfg.lanes_per_bead,
                   e->cfg.step_min_blocks, e->cfg.step_strategy, e->cfg.block_threads, step_grid,
                   e->stream));
  e->launches += kStepLaunches;
  return SOP_OK;
}

// One batched step: k_prep (bookkeeping, binning, list slices, energies, observables),
// k_step, sized by the engine's fixed grids and the device-resident counts.
// full: the first step after host-side work (every later k_prep reads the
// device-side work flags the previous one left).
int sop::enqueue_batched_step(sop_engine* e, bool full) {
  NvtxRange range("batched step: k_prep + k_step");
  CK(launch_prologue(e->A, e->d_ids, e->cfg.max_replicas, e->d_counts, 0, 0,
                     (full || e->cfg.lean_prep < 0) ? 1 : 0,
                     e->pro_grid, e->stream));
  CK(launch_step(e->A, e->d_items, (int)e->items_cap, e->d_counts + 1, cta_first(e), step_queue(e), e->max_staged,
                 e->cfg.lanes_per_bead, e->cfg.step_min_blocks, e->cfg.step_strategy,
                 e->cfg.block_threads, e->step_grid, e->stream));
  e->launches += kStepLaunches;
  if (e->has64) {  // FP64-precision replicas, after the mixed ones
    CK(launch_step64(e->A, e->d_items64, (int)e->items64_cap, e->d_counts + 2, e->pro_grid,
                     e->stream));
    e->launches++;
  }
  return SOP_OK;
}

__global__ void k_begin(RepDev* rep, const int* ids, int nrep, long long nsteps) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrep) return;
  RepDev* R = &rep[ids[k]];
  if (!R->active) return;
  R->t_end = R->t + nsteps;
  R->first_pending = 1;
  R->running = 1;
}

__global__ void k_set_phase(RepDev* rep, int r, int phase) {
  RepDev* R = &rep[r];
  R->phase = phase;
  R->t_cur = R->t;
  R->out = 0;
}

// A bounded device wait ran out, or a checked build found a bad index (error
// word `err`, already read back): remember which, clear the word and the work
// queue (a unit published after its consumer gave up would otherwise be taken
// by the next step), and report.
static int timed_out(sop_engine* e, int err) {
  e->wait_errors = err;
  CK(cudaMemsetAsync(e->A.err, 0, sizeof(int), e->stream));
  CK(cudaMemsetAsync(e->A.units, 0xFF, sizeof(int4) * e->A.unit_cap, e->stream));
  CK(cudaMemsetAsync(e->A.unit_cnt, 0, sizeof(int), e->stream));
  CK(cudaMemsetAsync(e->A.unit_take, 0, sizeof(int), e->stream));
  CK(cudaMemsetAsync(e->A.unit_exit, 0, sizeof(int), e->stream));
  CK(cudaMemsetAsync(e->A.pro_done, 0, sizeof(int), e->stream));
  CK(cudaStreamSynchronize(e->stream));
  e->graph_valid = false;
  return SOP_ERR_TIMEOUT;
}

static int check_errors(sop_engine* e) {
  int err = 0;
  CK(cudaMemcpyAsync(&err, e->A.err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  if (!err) return SOP_OK;
  const int rc = timed_out(e, err);
  // a checked build found a partner index outside its replica
  return (err & kErrIndex) ? SOP_ERR_INDEX : rc;
}

extern "C" int sop_engine_inject_stall(sop_engine* e, int64_t publish_delay_ns, int skip_stage_copy) {
  if (!e || publish_delay_ns < 0 || publish_delay_ns > 1000000000LL) return SOP_ERR_ARG;
  e->A.publish_delay_ns = publish_delay_ns;
  e->A.skip_stage_copy = skip_stage_copy ? 1 : 0;
  e->graph_valid = false;  // kernels take the device arrays by value
  return SOP_OK;
}

extern "C" int sop_engine_wait_errors(sop_engine* e, int* bits) {
  if (!e || !bits) return SOP_ERR_ARG;
  *bits = e->wait_errors;
  return SOP_OK;
}

// ---- plain single-system path ------------------------------------------------------

extern "C" int sop_run_plain(sop_engine* e, int r, int64_t nsteps) {
  NvtxRange range("sop_run_plain");
  if (!e || !live(e, r) || nsteps < 0) return SOP_ERR_ARG;
  if (nsteps == 0) return SOP_OK;
  Replica& R = e->reps[r];
  CK(cudaSetDevice(e->cfg.device));
  // per-replica id and items (kept at the top of the id / item arrays)
  const int id_slot = scratch_id(e, 1);
  const std::vector<StepItem> items = replica_items(e, r);
  const int staged = items[0].staged;
  const long long item_slot = e->items_cap - (long long)items.size();
  if (item_slot < (long long)e->items.size()) return SOP_ERR_FULL;
  CK(cudaMemcpyAsync(e->d_ids + id_slot, &r, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  CK(h2d(e->d_items + item_slot, items.data(), items.size(), e->stream));
  k_begin<<<1, 32, 0, e->stream>>>(e->A.rep, e->d_ids + id_slot, 1, nsteps);
  e->launches++;
  CK(cudaGetLastError());
  CK(cudaEventRecord(e->ev[0], e->stream));
  const int grid = std::min((int)items.size(), 4 * e->prop.multiProcessorCount);
  const int bgrid = std::min((R.n + e->A.slice_beads - 1) / e->A.slice_beads + 1,
                             2 * e->prop.multiProcessorCount);
  for (int64_t s = 0; s <= nsteps; s++) {
    int rc = enqueue_step(e, e->d_ids + id_slot, 1, e->d_items + item_slot, (int)items.size(),
                          staged ? R.n : 0, grid, bgrid, R.params.precision == SOP_PREC_FP64);
    if (rc) return rc;
  }
  // observables are computed on demand (sop_observables), not at run end
  CK(cudaEventRecord(e->ev[1], e->stream));
  CK(cudaStreamSynchronize(e->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
  e->last_total_ms = ms;
  e->last_step_ms = -1;
  e->last_step_launches = nsteps + 1;
  return check_errors(e);
}

// ---- batched path: all replicas, graph-captured chunks ------------------------------

static int capture_graph(sop_engine* e) {
  if (e->graph_valid) return SOP_OK;
  NvtxRange range("capture step graph");
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  int64_t before = e->launches;
  for (int s = 0; s < e->cfg.graph_steps; s++) {
    int rc = enqueue_batched_step(e, s == 0);
    if (rc) { cudaStreamEndCapture(e->stream, &g); return rc; }
  }
  e->graph_launches = e->launches - before;
  e->launches = before;  // counted when replayed
  CK(cudaStreamEndCapture(e->stream, &g));
  CK(cudaGraphInstantiate(&e->graph_exec, g, 0));
  cudaGraphDestroy(g);
  e->graph_valid = true;
  return SOP_OK;
}

int sop::run_batched(sop_engine* e, int64_t nsteps, bool timed) {
  int rc = refresh_layout(e);
  if (rc) return rc;
  if (e->active.empty() || nsteps <= 0) return SOP_OK;
  rc = capture_graph(e);
  if (rc) return rc;
  const int nrep = (int)e->active.size();
  k_begin<<<(nrep + 127) / 128, 128, 0, e->stream>>>(e->A.rep, e->d_ids, nrep, nsteps);
  e->launches++;
  CK(cudaGetLastError());
  if (timed) CK(cudaEventRecord(e->ev[0], e->stream));
  const int64_t iters = nsteps + 1;
  const int S = e->cfg.graph_steps;
  const int64_t full = iters / S;
  {
    NvtxRange graphs("graph launches");
    for (int64_t k = 0; k < full; k++) {
      CK(cudaGraphLaunch(e->graph_exec, e->stream));
      e->launches += e->graph_launches;
    }
  }
  for (int64_t k = full * S; k < iters; k++) {
    rc = enqueue_batched_step(e, k == full * S);
    if (rc) return rc;
  }
  // observables are computed on demand (sop_observables), not at run end
  if (timed) CK(cudaEventRecord(e->ev[1], e->stream));
  CK(cudaStreamSynchronize(e->stream));
  if (timed) {
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
    e->last_total_ms = ms;
  }
  e->last_step_launches = iters;
  return check_errors(e);
}

extern "C" int sop_replica_start(sop_engine* e, int r, int64_t nsteps) {
  if (!e || !live(e, r) || nsteps < 1) return SOP_ERR_ARG;
  CK(cudaSetDevice(e->cfg.device));
  const int slot = scratch_id(e, 2);
  CK(cudaMemcpyAsync(e->d_ids + slot, &r, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  k_begin<<<1, 32, 0, e->stream>>>(e->A.rep, e->d_ids + slot, 1, nsteps);
  e->launches++;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(e->stream));  // the id slot is reused by the next call
  return SOP_OK;
}

extern "C" int sop_replicas_retire(sop_engine* e, const int* ids, int n, double* energy6, double* obs5,
                                   int* status) {
  NvtxRange range("retire replicas");
  if (!e || n < 0 || (n > 0 && !ids) || n > e->cfg.max_replicas) return SOP_ERR_ARG;
  if (n == 0) return SOP_OK;
  std::vector<char> seen(e->cfg.max_replicas, 0);
  for (int k = 0; k < n; k++) {
    if (!live(e, ids[k]) || seen[ids[k]]) return SOP_ERR_ARG;  // each replica once
    seen[ids[k]] = 1;
  }
  if (e->chunk_open) return SOP_ERR_STATE;
  CK(cudaSetDevice(e->cfg.device));
  CK(cudaStreamSynchronize(e->stream));
  // final energies and observables of all of them, then one packed read-back
  // that also clears their descriptors (removal)
  CK(cudaMemcpyAsync(e->d_pack_ids, ids, n * sizeof(int), cudaMemcpyHostToDevice, e->stream));
  int rc_e = enqueue_energy(e, ids, e->d_pack_ids, n);
  if (rc_e) return rc_e;
  CK(launch_observables(e->A, e->d_pack_ids, n, e->stream));
  e->launches++;
  int err = 0;
  const int rc = read_packed_reps(e, n, 1, &err);
  if (rc) return rc;
  for (int k = 0; k < n; k++) {
    const RepDev& d = e->h_reps[k];
    if (energy6) std::memcpy(energy6 + 6 * k, d.energy, sizeof d.energy);
    if (obs5) std::memcpy(obs5 + 5 * k, d.obs, sizeof d.obs);
    if (status) status[k] = d.status | (err ? 0x100 : 0);
    // removal: the descriptor was cleared by the read-back, arenas returned
    sop::Replica& R = e->reps[ids[k]];
    e->beads.release(R.off, R.n);
    e->lists.release(R.nl_base, (long long)R.n * R.L);
    e->nats.release(R.nat_base, R.nnat_e);
    e->bnds.release(R.bnd_base, R.nbnd_e);
    e->angs.release(R.ang_base, R.nang_e);
    e->excs.release(R.exc_base, R.nexc_e);
    e->cells.release(R.cell_base, R.ncell_e);
    R = sop::Replica();
  }
  e->layout_dirty = true;
  return SOP_OK;
}

extern "C" int sop_run_chunk_begin(sop_engine* e, int64_t steps) {
  NvtxRange range("run chunk: launch");
  if (!e || steps < 0) return SOP_ERR_ARG;
  if (e->chunk_open) return SOP_ERR_STATE;
  CK(cudaSetDevice(e->cfg.device));
  int rc = refresh_layout(e);
  if (rc) return rc;
  if (e->active.empty() || steps == 0) return SOP_OK;
  rc = capture_graph(e);
  if (rc) return rc;
  CK(cudaMemsetAsync(e->A.done_cnt, 0, sizeof(int), e->stream));
  CK(cudaEventRecord(e->ev[0], e->stream));
  const int S = e->cfg.graph_steps;
  for (int64_t k = 0; k < steps / S; k++) {
    CK(cudaGraphLaunch(e->graph_exec, e->stream));
    e->launches += e->graph_launches;
  }
  for (int64_t k = steps / S * S; k < steps; k++) {
    rc = enqueue_batched_step(e, k == steps / S * S);
    if (rc) return rc;
  }
  CK(cudaEventRecord(e->ev[1], e->stream));
  CK(cudaMemcpyAsync(e->h_done, e->A.done_cnt, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  e->chunk_open = true;
  return SOP_OK;
}

extern "C" int sop_run_chunk_end(sop_engine* e, int* finished, int cap, int* nfinished) {
  NvtxRange range("run chunk: wait");
  if (!e || (cap > 0 && !finished)) return SOP_ERR_ARG;
  if (nfinished) *nfinished = 0;
  if (!e->chunk_open) return SOP_OK;
  e->chunk_open = false;
  CK(cudaStreamSynchronize(e->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
  e->last_total_ms = ms;
  const int nd = std::min(*e->h_done, e->A.done_cap);
  if (nd > 0 && cap > 0)
    CK(cudaMemcpy(finished, e->A.done_list, std::min(nd, cap) * sizeof(int), cudaMemcpyDeviceToHost));
  if (nfinished) *nfinished = nd;
  return check_errors(e);
}

extern "C" int sop_run_chunk(sop_engine* e, int64_t steps, int* finished, int cap, int* nfinished) {
  if (!e || steps < 0 || (cap > 0 && !finished)) return SOP_ERR_ARG;
  int rc = sop_run_chunk_begin(e, steps);
  if (rc) return rc;
  return sop_run_chunk_end(e, finished, cap, nfinished);
}

int sop::begin_all(sop_engine* e, int64_t nsteps) {
  int rc = refresh_layout(e);
  if (rc) return rc;
  const int nrep = (int)e->active.size();
  if (nrep == 0) return SOP_ERR_STATE;
  k_begin<<<(nrep + 127) / 128, 128, 0, e->stream>>>(e->A.rep, e->d_ids, nrep, nsteps);
  e->launches++;
  CK(cudaGetLastError());
  return SOP_OK;
}

int sop::run_steps(sop_engine* e, int64_t steps, float* ms) {
  int rc = refresh_layout(e);
  if (rc) return rc;
  rc = capture_graph(e);
  if (rc) return rc;
  CK(cudaEventRecord(e->ev[0], e->stream));
  const int S = e->cfg.graph_steps;
  for (int64_t k = 0; k < steps / S; k++) {
    CK(cudaGraphLaunch(e->graph_exec, e->stream));
    e->launches += e->graph_launches;
  }
  for (int64_t k = steps / S * S; k < steps; k++) {
    rc = enqueue_batched_step(e, k == steps / S * S);
    if (rc) return rc;
  }
  CK(cudaEventRecord(e->ev[1], e->stream));
  CK(cudaStreamSynchronize(e->stream));
  float t = 0;
  cudaEventElapsedTime(&t, e->ev[0], e->ev[1]);
  if (ms) *ms = t;
  return check_errors(e);
}

sop::LaunchShape sop::get_launch_shape(const sop_engine* e) {
  LaunchShape s;
  s.threads = e->cfg.block_threads;
  s.chunk = e->cfg.chunk_beads;
  s.stage = e->cfg.stage_limit > 0 ? e->cfg.stage_limit : -1;
  s.slice = e->cfg.build_slice_beads;
  s.min_blocks = e->cfg.step_min_blocks;
  s.strategy = e->cfg.step_strategy;
  s.lanes = e->cfg.lanes_per_bead;
  s.group_pct = e->cfg.group_rebuild_pct;
  s.item_cost = e->cfg.item_cost_beads;
  s.queue = e->cfg.queue_blocks;
  return s;
}

void sop::set_launch_shape(sop_engine* e, const LaunchShape& s) {
  e->cfg.block_threads = s.threads;
  e->cfg.step_strategy = s.strategy == 1 ? 1 : 0;
  e->cfg.step_min_blocks = (s.min_blocks >= 2 && s.min_blocks <= 4) ? s.min_blocks : 3;
  if (e->cfg.step_strategy == 1 && e->cfg.step_min_blocks == 4) e->cfg.step_min_blocks = 3;
  e->cfg.lanes_per_bead = s.lanes;
  e->cfg.build_slice_beads = std::max(s.slice, kMinSliceBeads);
  e->A.slice_beads = e->cfg.build_slice_beads;
  e->cfg.chunk_beads = s.chunk;
  e->cfg.stage_limit = std::min(s.stage, kStageMax);
  e->max_staged = e->cfg.stage_limit > 0 ? e->cfg.stage_limit : 0;
  e->cfg.group_rebuild_pct = (s.group_pct > 0 && s.group_pct < 100) ? s.group_pct : 0;
  e->cfg.item_cost_beads = s.item_cost < 0 ? -1 : std::min(s.item_cost, 1 << 20);
  e->cfg.queue_blocks = s.queue < 0 ? -1 : std::min(s.queue, kMaxQueueBlocks);
  e->A.group_frac2 = e->cfg.group_rebuild_pct > 0
                         ? (float)(1e-4 * e->cfg.group_rebuild_pct * e->cfg.group_rebuild_pct)
                         : 4.0f;
  e->step_grid = std::max(1, step_blocks_per_sm(e->cfg.lanes_per_bead, e->cfg.step_min_blocks,
                                                   e->cfg.step_strategy, s.threads, e->max_staged)) *
                 e->prop.multiProcessorCount;
  e->layout_dirty = true;
  e->graph_valid = false;  // kernels take the device arrays by value
}

extern "C" int sop_run(sop_engine* e, int64_t nsteps) {
  if (!e || nsteps < 0) return SOP_ERR_ARG;
  NvtxRange range("sop_run");
  CK(cudaSetDevice(e->cfg.device));
  return run_batched(e, nsteps, true);
}

extern "C" int sop_last_run_timing(sop_engine* e, double* total_ms, double* step_ms,
                                   int64_t* step_launches) {
  if (!e) return SOP_ERR_ARG;
  if (total_ms) *total_ms = e->last_total_ms;
  if (step_ms) *step_ms = e->last_step_ms;
  if (step_launches) *step_launches = e->last_step_launches;
  return SOP_OK;
}

extern "C" int sop_profile_steps_ex(sop_engine* e, int64_t nsteps, double* ms) {
  if (!e || nsteps <= 0 || !ms) return SOP_ERR_ARG;
  CK(cudaSetDevice(e->cfg.device));
  int rc = refresh_layout(e);
  if (rc) return rc;
  if (e->active.empty()) return SOP_ERR_STATE;
  const int nrep = (int)e->active.size();
  k_begin<<<(nrep + 127) / 128, 128, 0, e->stream>>>(e->A.rep, e->d_ids, nrep, nsteps);
  e->launches++;
  const int64_t iters = nsteps + 1;
  constexpr int kE = 5;  // event marks: start, before k_prep, after it, (the same), after k_step
  std::vector<cudaEvent_t> ev(kE * iters);
  for (auto& x : ev) CK(cudaEventCreate(&x));
  for (int64_t s = 0; s < iters; s++) {
    cudaEvent_t* E = &ev[kE * s];
    CK(cudaEventRecord(E[0], e->stream));
    CK(launch_prologue(e->A, e->d_ids, e->cfg.max_replicas, e->d_counts, 0, 0, s == 0, e->pro_grid,
                       e->stream, E[1], E[2]));
    CK(cudaEventRecord(E[3], e->stream));
    CK(launch_step(e->A, e->d_items, (int)e->items_cap, e->d_counts + 1, cta_first(e), step_queue(e), e->max_staged,
                   e->cfg.lanes_per_bead, e->cfg.step_min_blocks, e->cfg.step_strategy, e->cfg.block_threads, e->step_grid, e->stream));
    CK(cudaEventRecord(E[4], e->stream));
    e->launches += kStepLaunches;
  }
  CK(cudaStreamSynchronize(e->stream));
  double acc[4] = {0, 0, 0, 0};
  for (int64_t s = 0; s < iters; s++)
    for (int k = 0; k < 4; k++) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[kE * s + k], ev[kE * s + k + 1]);
      acc[k] += t;
    }
  for (auto& x : ev) cudaEventDestroy(x);
  for (int k = 0; k < 4; k++) ms[k] = acc[k] / iters;
  return check_errors(e);
}

extern "C" int sop_profile_steps(sop_engine* e, int64_t nsteps, double* step_ms, double* pro_ms) {
  double ms[4];
  int rc = sop_profile_steps_ex(e, nsteps, ms);
  if (rc) return rc;
  if (step_ms) *step_ms = ms[3];
  if (pro_ms) *pro_ms = ms[0] + ms[1] + ms[2];
  return SOP_OK;
}

extern "C" int sop_run_host(sop_engine* e, const double* xyz_in, const double* vel_in,
                            int64_t nsteps, double* xyz_out, double* vel_out) {
  if (!e || !xyz_in || nsteps < 0) return SOP_ERR_ARG;
  int rc = refresh_layout(e);
  if (rc) return rc;
  std::vector<int> ids;
  std::vector<long long> poff;
  long long total = 0;
  for (int r = 0; r < (int)e->reps.size(); r++)
    if (e->reps[r].live) {
      ids.push_back(r);
      poff.push_back(total);
      total += e->reps[r].n;
    }
  const int nrep = (int)ids.size();
  if (nrep == 0) return SOP_OK;
  // one copy in, scatter on the device, lists rebuilt at the new positions
  CK(h2d(e->d_pack_ids, ids.data(), nrep, e->stream));
  CK(h2d(e->d_pack_off, poff.data(), nrep, e->stream));
  CK(h2d(e->d_pack_xyz, xyz_in, 3 * total, e->stream));
  if (vel_in) CK(h2d(e->d_pack_vel, vel_in, 3 * total, e->stream));
  CK(launch_scatter_state(e->A, e->d_pack_ids, nrep, e->d_pack_off, e->d_pack_xyz,
                          vel_in ? e->d_pack_vel : nullptr, e->stream));
  CK(launch_prologue(e->A, e->d_pack_ids, nrep, nullptr, 1, -1, 1, e->pro_grid, e->stream));
  e->launches += kPrologueLaunches;
  rc = run_batched(e, nsteps, false);
  if (rc) return rc;
  // gather on the device, one copy out
  CK(launch_gather_state(e->A, e->d_pack_ids, nrep, e->d_pack_off, e->d_pack_xyz, e->d_pack_vel,
                         e->stream));
  e->launches++;
  if (xyz_out)
    CK(cudaMemcpyAsync(xyz_out, e->d_pack_xyz, 3 * total * sizeof(double), cudaMemcpyDeviceToHost,
                       e->stream));
  if (vel_out)
    CK(cudaMemcpyAsync(vel_out, e->d_pack_vel, 3 * total * sizeof(double), cudaMemcpyDeviceToHost,
                       e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

// ---- reference-named operations -------------------------------------------------

extern "C" int sop_update_neighbor_list(sop_engine* e, int r) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  return build_now(e, r, SOP_LIST_NEIGHBOR);
}

extern "C" int sop_update_cell_list(sop_engine* e, int r) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  return build_now(e, r, SOP_LIST_CELL);
}

extern "C" int sop_update_pair_list(sop_engine* e, int r) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  Replica& R = e->reps[r];
  CK(launch_pairlist(e->A, r, (int)R.off, R.n, e->stream));
  e->launches++;
  CK(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}

extern "C" int sop_get_pair_list(sop_engine* e, int r, int which, int* ii, int* jj, int cap,
                                 int* count) {
  if (!e || !live(e, r) || which < 0 || which > 3 || !count) return SOP_ERR_ARG;
  Replica& R = e->reps[r];
  CK(cudaMemsetAsync(e->A.pairs_cnt, 0, sizeof(int), e->stream));
  CK(launch_export(e->A, r, (int)R.off, R.n, which, e->pairs_cap, e->stream));
  e->launches++;
  int n = 0;
  CK(cudaMemcpyAsync(&n, e->A.pairs_cnt, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  if (n > e->pairs_cap) return SOP_ERR_OVERFLOW;
  std::vector<unsigned long long> buf(n);
  if (n) CK(cudaMemcpy(buf.data(), e->A.pairs_out, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  std::sort(buf.begin(), buf.end());
  *count = n;
  if (ii && jj) {
    for (int k = 0; k < n && k < cap; k++) {
      ii[k] = (int)(buf[k] >> 32);
      jj[k] = (int)(buf[k] & 0xffffffffu);
    }
    if (n > cap) return SOP_ERR_OVERFLOW;
  }
  return SOP_OK;
}

static int run_phase(sop_engine* e, int r, int phase) {
  Replica& R = e->reps[r];
  const std::vector<StepItem> items = replica_items(e, r);
  const int staged = items[0].staged;
  const long long item_slot = e->items_cap - (long long)items.size();
  CK(h2d(e->d_items + item_slot, items.data(), items.size(), e->stream));
  k_set_phase<<<1, 1, 0, e->stream>>>(e->A.rep, r, phase);
  const int grid = std::min((int)items.size(), 4 * e->prop.multiProcessorCount);
  if (R.params.precision == SOP_PREC_FP64)
    CK(launch_step64(e->A, e->d_items + item_slot, (int)items.size(), nullptr, grid, e->stream));
  else
    CK(launch_step(e->A, e->d_items + item_slot, (int)items.size(), nullptr, nullptr, 0, staged ? R.n : 0,
                   e->cfg.lanes_per_bead, e->cfg.step_min_blocks, e->cfg.step_strategy,
                   e->cfg.block_threads, grid, e->stream));
  e->launches += 2;
  CK(cudaStreamSynchronize(e->stream));
  return check_errors(e);
}

extern "C" int sop_force_eval(sop_engine* e, int r, double* force_xyz) {
  NvtxRange range("sop_force_eval");
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  int rc = run_phase(e, r, PH_FORCE);
  if (rc) return rc;
  Replica& R = e->reps[r];
  if (force_xyz) {
    const int n = R.n;
    std::vector<double> soa(3 * (size_t)n);
    for (int c = 0; c < 3; c++)
      CK(cudaMemcpyAsync(soa.data() + (size_t)c * n, e->A.force + c * e->cap + R.off,
                         n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 3; c++) force_xyz[3 * i + c] = soa[(size_t)c * n + i];
  }
  return SOP_OK;
}

extern "C" int sop_energy_eval(sop_engine* e, int r, double* out) {
  NvtxRange range("sop_energy_eval");
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  CK(cudaMemcpyAsync(e->d_ids + scratch_id(e, 0), &r, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  int rc_e = enqueue_energy(e, &r, e->d_ids + scratch_id(e, 0), 1);
  if (rc_e) return rc_e;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  if (out) std::memcpy(out, d.energy, sizeof d.energy);
  return SOP_OK;
}

extern "C" int sop_observables(sop_engine* e, int r, double* out) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  CK(cudaMemcpyAsync(e->d_ids + scratch_id(e, 0), &r, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  CK(launch_observables(e->A, e->d_ids + scratch_id(e, 0), 1, e->stream));
  e->launches++;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  if (out) std::memcpy(out, d.obs, sizeof d.obs);
  return SOP_OK;
}

extern "C" int sop_replica_outputs(sop_engine* e, int r, double* energy6, double* obs5) {
  if (!e || !live(e, r)) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  if (energy6) std::memcpy(energy6, d.energy, sizeof d.energy);
  if (obs5) std::memcpy(obs5, d.obs, sizeof d.obs);
  return SOP_OK;
}

extern "C" int sop_replica_set_step(sop_engine* e, int r, int64_t step) {
  if (!e || !live(e, r) || step < 0) return SOP_ERR_ARG;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  if (d.running) return SOP_ERR_STATE;
  d.t = step;
  return put_rep(e, r, d);
}

extern "C" int sop_underdamped_iteration(sop_engine* e, int r) {
  // incr = a1 v + a2 F, x += incr, F = force(x), v = a3 incr + a4 F: a run of one
  // iteration (the restart step recomputes F at x with the same noise index)
  return sop_run_plain(e, r, 1);
}

// ---- host-side numerics self-checks ------------------------------------------------

extern "C" void sop_selftest_split(double x, float* hi, float* lo) {
  float h, l;
  split_double(x, h, l);
  if (hi) *hi = h;
  if (lo) *lo = l;
}

extern "C" void sop_selftest_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox4x32_10(ctr, key, out);
}
