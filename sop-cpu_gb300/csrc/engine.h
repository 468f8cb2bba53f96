// Internal host-side state of the GB300 SOP engine (not part of the C ABI).
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <vector>

#include "../../include/sop_gpu.h"
#include "kernels.cuh"
#include "sop_common.cuh"

namespace sop {

// First-fit allocator of index ranges inside one preallocated device array.
class RangeAlloc {
 public:
  void init(long long cap) {
    free_.clear();
    if (cap > 0) free_[0] = cap;
    cap_ = cap;
    used_ = 0;
  }
  bool alloc(long long n, long long align, long long* out);
  void release(long long start, long long n);
  long long largest() const;
  long long used() const { return used_; }
  long long capacity() const { return cap_; }

 private:
  std::map<long long, long long> free_;
  long long cap_ = 0, used_ = 0;
};

// Host record of one admitted system.
struct Replica {
  bool live = false;
  int n = 0;
  long long off = 0, nl_base = 0;
  int L = 0;
  long long nat_base = 0, nnat_e = 0, bnd_base = 0, nbnd_e = 0, ang_base = 0, nang_e = 0,
            exc_base = 0, nexc_e = 0, cell_base = 0, ncell_e = 0;
  int nnat_pairs = 0;
  sop_params params{};
  std::vector<int> type, chain;
};

const FFTables& tables();

}  // namespace sop

// Named host-side ranges for profilers (NVTX v3, header-only: without an
// attached tool each push / pop is a cheap no-op).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr int64_t kDefaultWaitNs = 2000000000LL;  // device-side wait limits: 2 s
constexpr int64_t kMaxWaitNs = 60000000000LL;
constexpr int kMaxQueueBlocks = 8;  // item blocks per step CTA in the CTA queue (at most)

struct sop_engine {
  sop_engine_config cfg{};
  cudaDeviceProp prop{};
  cudaStream_t stream = nullptr;
  sop::DevArrays A{};
  long long cap = 0;
  sop::RangeAlloc beads, lists, nats, bnds, angs, excs, cells;
  std::vector<sop::Replica> reps;
  sop::RepDev* h_rep = nullptr;  // pinned staging for descriptor copies
  sop::RepDev* h_reps = nullptr; // pinned descriptors read back (all of them, or a packed batch)
  sop::RepDev* d_reps_pack = nullptr;  // descriptors of one admission / retirement batch, packed
  int* d_en_base = nullptr;       // energy kernel: first partial-sum slot of each replica of a batch
  long long en_part_cap = 0;      // energy kernel: partial-sum slots (4 doubles each)
  int* h_done = nullptr;         // pinned: replicas whose window closed in the open chunk
  bool chunk_open = false;       // a chunk was launched and not yet waited for
  // batched layout
  int* d_ids = nullptr;             // active replica ids; scratch slots at the end
  sop::StepItem* d_items = nullptr; // step work items; scratch at the end
  long long items_cap = 0;
  std::vector<int> active;
  std::vector<sop::StepItem> items;
  sop::StepItem* d_items64 = nullptr;  // items of FP64-precision replicas (k_step64)
  std::vector<sop::StepItem> items64;
  long long items64_cap = 0;
  bool has64 = false;                  // an FP64 replica was ever laid out (k_step64 launched)
  int max_n = 0, max_staged = 0, step_grid = 1, pro_grid = 1;
  int* d_counts = nullptr;          // {active replicas, work items}, read by the kernels
  int* d_cta_first = nullptr;       // per step CTA, its first work item (cost-balanced split)
  int cta_first_cap = 0;
  std::vector<int> h_cta_first;
  long long blk_cap = 0;            // CTA queue blocks (DevArrays::blk)
  bool step_queue = false;          // the batched step's CTAs take blocks from the queue
  std::vector<int> h_blk;
  // packed host-order state of sop_run_host (one copy each way)
  double* d_pack_xyz = nullptr;
  double* d_pack_vel = nullptr;
  int* d_pack_ids = nullptr;
  long long* d_pack_off = nullptr;
  bool layout_dirty = true;
  // CUDA graph of graph_steps batched steps
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_valid = false;
  // bookkeeping
  int pairs_cap = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t launches = 0;
  int wait_errors = 0;  // error-word bits of the last call that timed out
  int64_t graph_launches = 0;  // launches of one replay of the step graph
  double last_total_ms = 0, last_step_ms = -1;
  int64_t last_step_launches = 0;
};

namespace sop {
int upload_positions(sop_engine* e, int r, const double* xyz, int which_bufs);
int upload_velocities(sop_engine* e, int r, const double* vel);
int get_rep(sop_engine* e, int r, RepDev* out);
int put_rep(sop_engine* e, int r, const RepDev& d);
int build_now(sop_engine* e, int r, int mode);
int grow_rows(sop_engine* e, int r, int need);
int rebuild_fit(sop_engine* e, int r, int mode);
int refresh_layout(sop_engine* e);
// batched steps inside an open run window (k_begin already issued); ms = CUDA-event time
int run_steps(sop_engine* e, int64_t steps, float* ms);
// open a run window of nsteps for every active replica
int begin_all(sop_engine* e, int64_t nsteps);
// Knobs that change how the batched step is launched but not what it computes.
struct LaunchShape {
  int threads;     // step-kernel block size
  int chunk;       // beads per step work item
  int stage;       // stage limit (beads; -1 = never staged)
  int slice;       // beads per list-build slice
  int min_blocks;  // step-kernel register budget: 2 or 3 CTAs per SM
  int strategy;    // 0 CTA items, 1 warp tasks
  int lanes;       // lanes per bead
  int group_pct;   // grouped skin rebuilds (0 = off)
  int item_cost;   // step CTA blocks by estimated cost (bead equivalents per item; <0 = equal counts)
  int queue;       // item blocks per CTA in the CTA queue (0 = automatic, <0 = one fixed block per CTA)
};
LaunchShape get_launch_shape(const sop_engine* e);
// recompute the persistent grid, invalidate layout and graph
void set_launch_shape(sop_engine* e, const LaunchShape& s);
int enqueue_step(sop_engine* e, const int* d_ids, int nrep, const StepItem* d_items, int nitems,
                 int max_staged, int step_grid, int pro_grid, bool fp64);
// one step of every active replica, sized only by device-resident counts
int enqueue_batched_step(sop_engine* e, bool full);
int run_batched(sop_engine* e, int64_t nsteps, bool timed);
inline int scratch_id(const sop_engine* e, int k) { return e->cfg.max_replicas + k; }
}  // namespace sop
