// Launch interface between the engine (engine.cu) and the kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "sop_common.cuh"

namespace sop {

// Raw device pointers of the packed arrays, passed by value to every kernel.
struct DevArrays {
  double* X[2];       // SoA unc_pos, x|y|z blocks of `cap`
  float4* stage[2];   // {hi.xyz,type},{lo.xyz,chain} per bead
  float* incr;        // SoA position increment of the last step
  double* incr64;     // the same in FP64 (replicas with FP64 precision)
  double* vel;        // SoA velocities
  double* force;      // SoA forces of the last force-only / final step
  float4* xb;         // positions at the last list build
  int4* topo;         // {nat_start, bnd_start, ang_start, nat_cnt | bnd_cnt<<16 | ang_cnt<<24}
  int2* exc_rng;      // {exc_start, exc_cnt}
  int4* nat;          // {j | NL | PL, r0^2 hi f32, r0^2 lo f32, r0 f32}
  double* nat_r0;     // FP64 native distance per native entry
  int4* bnd;          // {j, r0 f32, r0^2 hi f32, r0^2 lo f32}
  double* bnd_r0;     // FP64 bond length per bond entry
  int* ang;           // soft-sphere partner per angle entry
  int* exc;           // excluded partners (sorted per bead)
  int* nl;            // neighbor-list entries
  int* nl_cnt;        // row length per bead
  int* nl_near;       // per bead: row entries [nl_near, nl_cnt) are far (see build_slice)
  RepDev* rep;        // replica descriptors
  long long cap;      // bead capacity (SoA stride)
  unsigned long long* pairs_out;  // export buffer (i<<32|j)
  int* pairs_cnt;
  int* err;           // engine-wide error word (bounded waits that gave up)
  long long queue_wait_ns;     // k_prep: wait for a unit being published
  long long stage_wait_ns;     // k_step: wait for the staging copy
  long long publish_delay_ns;  // diagnostics: producers stall before publishing
  int skip_stage_copy;         // diagnostics: staging copies expected, not issued
  int4* units;        // per-step work queue (builds in slices, energies, observables)
  int* unit_cnt;      // units queued this step
  int* unit_exit;     // k_prep CTAs finished (the last one resets the queue)
  int* unit_take;     // next unit ticket
  int* pro_done;      // k_prep CTAs done publishing
  int* slice_done;    // per replica: build slices finished this step
  int unit_cap;
  int* done_list;     // replicas whose run window closed (final step taken)
  int* done_cnt;
  int done_cap;
  // cell bins of the last list build (binning -> build slices)
  float4* bin_p;      // per bead: position relative to the grid origin, .w = type | chain << 2 (int bits)
  int* bin_sorted;    // per bead slot: local bead ids sorted by cell, bead order within a cell
  int* bin_cell;      // per bead: cell index
  int* cstart;        // per replica cell range (RepDev::cell_base): exclusive prefix of cell counts
  int* ccur;          // same layout: scatter cursors
  struct BinHdr* bin_hdr;  // per replica: grid of the last binning
  int slice_beads;    // beads per list-build slice unit
  int* step_ctr;      // warp-task step kernel: {next item, finished warps}
  int* any_rebuild;   // a SKIN displacement trigger fired in the last step
  // {[0] the next k_prep may have queued work, [1] the same, being decided by
  //  this k_prep, [2] lean k_preps that found work all the same (diagnostic)}
  int* prep_flag;
  // energy slices of sop_energy_eval / retirement: 4 partial sums per slice,
  // and per replica of the batch the count of finished slices (reset to 0)
  double* en_part;
  int* en_done;
  float group_frac2;  // (grouping fraction of the trigger distance)^2; > 1 = no grouping
  int row_bands;      // list rows keep their far entries at the end (0 = off)
  // k_step's CTA queue: blocks of work items {first, end} that the CTAs take
  // in turn when blk_dyn is set; blk_q = {next block, CTAs done, blocks}
  int2* blk;
  int* blk_q;
  int blk_dyn;
};

// Bits of the engine's error word (DevArrays::err): 1 and 2 a bounded wait
// ran out (staging copy, work queue); kErrIndex a checked build found a
// partner index outside its replica.
constexpr int kErrIndex = 4;

// Grid of one replica's last binning.
struct BinHdr {
  int ok, status, nx, ny, nz, K, ncell;  // K: stencil half-width in cells
  int img;                               // minimum images: one cell, every bead a candidate
  float edge, ox, oy, oz, margin;        // margin: relative FP32 screening band
  int cx0, cy0, cz0;                     // cell-mode origin cell (floor(x / lcell))
  // non-native list and pair cutoffs^2 by [bead type][partner type 1, 2], in
  // FP64 for the exact decisions and rounded to FP32 for the screen
  float rl2f[kMaxTypes][2], pl2f[kMaxTypes][2];
  // (pair cutoff + band width)^2 in FP32: a list entry farther than this at
  // the build is "far" and sits at the end of its row
  float bandf[kMaxTypes][2];
  double rl2d[kMaxTypes][2], pl2d[kMaxTypes][2];
};

constexpr int kSliceBeads = 32;       // default beads per list-build work unit
constexpr int kMinSliceBeads = 16;
constexpr int kMaxReplicaBeads = 1 << 22;

// Work item of the step kernel: beads [b0,b1) of replica r; staged = the
// replica's positions fit in shared memory.
struct StepItem {
  int r, b0, b1, staged;
};

constexpr int kStageMax = 6144;       // beads staged in shared memory (192 KB)
constexpr int kBuildThreads = 512;
constexpr int kEnergySlice = 256;     // beads per CTA of the energy kernel
// kernel launches of one step: k_prep (bookkeeping, binning, list builds), k_step
constexpr int kPrologueLaunches = 1;
constexpr int kStepLaunches = 2;
// cells a replica's binning may use (grid cells grow wider beyond that)
inline long long cell_capacity(int n) { return 4LL * n + 4096; }

void upload_tables(const FFTables& t, cudaStream_t s);
// Opt the kernels into shared memory (once per device): optin_bytes per block
// at most, sm_bytes per SM.
cudaError_t init_kernels(int optin_bytes, int sm_bytes);

// Prologue + list build over `nrep` replica ids in one cooperative launch of
// k_prep (bookkeeping, cell binning of the replicas that rebuild, list slices,
// energies, observables).
// force_build: build for every listed replica from the CURRENT buffer
// (reference-named list updates), else the step cadence decides.
// nrep / nitems: host counts (grid sizing); *_dev: the same counts in device
// memory, read by the kernels when given (graphs survive layout changes).
// after_decide / after_bin: events recorded before and after k_prep (profiling)
// full: run the consumer phase whatever the device-side work flags say (the
// first k_prep after any host-side change to replica state)
cudaError_t launch_prologue(const DevArrays& A, const int* rep_ids, int nrep, const int* nrep_dev,
                            int force_build, int build_mode, int full, int grid, cudaStream_t s,
                            cudaEvent_t after_decide = nullptr, cudaEvent_t after_bin = nullptr);
// min_blocks: the step-kernel variant whose registers are sized for 2 or 3
// resident CTAs per SM
// strategy: 0 = CTA work items with shared-memory staging (k_step), 1 = warp
// tasks gathering through L1/L2 (k_step_w); bit-identical results
// cta_first: grid + 1 item boundaries, CTA b steps items [cta_first[b],
// cta_first[b + 1]) (the CTA strategy; null = equal item counts)
// queue: the CTAs take item blocks from A.blk / A.blk_q instead (the CTA
// strategy; the blocks index `items`)
cudaError_t launch_step(const DevArrays& A, const StepItem* items, int nitems, const int* nitems_dev,
                        const int* cta_first, int queue, int max_staged, int lanes, int min_blocks,
                        int strategy, int threads, int grid, cudaStream_t s);
// the FP64-precision step over its own items (one thread per bead)
cudaError_t launch_step64(const DevArrays& A, const StepItem* items, int nitems, const int* nitems_dev,
                          int grid, cudaStream_t s);
// energies of rep_ids[0..nrep) in slices of kEnergySlice beads; slice_base[k]:
// replica k's first slot in en_part; max_slices: the most slices of any of them
cudaError_t launch_energy(const DevArrays& A, const int* rep_ids, const int* slice_base, int nrep,
                          int max_slices, cudaStream_t s);
cudaError_t launch_observables(const DevArrays& A, const int* rep_ids, int nrep, cudaStream_t s);
cudaError_t launch_pairlist(const DevArrays& A, int r, int off, int n, cudaStream_t s);
// packed (x y z per bead, replicas back to back at 3*poff[k]) <-> device state
cudaError_t launch_scatter_state(const DevArrays& A, const int* ids, int nrep, const long long* poff,
                                 const double* xyz, const double* vel, cudaStream_t s);
cudaError_t launch_gather_state(const DevArrays& A, const int* ids, int nrep, const long long* poff,
                                double* xyz, double* vel, cudaStream_t s);
cudaError_t launch_export(const DevArrays& A, int r, int off, int n, int which, int cap,
                          cudaStream_t s);
int step_kernel_max_smem();
// resident step-kernel CTAs per SM for this configuration
int step_blocks_per_sm(int lanes, int min_blocks, int strategy, int threads, int max_staged);
// block sizes 64..256 (multiples of 32) for every lanes / strategy; 512 for
// the CTA strategy with 1, 2 or 4 lanes per bead
bool step_shape_supported(int lanes, int strategy, int threads);

}  // namespace sop
