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
  RepDev* rep;        // replica descriptors
  long long cap;      // bead capacity (SoA stride)
  unsigned long long* pairs_out;  // export buffer (i<<32|j)
  int* pairs_cnt;
  int* err;           // engine-wide error word (bounded waits that gave up)
  int4* units;        // per-step work queue (builds in slices, energies, observables)
  int* unit_cnt;      // units queued this step
  int* unit_exit;     // k_build CTAs finished (the last one resets the queue)
  int* slice_done;    // per replica: build slices finished this step
  int unit_cap;
  int* done_list;     // replicas whose run window closed (final step taken)
  int* done_cnt;
  int done_cap;
};

constexpr int kSliceBeads = 128;      // beads per list-build work unit

// Work item of the step kernel: beads [b0,b1) of replica r; staged = the
// replica's positions fit in shared memory.
struct StepItem {
  int r, b0, b1, staged;
};

constexpr int kStageMax = 6144;       // beads staged in shared memory (192 KB)
constexpr int kBuildMax = 8192;       // beads per single-CTA list build
constexpr int kMaxCells = 4096;       // cells of one list-build grid
constexpr int kBuildThreads = 512;

void upload_tables(const FFTables& t, cudaStream_t s);
// Opt the kernels into `optin_bytes` of shared memory per block (once per device).
cudaError_t init_kernels(int optin_bytes);

// Prologue + list build: one persistent CTA group over `nrep` replica ids.
// force_build: build for every listed replica from the CURRENT buffer
// (reference-named list updates), else the step cadence decides.
// nrep / nitems: host counts (grid sizing); *_dev: the same counts in device
// memory, read by the kernels when given (graphs survive layout changes).
cudaError_t launch_prologue(const DevArrays& A, const int* rep_ids, int nrep, const int* nrep_dev,
                            int max_n, int force_build, int build_mode, int grid, cudaStream_t s);
cudaError_t launch_step(const DevArrays& A, const StepItem* items, int nitems, const int* nitems_dev,
                        int max_staged, int lanes, int threads, int grid, cudaStream_t s);
cudaError_t launch_energy(const DevArrays& A, const int* rep_ids, int nrep, cudaStream_t s);
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
int step_blocks_per_sm(int lanes, int threads, int max_staged);

}  // namespace sop
