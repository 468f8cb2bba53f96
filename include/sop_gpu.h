/* sop_gpu.h -- C ABI of the GB300 SOP engine (libsopgpu.so).
 *
 * One engine owns one CUDA device, one stream and all device memory of the
 * systems ("replicas") admitted to it.  Every entry point returns an int
 * status (SOP_OK or a negative SOP_ERR_*); no C++ exception crosses the ABI.
 * An engine is driven by one host thread at a time.  Bead indices are 0-based
 * in arrays; pair lists handed back use the reference's 1-based numbering.
 *
 * Reference interfaces replaced (SOP-CPU, file:line):
 *   update_neighbor_list()        neighbor_list.cpp:6    -> sop_update_neighbor_list
 *   update_cell_list()            cell_list.cpp:6        -> sop_update_cell_list
 *   update_pair_list()            sop.cpp:473            -> sop_update_pair_list
 *   force_eval() / set_forces()   energy.cpp:21, 78      -> sop_force_eval, sop_params.force_terms
 *   energy_eval() / set_potential energy.cpp:6, 47       -> sop_energy_eval
 *   underdamped_iteration(coord*) sop.cpp:282            -> sop_underdamped_iteration
 *   calculate_observables(coord*) sop.cpp:200            -> sop_observables
 *   underdamped_ctrl() step loop  sop.cpp:93-198         -> sop_run_plain (one system),
 *                                                           sop_run (all systems, batched)
 *   load bonds/angles/vdw/init    params.cpp:110-260     -> sop_replica_add (arrays)
 *   set <keyword>                 params.cpp:12-101      -> sop_params
 */
#ifndef SOP_GPU_H
#define SOP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define SOP_OK 0
#define SOP_ERR_ARG -1         /* bad argument (null pointer, size, index)      */
#define SOP_ERR_CUDA -2        /* a CUDA runtime call failed                    */
#define SOP_ERR_NOMEM -3       /* device or host allocation failed              */
#define SOP_ERR_STATE -4       /* call not valid in the current state           */
#define SOP_ERR_OVERFLOW -5    /* a neighbor-list row or output buffer is full  */
#define SOP_ERR_UNSUPPORTED -6 /* input outside what the engine implements      */
#define SOP_ERR_NODEV -7       /* no usable CUDA device                         */
#define SOP_ERR_REPLICA -8     /* a replica carries an error status (see below) */
#define SOP_ERR_FULL -9        /* no room: admission refused, retry later        */
#define SOP_ERR_TIMEOUT -10    /* a bounded device-side wait ran out; the replicas
                                  stepped in that call are in an undefined state */
#define SOP_ERR_INDEX -11      /* checked build (libsopgpu_checked.so): a list,
                                  bin, native, bond or angle entry named a bead
                                  outside its replica; the entry was skipped and
                                  the stepped replicas are in an undefined state */

/* per-replica status bits (sop_replica_status) */
#define SOP_ST_NONFINITE 0x1     /* NaN/inf force or position                   */
#define SOP_ST_FENE 0x2          /* a bond stretched to |d - r0| >= R0           */
#define SOP_ST_LIST_OVERFLOW 0x4 /* a neighbor-list row overflowed; frozen       */
#define SOP_ST_PERIODIC 0x8      /* reserved: no longer raised (a replica whose
                                    extent reaches boxl/2 steps with minimum
                                    images, global.cpp:223-227)                 */
#define SOP_ST_GRID 0x10         /* cell grid larger than the engine supports    */

/* list modes: which pair search feeds the per-step pair-list filter */
#define SOP_LIST_NONE 0     /* cutofftype unset: every candidate interacts     */
#define SOP_LIST_NEIGHBOR 1 /* 3.2x neighbor list every nnlup steps (reference) */
#define SOP_LIST_CELL 2     /* cell-adjacency screen every nnlup steps          */
#define SOP_LIST_SKIN 3     /* Verlet list at 2.5x + skin, rebuilt on displacement */

/* force terms (energy.cpp:78-113 switch slots 1, 2, 3, 6) */
#define SOP_TERM_RANDOM 0x1
#define SOP_TERM_FENE 0x2
#define SOP_TERM_ANGLE 0x4
#define SOP_TERM_VDW 0x8
#define SOP_TERM_ALL 0xF

/* integrators (set dynamics, params.cpp:19-31) */
#define SOP_DYN_UNDERDAMPED 0 /* underdamped_iteration, sop.cpp:282-329 */
#define SOP_DYN_OVERDAMPED 1  /* overdamped_iteration, sop.cpp:331-363  */

/* integrator precision */
#define SOP_PREC_MIXED 0 /* FP32 pair forces, FP64 positions (default)      */
#define SOP_PREC_FP64 1  /* FP64 pair forces and update (drift reference)   */

/* Run and force-field parameters of one system: the reference globals the
 * hot path reads (params.cpp:262-400 defaults via sop_params_default). */
typedef struct sop_params {
  double T;       /* temperature, kcal/mol                                  */
  double zeta;    /* friction                                               */
  double h;       /* time step                                              */
  double a1, a2, a3, a4; /* integrator constants (params.cpp:22-27, 84-98)  */
  double boxl;    /* box edge for the minimum image                         */
  double lcell;   /* cell edge of the cell-adjacency mode (boxl/ncell)      */
  double ncell;   /* cells per box edge                                     */
  double k_bnd, R0;          /* FENE (params.cpp:268-271)                    */
  double sigma_ss, epsilon_ss; /* i,i+2 soft sphere (params.cpp:289-293)     */
  double skin;    /* SOP_LIST_SKIN: list cutoff is 2.5 sigma + skin, A       */
  double cell_edge; /* edge of the list build's cell grid, A: at least half
                       the list cutoff (smaller values and 0 give that half;
                       5x5x5 stencil), from the cutoff up a 3x3x3 stencil   */
  double pull_force; /* constant force on the two termini along their
                        separation, kcal/mol/A (0 = off; no reference term)  */
  uint64_t seed;  /* counter-based noise key                                */
  int nnlup;      /* list update period in steps                            */
  int nup;        /* output period in steps (energies, observables)         */
  int list_mode;  /* SOP_LIST_*                                             */
  int force_terms; /* SOP_TERM_* mask                                       */
  int precision;  /* SOP_PREC_*                                             */
  int pull_i, pull_j; /* pulled beads (default first and last)              */
  int dynamics;   /* SOP_DYN_UNDERDAMPED (sim_type 1) or SOP_DYN_OVERDAMPED (2) */
  double a5;      /* overdamped step factor h/zeta (params.cpp:31, 91, 392)  */
} sop_params;

/* One system: topology + initial state.  All arrays 0-based, borrowed. */
typedef struct sop_system_desc {
  int nbead;
  const double* xyz;       /* initial unc_pos, 3*nbead (pos = unc_pos)       */
  const double* vel;       /* initial velocities or NULL (zero)              */
  const int* bead_type;    /* 1 or 2 per bead, or NULL (all 1)               */
  const int* chain;        /* chain id per bead, or NULL (one chain)         */
  int nbnd; const int* ib; const int* jb; const double* r0;   /* FENE bonds  */
  int nang; const int* ia; const int* ka;                     /* i,k of angles */
  int nnat; const int* in_; const int* jn; const double* rn;  /* natives     */
  /* Non-native candidates are implicit: every pair with chain[i]!=chain[j] or
   * |i-j|>2 that is not native.  Pairs of that set that must NOT interact
   * (a vdw file listing fewer candidates) are given here: */
  int nexcl; const int* ie; const int* je;
  sop_params params;
} sop_system_desc;

typedef struct sop_engine sop_engine;

typedef struct sop_engine_config {
  int device;            /* CUDA ordinal                                       */
  int max_beads;         /* bead capacity of the packed arrays (0 = 1<<21)     */
  int max_replicas;      /* replica slots (0 = 4096)                           */
  int64_t max_list_entries; /* neighbor-list entry capacity (0 = 64 per bead)  */
  int block_threads;     /* fused step kernel block size, 64..512, multiple of
                            32 (0 = 256); 512 with lanes_per_bead 1, 2 or 4
                            and step_strategy 0 only (else UNSUPPORTED)     */
  int lanes_per_bead;    /* lanes cooperating on one bead: 1,2,4,8,16 (0 = 2)  */
  int graph_steps;       /* steps captured per CUDA graph launch (0 = 20)      */
  int stage_limit;       /* largest replica (beads) whose positions the step
                            kernel stages in shared memory by TMA; larger ones
                            are gathered through L1 (0 = 1664, <0 = never)    */
  int chunk_beads;       /* beads per step-kernel work item (0 = 128)          */
  int build_slice_beads; /* beads per list-build work unit, >= 16 (0 = 32)     */
  int step_min_blocks;   /* step-kernel variant: registers sized for 2, 3 or 4
                            resident CTAs per SM (0 = 4; 4 needs a stage
                            limit <= ~1700 to fit, CTA items only)            */
  int step_strategy;     /* 0: CTA work items staged in shared memory; 1: warp
                            tasks gathering through L1/L2 (same results)      */
  int group_rebuild_pct; /* skin-mode replicas whose displacement passed this %
                            of their trigger distance rebuild together with any
                            replica that must, so builds cluster into fewer
                            steps; forces and energies are exact integer sums,
                            so trajectories do not depend on it (0 = 50,
                            <0 = off)                                         */
  int lean_prep;         /* a step's preparation kernel skips its work-queue
                            phase when the previous step flagged no possible
                            work (no skin trigger, output, observables or
                            cadence build): 0 = on, <0 = off (same results)   */
  /* Limits of the two device-side waits (0 = 2 s each; at most 60 s).  Neither
   * is expected to run out: a CTA of the preparation kernel waits for a work
   * unit another CTA is still publishing, and a step-kernel CTA waits for
   * its bulk copy of positions into shared memory.  A wait that runs out
   * records it, lets its copies in flight land, and returns; the call then
   * fails with SOP_ERR_TIMEOUT and the engine clears the queue, so later
   * calls work (restore or re-add the replicas that call stepped). */
  int64_t queue_wait_ns;
  int64_t stage_wait_ns;
  /* How the batched step's work items (sorted by replica size, largest
   * first) are split into one contiguous block per CTA: <0 = equal item
   * counts; >= 0 = equal estimated cost, an item costing its beads plus this
   * many bead equivalents for the fixed per-item work (0 = 512).  Same
   * results either way. */
  int item_cost_beads;
  /* Far entries of the list rows (farther than the pair cutoff plus a band
   * width -- half the skin, or 0.35 sigma for cadence lists -- at the
   * build) are stored last, and the step skips them while no bead of the
   * replica has moved half the band width since the build: they cannot be
   * in the pair list then.  0 = on, <0 = off (same results either way). */
  int row_bands;
  /* Step CTAs take item blocks of about equal estimated cost
   * (item_cost_beads >= 0) from a queue, this many blocks per CTA, rather
   * than one fixed block each: CTAs whose items run long take fewer.  0 =
   * automatic: the queue with 8 blocks per CTA (one item each while the
   * layout has at most 8 items per CTA) while some replica is above the
   * stage limit (its items gather through L1/L2 and cost more per bead than
   * the split assumes), else one fixed block per CTA; <0 = one fixed block
   * per CTA.  Same results either way. */
  int queue_blocks;
} sop_engine_config;

/* ---- engine -------------------------------------------------------------- */
const char* sop_version(void);
/* sizeof one of this header's structs by name ("sop_params",
 * "sop_system_desc", "sop_engine_config", "sop_server_config",
 * "sop_request_result"), or -1 for any other name: a binding in another
 * language checks its struct layouts against the library it loaded. */
int sop_struct_size(const char* name);
const char* sop_status_string(int status);
void sop_params_default(sop_params* p);   /* params.cpp:262-400 defaults      */
void sop_engine_config_default(sop_engine_config* c);
int sop_engine_create(const sop_engine_config* cfg, sop_engine** out);
int sop_engine_destroy(sop_engine* e);
int sop_engine_sync(sop_engine* e);
/* bytes of device memory a system would take (admission by memory) */
int sop_system_bytes(const sop_engine* e, const sop_system_desc* d, int64_t* bytes);
int sop_engine_free_bytes(const sop_engine* e, int64_t* bytes);
/* kernels launched by this engine since creation (all entry points) */
int sop_engine_launches(const sop_engine* e, int64_t* launches);
/* preparation launches that skipped the work-queue phase but found queued work
 * all the same and ran it in one CTA (correct, slower; expected to stay 0) */
int sop_engine_prep_fallbacks(sop_engine* e, int64_t* count);
/* Diagnostics, no reference counterpart: host-controlled stalls that make the
 * device-side waits above run out, for tests of the timeout path (no fault,
 * no unbounded wait).  publish_delay_ns (0..1e9): every preparation CTA that
 * publishes list-build units first waits that long; skip_stage_copy != 0: the
 * step kernel's CTAs expect their position copies but do not issue them.
 * Both 0 = normal operation.  Call between runs. */
int sop_engine_inject_stall(sop_engine* e, int64_t publish_delay_ns, int skip_stage_copy);
/* Which waits ran out in the call that last returned SOP_ERR_TIMEOUT:
 * bit 0 the step kernel's copy wait, bit 1 the preparation kernel's queue
 * wait (0 if none since the engine was created). */
int sop_engine_wait_errors(sop_engine* e, int* bits);

/* ---- replicas ------------------------------------------------------------- */
/* Upload a system; builds its lists at the initial positions (the set-up of
 * underdamped_ctrl, sop.cpp:117-125) and evaluates nothing else. */
int sop_replica_add(sop_engine* e, const sop_system_desc* d, int* replica);

/* Admission in two halves, for servers: sop_prepare does the host work
 * (topology, row sizing, device bytes) without touching any device, so it
 * can run while the GPU steps other replicas; sop_replicas_admit places
 * prepared systems in order until a slot or an arena is missing (*admitted
 * of them; SOP_ERR_FULL if none), builds all their lists in one launch and,
 * when nsteps is given, opens each one's run window of nsteps[k] steps
 * (as sop_replica_start).  A prepared system may be admitted any number of
 * times (to any engine) and is released with sop_prepared_free. */
typedef struct sop_prepared sop_prepared;
int sop_prepare(const sop_system_desc* d, sop_prepared** out);
int sop_prepared_bytes(const sop_prepared* p, int64_t* bytes);
void sop_prepared_free(sop_prepared* p);
int sop_replicas_admit(sop_engine* e, sop_prepared* const* p, const int64_t* nsteps, int n,
                       int* replicas, int* admitted);
/* Final energies (6 per replica), observables (5) and status of each listed
 * replica, computed in one pass, then the replicas are removed.  Any output
 * pointer may be NULL. */
int sop_replicas_retire(sop_engine* e, const int* replicas, int n, double* energy6, double* obs5,
                        int* status);
int sop_replica_remove(sop_engine* e, int replica);
int sop_replica_set_params(sop_engine* e, int replica, const sop_params* p);
int sop_replica_get_params(sop_engine* e, int replica, sop_params* p);
/* host copies (any pointer may be NULL): wrapped pos, unc_pos, vel (3*nbead) */
int sop_replica_get_state(sop_engine* e, int replica, double* pos, double* unc_pos, double* vel);
/* overwrite unc_pos (and pos) and velocities; vel NULL = zero */
int sop_replica_set_state(sop_engine* e, int replica, const double* unc_pos, const double* vel);
int sop_replica_status(sop_engine* e, int replica, int* status, int64_t* steps_done);
/* diagnostics: out[0..7] = nbead, list row capacity L, longest row at the last
 * build, list builds so far, iteration t, status bits, native pairs, offset */
int sop_replica_info(sop_engine* e, int replica, int64_t* out);
int sop_replica_count(const sop_engine* e, int* n);

/* ---- reference-named operations on one replica (synchronous) -------------- */
int sop_update_neighbor_list(sop_engine* e, int replica);   /* neighbor_list.cpp:6 */
int sop_update_cell_list(sop_engine* e, int replica);       /* cell_list.cpp:6     */
int sop_update_pair_list(sop_engine* e, int replica);       /* sop.cpp:473         */
/* which: 0 neighbor att, 1 neighbor rep, 2 pair att, 3 pair rep.  Writes up to
 * cap pairs (1-based, i<j) sorted by (i,j); *count gets the full count. */
int sop_get_pair_list(sop_engine* e, int replica, int which, int* ii, int* jj, int cap, int* count);
/* forces at the current positions with the current pair list (energy.cpp:21);
 * the random term draws force evaluation number `noise_index` of the stream */
int sop_force_eval(sop_engine* e, int replica, double* force_xyz);
/* out[0..5] = e_bnd, e_ang_ss, e_vdw_rr, e_vdw_rr_att, e_vdw_rr_rep, rna_etot */
int sop_energy_eval(sop_engine* e, int replica, double* out);
/* one underdamped_iteration at the current pair list (sop.cpp:282-329) */
int sop_underdamped_iteration(sop_engine* e, int replica);
/* out[0..4] = Q, contct_nat, rgsq, kinT, end-to-end distance */
int sop_observables(sop_engine* e, int replica, double* out);

/* ---- stepping -------------------------------------------------------------- */
/* The plain single-system path: the underdamped_ctrl loop for one replica,
 * one kernel sequence per step, no graph, no batching. */
int sop_run_plain(sop_engine* e, int replica, int64_t nsteps);
/* All active replicas, packed into one persistent kernel per step, with
 * per-replica rebuilds, the step loop captured in CUDA graphs. */
int sop_run(sop_engine* e, int64_t nsteps);
/* Per-replica run windows for continuous batching: sop_replica_start opens
 * a window of nsteps for one replica (restart semantics: its first step
 * re-evaluates the force at the stored state); sop_run_chunk advances every
 * open window by up to `steps` batched steps; replicas whose window closed
 * during the chunk are returned in finished[0..*nfinished) (cap entries). */
int sop_replica_start(sop_engine* e, int replica, int64_t nsteps);
int sop_run_chunk(sop_engine* e, int64_t steps, int* finished, int cap, int* nfinished);
/* sop_run_chunk in two halves: _begin launches the steps and returns; the
 * host may then do host-only work (sop_prepare) while the GPU runs;
 * _end waits and hands back the replicas whose window closed.  Between the
 * two, no other call may use the engine. */
int sop_run_chunk_begin(sop_engine* e, int64_t steps);
int sop_run_chunk_end(sop_engine* e, int* finished, int cap, int* nfinished);
/* End-to-end call with HOST buffers (restart semantics, sop.cpp:132-147):
 * load unc_pos/vel of every active replica (packed in replica-id order,
 * 3*nbead each), evaluate the initial force, run nsteps, write them back. */
int sop_run_host(sop_engine* e, const double* xyz_in, const double* vel_in, int64_t nsteps,
                 double* xyz_out, double* vel_out);
/* device time of the last sop_run (ms) and of its fused step kernels (ms) */
int sop_last_run_timing(sop_engine* e, double* total_ms, double* step_kernel_ms,
                        int64_t* step_kernel_launches);
/* nsteps batched steps launched without a graph, with CUDA events around
 * each kernel: mean device ms per launch of the fused step kernel and of the
 * prologue (bookkeeping + list builds + output-step energies). */
int sop_profile_steps(sop_engine* e, int64_t nsteps, double* step_kernel_ms, double* prologue_ms);
/* The same run split per kernel, mean ms per step: ms[0] launch gap before
 * the preparation (~0), ms[1] k_prep (bookkeeping, cell binning, list slices,
 * energies, observables: one kernel), ms[2] the gap after it (~0), ms[3]
 * k_step. */
int sop_profile_steps_ex(sop_engine* e, int64_t nsteps, double* ms);

/* The energies the last output step computed (step t with t % nup == 0 or the
 * final step of a run window), with the pair list that step's force used, as
 * the reference's energy_eval at an nup step (sop.cpp:174-181); also the
 * stored observables.  Either pointer may be NULL. */
int sop_replica_outputs(sop_engine* e, int replica, double* energy6, double* obs5);
/* Set the step counter (the force-evaluation index that keys the noise
 * stream) of a replica between runs, e.g. to istep_restart on a restart
 * (sop.cpp:132-140). */
int sop_replica_set_step(sop_engine* e, int replica, int64_t step);

/* ---- checkpoint / restart ------------------------------------------------------ */
/* Exact snapshot of one replica (both position buffers, increments,
 * velocities, list rows with their pair-list bits, native flags, skin
 * references, step / noise counters and cadence), in place of the reference's
 * restart files (sop.cpp:132-140: coordinates, velocities, generator state).
 * buf == NULL: *size receives the bytes needed.  SOP_ERR_OVERFLOW if cap is
 * too small.  Restoring into a replica of the same system (any engine, any
 * launch configuration) continues the run bit for bit; the target keeps its
 * own parameters.  Call between runs or run chunks. */
int sop_replica_checkpoint(sop_engine* e, int replica, void* buf, int64_t cap, int64_t* size);
int sop_replica_restore(sop_engine* e, int replica, const void* buf, int64_t size);

/* ---- autotuner --------------------------------------------------------------- */
/* No reference counterpart.  Time the batched step of the active replicas
 * over candidate launch shapes (step strategy, stage limit, beads per work
 * item, block size 64-512, lanes per bead, register budget, beads per
 * list-build slice, rebuild grouping; one choice for the engine) and, for
 * replicas in skin mode, list skins 1-4 A and cell edges 6-12 A (one choice
 * per size bucket
 * [1,256) [256,1024) [1024,4096) [4096,...)); adopt the fastest.
 * Every trial runs steps_per_trial warm-up plus steps_per_trial timed REAL
 * steps inside one run window, so the call advances each active replica
 * exactly as one sop_run of the reported step count would -- bit for bit,
 * whatever is chosen: forces and pair energies are exact fixed-point sums of
 * their contributions and the pair filter is exact at every step, so no knob
 * moves a trajectory.  Call between runs.  report (may be NULL) receives a
 * text table of the trials.  sop_autotune tunes both groups. */
#define SOP_TUNE_SHAPE 1
#define SOP_TUNE_LISTS 2
int sop_autotune(sop_engine* e, int steps_per_trial, char* report, int report_cap);
int sop_autotune_ex(sop_engine* e, int steps_per_trial, int what, char* report, int report_cap);

/* ---- continuous-batching server ----------------------------------------------- */
typedef struct sop_server sop_server;
typedef struct sop_server_config {
  sop_engine_config engine;
  int max_active;          /* replica slots in flight (0 = 1024)              */
  int64_t memory_budget;   /* device bytes admissions may use (0 = no budget:
                              the engine's arenas are the only limit)        */
  int chunk_steps;         /* steps between admission/retirement points (0=200) */
} sop_server_config;
typedef struct sop_request_result {
  int64_t request_id;
  int status;              /* SOP_OK or an error code                         */
  int replica_status;
  int nbead;
  int64_t steps;
  double submit_s, start_s, finish_s; /* server clock, seconds              */
  double energy[6];        /* final energies (sop_energy_eval layout)         */
  double observables[5];   /* final observables (sop_observables layout)      */
} sop_request_result;
int sop_server_create(const sop_server_config* cfg, sop_server** out);
int sop_server_destroy(sop_server* s);
/* queue a request; the system is prepared on the host (topology, row sizing,
 * device bytes) and the desc arrays need not outlive the call. */
int sop_server_submit(sop_server* s, const sop_system_desc* d, int64_t nsteps, int64_t* request_id);
/* end the chunk the previous pump launched, retire the requests it finished,
 * admit queued requests, launch the next chunk and return while it runs;
 * *pending = requests still queued or running. */
int sop_server_pump(sop_server* s, int* pending);
/* completed requests since the last call */
int sop_server_poll(sop_server* s, sop_request_result* out, int cap, int* n);
/* seconds since the server was created (the clock of submit/start/finish) */
int sop_server_clock(sop_server* s, double* now_s);
int sop_server_stats(sop_server* s, int64_t* bead_steps, int* active, int* queued);
/* Host time the pumps spent admitting, running chunks and retiring (s). */
int sop_server_timing(sop_server* s, double* admit_s, double* run_s, double* retire_s);

/* ---- synthetic systems (test and bench workloads) -------------------------------- */
/* Seeded self-avoiding 3.8 A chain compacted by 2000-step-style minimisation. */
int sop_synth_chain(uint64_t seed, int nbead, int compact_steps, double* xyz);
/* nchain chains of chain_len beads packed into one globule. */
int sop_synth_globule(uint64_t seed, int nchain, int chain_len, int compact_steps, double* xyz);

/* ---- neighbor list without allocation ---------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: hosts whose device memory belongs to their own pool, and loops that
 * cannot take the device-wide synchronization cudaMalloc / cudaFree may
 * cause.  Every input and output is a device pointer owned by the caller; the
 * only other memory used is a fixed static scratch array in the library
 * (about 0.6 MB, held on each GPU that loads the library until exit), sized
 * for SOP_NOALLOC_MAX_BEADS.
 *   xyz      3*nbead doubles, x y z per bead (unc_pos), |x| < 1e6 A
 *   bead_type, chain   nbead ints each, or NULL (all type 1, one chain);
 *                      types must be 1 or 2
 *   nat_ptr, nat_idx   natives in CSR form (nat_ptr[nbead+1], partners of
 *                      bead i in nat_idx[nat_ptr[i]..nat_ptr[i+1]), sorted),
 *                      both listed per bead, or NULL for none
 *   pairs    2*cap ints: 1-based (i, j), i < j, in no particular order
 *   count    1 int: number of pairs found (only the first cap are written),
 *            or, when the input is rejected and no pair is written, -1
 *            (a position not finite or beyond 1e6 A) or -2 (a bead type
 *            other than 1 or 2); read it after the stream has finished
 *   stream   a cudaStream_t, or NULL for the default stream
 * Result: the engine's non-native neighbor list of the system, the set
 * sop_update_neighbor_list + sop_get_pair_list(which=1) give: pairs on
 * different chains or |i-j| > 2 apart, not native, with d^2 < (3.2 sigma)^2
 * in FP64, open boundaries (no box and no minimum image: a system that
 * needs images, extent near half its box, belongs in the engine).  nbead >
 * SOP_NOALLOC_MAX_BEADS returns SOP_ERR_UNSUPPORTED.  The first call on a
 * device looks up the scratch address there; make it before any stream
 * capture.  Calls share the scratch: calls that overlap on the GPU
 * (different streams, or devices sharing it) race and must be ordered. */
#define SOP_NOALLOC_MAX_BEADS 16384
int sop_neighbor_list_noalloc(const double* xyz, int nbead, const int* bead_type, const int* chain,
                              const int* nat_ptr, const int* nat_idx, int* pairs, int cap,
                              int* count, void* stream);

/* ---- measurement probe -------------------------------------------------------------- */
/* No counterpart in the reference.  L2 read bandwidth of `device` in GB/s: a
 * buffer of `bytes` (1-96 MB, so it stays in L2) read `reps` times by one
 * kernel with L1-bypassing 16-byte loads, best of five launches, CUDA events.
 * The benchmark's denominator for kernels whose working set lives in L2. */
int sop_probe_l2_read(int device, int64_t bytes, int reps, double* gbs);

/* ---- host-side numerics self-checks (no GPU needed) ------------------------------- */
/* split a double into the (hi, lo) float pair the engine stages */
void sop_selftest_split(double x, float* hi, float* lo);
/* three Philox-4x32-10 normals as the step kernel draws them (host build) */
void sop_selftest_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif /* SOP_GPU_H */
