/* Test infrastructure only: the CPU oracle for the SOP hot path.
 *
 * A reentrant C restatement of SOP-CPU's neighbor list, cell list, pair-list
 * filter, force terms, energy terms, observables and underdamped integrator,
 * keeping the reference's FP64 operation order so that, built with
 * -ffp-contract=off, its forces, energies and lists equal the compiled
 * reference's bit for bit on the same inputs (checked by tests/test_oracle.py
 * against oracle/_ref and the committed golden vectors).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it, and only as the checker or the timed CPU baseline.  The GPU
 * product never links or calls it.
 *
 * Conventions: arrays are 0-based, coordinates interleaved xyz (3*nbead);
 * list outputs use the reference's 1-based bead numbers.  Noise uses the same
 * counter-based Philox-4x32-10 stream as the GPU engine (the reference's
 * sequential ran2/gasdev stream cannot be matched in parallel), so noise-on
 * parity is statistical.
 */
#ifndef SOP_ORACLE_H
#define SOP_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct sopo_sys sopo_sys;

sopo_sys* sopo_create(void);
void sopo_destroy(sopo_sys* s);

/* Reference command script (io.cpp:9-89) with its load/set commands
 * (params.cpp:12-260); the trailing "run" is not executed.  0 on success. */
int sopo_load_script(sopo_sys* s, const char* path);

/* Direct construction.  Candidates follow the vdw-file rule: a candidate is
 * native iff r < rcut_nat[ti][tj] (params.cpp:197).  Bead indices 0-based. */
int sopo_set_topology(sopo_sys* s, int nbead,
                      int nbnd, const int* ib, const int* jb, const double* r0,
                      int nang, const int* ia, const int* ja, const int* ka,
                      int ncand, const int* ic, const int* jc, const double* rc,
                      const int* ti, const int* tj);
/* Candidate set generated implicitly: every pair (i<j) with chain[i]!=chain[j]
 * or j-i>2, in lexicographic order; natives are those with r<rcut_nat, taken
 * from the supplied native-distance arrays (others non-native).  type[] per
 * bead; chain may be NULL (one chain).  Natives must be listed i<j. */
int sopo_set_topology_implicit(sopo_sys* s, int nbead, const int* type, const int* chain,
                               int nbnd, const int* ib, const int* jb, const double* r0,
                               int nang, const int* ia, const int* ja, const int* ka,
                               int nnat, const int* in_, const int* jn, const double* rn);
/* The implicit candidate set restricted, for large systems, to the pairs
 * closer than `cutoff` at positions xyz (found through a cell grid), plus
 * every native pair; lexicographic order as above, so every list and sum the
 * reference forms over the full set is formed over this one in the same order
 * as long as no pair beyond `cutoff` could enter a list (the caller picks the
 * cutoff above the list cutoffs plus the motion it runs).  The
 * reference's own large-N recipe: pair lists filled from a CPU cell list. */
int sopo_set_topology_pruned(sopo_sys* s, int nbead, const int* type, const int* chain,
                             int nbnd, const int* ib, const int* jb, const double* r0,
                             int nang, const int* ia, const int* ja, const int* ka,
                             int nnat, const int* in_, const int* jn, const double* rn,
                             const double* xyz, double cutoff);

/* which: 0 pos, 1 unc_pos, 2 vel, 3 force, 4 incr (3*nbead doubles) */
int sopo_set_coords(sopo_sys* s, int which, const double* xyz);
int sopo_get_coords(const sopo_sys* s, int which, double* xyz);

/* Scalars by name: T, zeta, h, halfh, a1..a5, boxl, ncell, lcell, nstep, nup,
 * nnlup, run, seed, neighborlist, celllist, sim_type, k_bnd, R0, and the
 * pulling term pull_force (kcal/mol/A, 0 = off), pull_i, pull_j (<0: last).
 * "zeta"/"t_step"/"dynamics" follow the set-command side effects (params.cpp:
 * 84-98) only through sopo_set_command(). */
int sopo_set_param(sopo_sys* s, const char* name, double v);
double sopo_get_param(const sopo_sys* s, const char* name);
/* Apply one "set <key> <value>" exactly as set_params (params.cpp:12-101). */
int sopo_set_command(sopo_sys* s, const char* key, const char* value);

void sopo_set_force_terms(sopo_sys* s, int random_on, int fene_on, int ang_on, int vdw_on);

void sopo_setup(sopo_sys* s, int do_initial_eval);   /* underdamped_ctrl set-up */
void sopo_neighbor_list(sopo_sys* s);                 /* neighbor_list.cpp:6-117 */
void sopo_cell_list(sopo_sys* s);                     /* cell_list.cpp:6-98      */
void sopo_pair_list(sopo_sys* s);                     /* sop.cpp:473-553         */
void sopo_force_eval(sopo_sys* s);                    /* energy.cpp:21-45        */
void sopo_energy_eval(sopo_sys* s);                   /* energy.cpp:6-19         */
void sopo_observables(sopo_sys* s);                   /* sop.cpp:200-279         */
void sopo_iteration(sopo_sys* s);                     /* sop.cpp:282-329         */
void sopo_run(sopo_sys* s, int nsteps);               /* sop.cpp:153-172 loop    */

/* which: 0 nl att, 1 nl rep, 2 pl att, 3 pl rep; 1-based beads; returns count */
int sopo_get_list(const sopo_sys* s, int which, int* ii, int* jj);
int sopo_get_count(const sopo_sys* s, const char* name);
/* e_bnd, e_ang_ss, e_vdw_rr, e_vdw_rr_att, e_vdw_rr_rep, rna_etot, Q, rgsq, kinT */
double sopo_get_energy(const sopo_sys* s, const char* name);

/* Run n systems for nsteps each on nthreads host threads (one system per
 * thread at a time); returns wall seconds.  The CPU baseline. */
double sopo_run_many(sopo_sys** systems, int n, int nsteps, int nthreads);

/* Philox-4x32-10 (Salmon et al., SC'11), exposed for known-answer tests. */
void sopo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
