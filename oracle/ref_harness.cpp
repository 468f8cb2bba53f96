// Test infrastructure only: an in-process harness around the UNMODIFIED
// SOP-CPU reference sources, which oracle/Makefile compiles from the
// read-only reference tree into oracle/_ref/libsopref.so.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
// only as the checker.  Nothing here is shipped or measured as the product.
//
// The harness calls the reference's own functions (load, set_params,
// update_neighbor_list, update_cell_list, update_pair_list, force_eval,
// energy_eval, underdamped_iteration, calculate_observables) and copies the
// reference's globals in and out through a flat extern "C" surface that
// ctypes can bind.  The step loop in sopref_run() restates the schedule of
// underdamped_ctrl (sop.cpp:93-198) without its file output: local inlup
// starts at 1 (sop.cpp:100), rebuild when inlup % nnlup == 0
// (sop.cpp:156-165), pair-list filter every step (sop.cpp:167-170).
#include <cstring>
#include <cstdio>
#include "global.h"
#include "energy.h"
#include "io.h"
#include "params.h"
#include "neighbor_list.h"
#include "cell_list.h"
#include "sop.h"

extern "C" {

static coord* h_incr = nullptr;
static int h_incr_n = 0;
static int h_inlup = 1;

// Reset the reference's globals to alloc_arrays() defaults, parse the command
// script with read_input() (io.cpp:9-89) and execute its load/set commands
// (sop.cpp:63-71) without the final "run".  Returns the number of beads.
int sopref_load_script(const char* path) {
  alloc_arrays();                 // params.cpp:262-400 (defaults, seed -101)
  nil_att = nil_rep = 0;
  nnl_att = nnl_rep = 0;
  read_input(path);
  for (int i = 1; i <= ncmd; i++) {
    if (!strcmp(cmd[i], "load")) load(i);
    else if (!strcmp(cmd[i], "set")) set_params(i);
  }
  delete[] h_incr;
  h_incr = new coord[nbead + 1];
  h_incr_n = nbead;
  h_inlup = 1;
  return nbead;
}

// The set-up half of underdamped_ctrl (sop.cpp:106-147): zero v and F, build
// the initial neighbor/cell list and pair list, fill the term tables, then
// energy_eval() and force_eval() as on the first call.
void sopref_setup(int do_initial_eval) {
  for (int i = 1; i <= nbead; i++) {
    vel[i].x = vel[i].y = vel[i].z = 0.0;
    force[i].x = force[i].y = force[i].z = 0.0;
  }
  if (neighborlist == 1) { update_neighbor_list(); update_pair_list(); }
  else if (celllist == 1) { update_cell_list(); update_pair_list(); }
  set_potential();
  set_forces();
  if (do_initial_eval) { energy_eval(); force_eval(); }
  h_inlup = 1;
}

// Edit the force-term switches (global.cpp:200-202) and rebuild the table
// (energy.cpp:78-113).  Slot 1 random, 2 FENE, 3 soft-sphere angles, 6 vdw.
void sopref_set_force_terms(int random_on, int fene_on, int ang_on, int vdw_on) {
  force_term_on[1] = random_on;
  force_term_on[2] = fene_on;
  force_term_on[3] = ang_on;
  force_term_on[6] = vdw_on;
  nforce_term = random_on + fene_on + ang_on + vdw_on;
  set_forces();
}

void sopref_neighbor_list() { update_neighbor_list(); }
void sopref_cell_list() { update_cell_list(); }
void sopref_pair_list() { update_pair_list(); }
void sopref_force_eval() { force_eval(); }
void sopref_energy_eval() { energy_eval(); }
void sopref_observables() { calculate_observables(h_incr); }
void sopref_iteration() {
  if (sim_type == 2) overdamped_iteration(h_incr);
  else underdamped_iteration(h_incr);
}

// n iterations of the underdamped_ctrl loop body (sop.cpp:153-172); the
// overdamped_ctrl body (sop.cpp:425-444) has the same schedule.
void sopref_run(int nsteps) {
  for (int s = 0; s < nsteps; s++) {
    if ((h_inlup % nnlup) == 0) {
      if (neighborlist == 1) update_neighbor_list();
      else if (celllist == 1) update_cell_list();
      h_inlup = 0;
    }
    h_inlup++;
    if (neighborlist == 1 || celllist == 1) update_pair_list();
    if (sim_type == 2) overdamped_iteration(h_incr);
    else underdamped_iteration(h_incr);
  }
}

int sopref_get_int(const char* name) {
  if (!strcmp(name, "nbead")) return nbead;
  if (!strcmp(name, "nbnd")) return nbnd;
  if (!strcmp(name, "nang")) return nang;
  if (!strcmp(name, "ncon_att")) return ncon_att;
  if (!strcmp(name, "ncon_rep")) return ncon_rep;
  if (!strcmp(name, "nnl_att")) return nnl_att;
  if (!strcmp(name, "nnl_rep")) return nnl_rep;
  if (!strcmp(name, "nil_att")) return nil_att;
  if (!strcmp(name, "nil_rep")) return nil_rep;
  if (!strcmp(name, "nnlup")) return nnlup;
  if (!strcmp(name, "nup")) return nup;
  if (!strcmp(name, "neighborlist")) return neighborlist;
  if (!strcmp(name, "celllist")) return celllist;
  if (!strcmp(name, "contct_nat")) return contct_nat;
  if (!strcmp(name, "sim_type")) return sim_type;
  if (!strcmp(name, "inlup")) return h_inlup;
  return -1;
}

double sopref_get_double(const char* name) {
  if (!strcmp(name, "e_bnd")) return e_bnd;
  if (!strcmp(name, "e_ang_ss")) return e_ang_ss;
  if (!strcmp(name, "e_vdw_rr")) return e_vdw_rr;
  if (!strcmp(name, "e_vdw_rr_att")) return e_vdw_rr_att;
  if (!strcmp(name, "e_vdw_rr_rep")) return e_vdw_rr_rep;
  if (!strcmp(name, "rna_etot")) return rna_etot;
  if (!strcmp(name, "Q")) return Q;
  if (!strcmp(name, "rgsq")) return rgsq;
  if (!strcmp(name, "kinT")) return kinT;
  if (!strcmp(name, "T")) return T;
  if (!strcmp(name, "h")) return h;
  if (!strcmp(name, "zeta")) return zeta;
  if (!strcmp(name, "a1")) return a1;
  if (!strcmp(name, "a2")) return a2;
  if (!strcmp(name, "a3")) return a3;
  if (!strcmp(name, "a4")) return a4;
  if (!strcmp(name, "a5")) return a5;
  if (!strcmp(name, "boxl")) return boxl;
  if (!strcmp(name, "lcell")) return lcell;
  if (!strcmp(name, "ncell")) return ncell;
  if (!strcmp(name, "nstep")) return nstep;
  return 0.0 / 0.0;
}

void sopref_set_double(const char* name, double v) {
  if (!strcmp(name, "T")) T = v;
  else if (!strcmp(name, "boxl")) boxl = v;
  else if (!strcmp(name, "lcell")) lcell = v;
  else if (!strcmp(name, "ncell")) ncell = v;
}

static coord* coord_array(int which) {
  switch (which) {
    case 0: return pos;
    case 1: return unc_pos;
    case 2: return vel;
    case 3: return force;
    case 4: return h_incr;
    default: return nullptr;
  }
}

// which: 0 pos, 1 unc_pos, 2 vel, 3 force, 4 incr.  out[3*i+k], 0-based beads.
void sopref_get_coords(int which, double* out) {
  coord* c = coord_array(which);
  for (int i = 1; i <= nbead; i++) {
    out[3 * (i - 1) + 0] = c[i].x;
    out[3 * (i - 1) + 1] = c[i].y;
    out[3 * (i - 1) + 2] = c[i].z;
  }
}

void sopref_set_coords(int which, const double* in) {
  coord* c = coord_array(which);
  for (int i = 1; i <= nbead; i++) {
    c[i].x = in[3 * (i - 1) + 0];
    c[i].y = in[3 * (i - 1) + 1];
    c[i].z = in[3 * (i - 1) + 2];
  }
}

// which: 0 neighbor list att, 1 neighbor list rep, 2 pair list att, 3 pair
// list rep.  Writes 1-based bead indices in list order; returns the count.
int sopref_get_list(int which, int* ii, int* jj) {
  int n = 0;
  const int* a = nullptr;
  const int* b = nullptr;
  switch (which) {
    case 0: n = nnl_att; a = ibead_neighbor_list_att; b = jbead_neighbor_list_att; break;
    case 1: n = nnl_rep; a = ibead_neighbor_list_rep; b = jbead_neighbor_list_rep; break;
    case 2: n = nil_att; a = ibead_pair_list_att; b = jbead_pair_list_att; break;
    case 3: n = nil_rep; a = ibead_pair_list_rep; b = jbead_pair_list_rep; break;
    default: return -1;
  }
  if (ii && jj) {
    for (int k = 1; k <= n; k++) { ii[k - 1] = a[k]; jj[k - 1] = b[k]; }
  }
  return n;
}

}  // extern "C"
