// shim_main.cpp -- driver of the CPU test of gpu_backend.cpp.  It runs the
// reference's own defaults, command-script reader and loaders (params.cpp
// alloc_arrays, io.cpp read_input,
// params.cpp load / set_params) on an input script, attaches the backend
// (which then talks to the recording stub of the C ABI, stub_abi.cpp), calls
// every forwarded entry point once, edits the force-term switches the way a
// reference user does (global.cpp:200-203), and prints the globals the
// backend wrote back.
#include <cstdio>
#include <cstring>

#include "global.h"
#include "io.h"
#include "params.h"

void gpu_attach();
void gpu_detach();
void gpu_begin(long long);
void gpu_steps(long long);
void gpu_output();
void gpu_read_state();
int gpu_force_terms();
void update_neighbor_list();
void update_cell_list();
void update_pair_list();
void force_eval();
void energy_eval();
void underdamped_iteration(coord*);
void overdamped_iteration(coord*);

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  alloc_arrays();  // the reference's defaults, as its main does (sop.cpp:34-35)
  read_input(argv[1]);
  for (int i = 1; i <= ncmd; i++) {
    if (!std::strcmp(cmd[i], "load")) load(i);
    else if (!std::strcmp(cmd[i], "set")) set_params(i);
  }
  gpu_attach();
  std::printf("terms %d\n", gpu_force_terms());
  update_neighbor_list();
  update_cell_list();
  update_pair_list();
  force_eval();
  std::printf("force1 %.17g %.17g %.17g\n", force[1].x, force[1].y, force[1].z);
  std::printf("forceN %.17g %.17g %.17g\n", force[nbead].x, force[nbead].y, force[nbead].z);
  energy_eval();
  std::printf("energy %g %g %g %g %g %g\n", e_bnd, e_ang_ss, e_vdw_rr, e_vdw_rr_att, e_vdw_rr_rep,
              rna_etot);
  // random term off, the remaining three terms called (noise-off dynamics)
  force_term_on[1] = 0;
  nforce_term = 3;
  std::printf("terms %d\n", gpu_force_terms());
  force_eval();
  // only FENE: slot 2 on, others off
  force_term_on[3] = 0;
  force_term_on[6] = 0;
  nforce_term = 1;
  std::printf("terms %d\n", gpu_force_terms());
  force_eval();
  force_term_on[1] = force_term_on[3] = force_term_on[6] = 1;
  nforce_term = 4;
  underdamped_iteration(nullptr);
  std::printf("pos1 %.17g %.17g %.17g\n", pos[1].x, pos[1].y, pos[1].z);
  std::printf("uncN %.17g %.17g %.17g\n", unc_pos[nbead].x, unc_pos[nbead].y, unc_pos[nbead].z);
  std::printf("vel2 %.17g %.17g %.17g\n", vel[2].x, vel[2].y, vel[2].z);
  overdamped_iteration(nullptr);
  gpu_begin(1000);
  gpu_steps(50);
  gpu_output();
  std::printf("output %g %g %g %g %g %d %g %g\n", e_bnd, e_ang_ss, e_vdw_rr, rna_etot, Q, contct_nat,
              rgsq, kinT);
  gpu_read_state();
  gpu_detach();
  std::printf("done\n");
  return 0;
}
