// Link check of gpu_backend.cpp against libsopgpu.so: takes the address of
// every function the backend defines, so the link must resolve each one's
// uses of the reference's globals and of the engine library.  Built by
// `make check`; prints the count (the CPU test of what the functions do is
// shim_main.cpp with the recording stub).
#include <cstdio>

#include "global.h"

void gpu_attach();
void gpu_detach();
void update_neighbor_list();
void update_cell_list();
void update_pair_list();
void force_eval();
void energy_eval();
void underdamped_iteration(coord*);
void overdamped_iteration(coord*);
void gpu_begin(long long);
void gpu_steps(long long);
void gpu_output();
void gpu_read_state();
int gpu_force_terms();

int main() {
  void (*fs[])() = {gpu_attach, gpu_detach, update_neighbor_list, update_cell_list,
                    update_pair_list, force_eval, energy_eval, gpu_output, gpu_read_state};
  void (*gs[])(long long) = {gpu_begin, gpu_steps};
  void (*its[])(coord*) = {underdamped_iteration, overdamped_iteration};
  int (*ts[])() = {gpu_force_terms};
  std::printf("%zu entry points\n", sizeof fs / sizeof fs[0] + sizeof gs / sizeof gs[0] +
                                        sizeof its / sizeof its[0] + sizeof ts / sizeof ts[0]);
  return 0;
}
