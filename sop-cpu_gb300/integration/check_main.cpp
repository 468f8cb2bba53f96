// Link check of gpu_backend.cpp: takes the address of every function the shim
// defines, so the link must resolve each one's uses of the reference's
// globals and of libsopgpu.so.  Built by `make check`; never run.
#include <cstdio>

void gpu_attach();
void update_neighbor_list();
void update_cell_list();
void update_pair_list();
void force_eval();
void energy_eval();
void gpu_begin(long long);
void gpu_steps(long long);
void gpu_output();
void gpu_read_state();

int main() {
  void (*fs[])() = {gpu_attach, update_neighbor_list, update_cell_list, update_pair_list,
                    force_eval, energy_eval, gpu_output, gpu_read_state};
  void (*gs[])(long long) = {gpu_begin, gpu_steps};
  std::printf("%zu entry points\n", sizeof fs / sizeof fs[0] + sizeof gs / sizeof gs[0]);
  return 0;
}
