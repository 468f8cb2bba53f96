// stub_abi.cpp -- a recording stand-in for libsopgpu.so, for the CPU test of
// gpu_backend.cpp.  It implements the C-ABI calls the backend makes, runs no
// GPU code, and writes one text line per call (and the whole system
// description of sop_replica_add) to the file named by SOP_STUB_LOG.  The call
// named by SOP_STUB_FAIL returns SOP_ERR_CUDA instead, so the test can check
// that the backend stops on a failed status.  Results it hands back are
// recognisable functions of the bead index (force = bead + 0.25 component,
// positions = 10 bead + component, ...) so the test can check the 0-based to
// 1-based copies.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "sop_gpu.h"

namespace {

FILE* logf() {
  static FILE* f = nullptr;
  if (!f) {
    const char* path = std::getenv("SOP_STUB_LOG");
    f = path ? std::fopen(path, "w") : stderr;
    if (!f) f = stderr;
  }
  return f;
}

int call(const char* name) {
  std::fprintf(logf(), "call %s\n", name);
  std::fflush(logf());
  const char* failing = std::getenv("SOP_STUB_FAIL");
  return (failing && !std::strcmp(failing, name)) ? SOP_ERR_CUDA : SOP_OK;
}

void log_params(const char* tag, const sop_params& p) {
  std::fprintf(logf(),
               "%s T %.17g zeta %.17g h %.17g a1 %.17g a2 %.17g a3 %.17g a4 %.17g a5 %.17g "
               "boxl %.17g lcell %.17g ncell %.17g k_bnd %.17g R0 %.17g sigma_ss %.17g "
               "epsilon_ss %.17g nnlup %d nup %d list_mode %d dynamics %d force_terms %d seed %lld\n",
               tag, p.T, p.zeta, p.h, p.a1, p.a2, p.a3, p.a4, p.a5, p.boxl, p.lcell, p.ncell,
               p.k_bnd, p.R0, p.sigma_ss, p.epsilon_ss, p.nnlup, p.nup, p.list_mode, p.dynamics,
               p.force_terms, (long long)p.seed);
}

int g_nbead = 0;
sop_engine* const kEngine = reinterpret_cast<sop_engine*>(0x1000);

}  // namespace

extern "C" {

const char* sop_status_string(int status) { return status == SOP_OK ? "ok" : "stub failure"; }

void sop_params_default(sop_params* p) {
  std::memset(p, 0, sizeof *p);
  p->pull_j = -1;
}

void sop_engine_config_default(sop_engine_config* c) { std::memset(c, 0, sizeof *c); }

int sop_engine_create(const sop_engine_config* cfg, sop_engine** out) {
  int rc = call("sop_engine_create");
  std::fprintf(logf(), "config max_beads %d max_replicas %d max_list_entries %lld\n", cfg->max_beads,
               cfg->max_replicas, (long long)cfg->max_list_entries);
  if (rc == SOP_OK) *out = kEngine;
  return rc;
}

int sop_engine_destroy(sop_engine*) { return call("sop_engine_destroy"); }

int sop_replica_add(sop_engine* e, const sop_system_desc* d, int* replica) {
  int rc = call("sop_replica_add");
  if (rc != SOP_OK) return rc;
  if (e != kEngine) return SOP_ERR_ARG;
  FILE* f = logf();
  g_nbead = d->nbead;
  std::fprintf(f, "nbead %d\n", d->nbead);
  std::fprintf(f, "xyz");
  for (int k = 0; k < 3 * d->nbead; k++) std::fprintf(f, " %.17g", d->xyz[k]);
  std::fprintf(f, "\ntype");
  for (int k = 0; k < d->nbead; k++) std::fprintf(f, " %d", d->bead_type ? d->bead_type[k] : 1);
  std::fprintf(f, "\nbonds %d", d->nbnd);
  for (int k = 0; k < d->nbnd; k++) std::fprintf(f, " %d %d %.17g", d->ib[k], d->jb[k], d->r0[k]);
  std::fprintf(f, "\nangles %d", d->nang);
  for (int k = 0; k < d->nang; k++) std::fprintf(f, " %d %d", d->ia[k], d->ka[k]);
  std::fprintf(f, "\nnatives %d", d->nnat);
  for (int k = 0; k < d->nnat; k++) std::fprintf(f, " %d %d %.17g", d->in_[k], d->jn[k], d->rn[k]);
  std::fprintf(f, "\nexclusions %d", d->nexcl);
  for (int k = 0; k < d->nexcl; k++) std::fprintf(f, " %d %d", d->ie[k], d->je[k]);
  std::fprintf(f, "\n");
  log_params("params", d->params);
  std::fflush(f);
  *replica = 0;
  return SOP_OK;
}

int sop_replica_set_params(sop_engine*, int, const sop_params* p) {
  int rc = call("sop_replica_set_params");
  log_params("set_params", *p);
  return rc;
}

int sop_update_neighbor_list(sop_engine*, int) { return call("sop_update_neighbor_list"); }
int sop_update_cell_list(sop_engine*, int) { return call("sop_update_cell_list"); }
int sop_update_pair_list(sop_engine*, int) { return call("sop_update_pair_list"); }

int sop_force_eval(sop_engine*, int, double* f) {
  int rc = call("sop_force_eval");
  for (int i = 0; i < g_nbead; i++)
    for (int c = 0; c < 3; c++) f[3 * i + c] = i + 0.25 * c;
  return rc;
}

int sop_energy_eval(sop_engine*, int, double* out) {
  int rc = call("sop_energy_eval");
  for (int k = 0; k < 6; k++) out[k] = k + 1.5;
  return rc;
}

int sop_underdamped_iteration(sop_engine*, int) { return call("sop_underdamped_iteration"); }
int sop_replica_start(sop_engine*, int, int64_t nsteps) {
  int rc = call("sop_replica_start");
  std::fprintf(logf(), "nsteps %lld\n", (long long)nsteps);
  return rc;
}
int sop_run_chunk(sop_engine*, int64_t, int*, int, int* nfinished) {
  *nfinished = 0;
  return call("sop_run_chunk");
}

int sop_replica_outputs(sop_engine*, int, double* energy6, double* obs5) {
  int rc = call("sop_replica_outputs");
  if (energy6)
    for (int k = 0; k < 6; k++) energy6[k] = 100 + k;
  if (obs5)
    for (int k = 0; k < 5; k++) obs5[k] = 200 + k;
  return rc;
}

int sop_observables(sop_engine*, int, double* out) {
  int rc = call("sop_observables");
  for (int k = 0; k < 5; k++) out[k] = 300 + k;
  return rc;
}

int sop_replica_get_state(sop_engine*, int, double* pos, double* unc, double* vel) {
  int rc = call("sop_replica_get_state");
  for (int i = 0; i < g_nbead; i++)
    for (int c = 0; c < 3; c++) {
      pos[3 * i + c] = 10.0 * i + c;
      unc[3 * i + c] = 10.0 * i + c + 0.5;
      vel[3 * i + c] = -(10.0 * i + c);
    }
  return rc;
}

}  // extern "C"
