// gpu_backend.cpp -- the file a SOP-CPU maintainer adds to the reference's
// tree to run its entry points on the GB300 engine.  Compiled with the
// reference's own sources (whose CPU definitions of the forwarded functions
// are then left out, e.g. behind -DSOP_GPU) and linked with -lsopgpu.  The
// reference's globals stay the source of truth for the inputs; the state
// moves back to them after a forwarded iteration and when gpu_read_state()
// is called (the run-window path: every nup steps).
//
// Every library call is checked: a failure ends the program with the
// library's message and exit(-1), the reference's own way out of a fatal
// input error (e.g. sop.cpp:88).
//
// make -C sop-cpu_gb300/integration check   compiles it against the reference's
//   headers and links it with the reference's globals and libsopgpu.so;
// make -C sop-cpu_gb300/integration shim-test   links it with the reference's
//   loaders (params.cpp, io.cpp) and a recording stub of the C ABI, so a CPU
//   test can check what it hands to the engine.
#include <algorithm>
#include <cstddef>  // size_t: global.h uses it without including it
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <unordered_set>
#include <vector>

#include "global.h"
#include "sop_gpu.h"

static sop_engine* g_eng;
static int g_rep = -1;

static void check(int rc, const char* what) {
  if (rc != SOP_OK) {
    std::fprintf(stderr, "GPU backend: %s failed: %s (%d)\n", what, sop_status_string(rc), rc);
    std::exit(-1);
  }
}

static void fail(const char* why) {
  std::fprintf(stderr, "GPU backend: %s\n", why);
  std::exit(-1);
}

// force_term_on[] / nforce_term (global.cpp:200-203) as the engine's term
// mask: set_forces (energy.cpp:78-113) installs the switched-on terms of slots
// 1 (random), 2 (FENE), 3 (angles) and 6 (vdw) in slot order, other slots
// install nothing, and force_eval (energy.cpp:21-45) calls the first
// nforce_term installed terms.
int gpu_force_terms() {
  static const int slot_bit[7] = {0, SOP_TERM_RANDOM, SOP_TERM_FENE, SOP_TERM_ANGLE, 0, 0,
                                  SOP_TERM_VDW};
  int mask = 0, used = 0;
  for (int i = 1; i <= 6 && used < nforce_term; i++) {
    if (!slot_bit[i] || !force_term_on[i]) continue;
    mask |= slot_bit[i];
    used++;
  }
  return mask;
}

// The run and force-field parameters the reference's globals hold now
// (set_params, params.cpp:12-101; defaults params.cpp:262-400).
static sop_params current_params() {
  sop_params p;
  sop_params_default(&p);
  p.T = T; p.zeta = zeta; p.h = h;
  p.a1 = a1; p.a2 = a2; p.a3 = a3; p.a4 = a4; p.a5 = a5;
  p.boxl = boxl; p.lcell = lcell; p.ncell = ncell;
  p.k_bnd = k_bnd; p.R0 = R0; p.sigma_ss = sigma_ss; p.epsilon_ss = epsilon_ss;
  p.nnlup = nnlup; p.nup = nup;
  p.list_mode = neighborlist ? SOP_LIST_NEIGHBOR : celllist ? SOP_LIST_CELL : SOP_LIST_NONE;
  p.dynamics = sim_type == 2 ? SOP_DYN_OVERDAMPED : SOP_DYN_UNDERDAMPED;
  p.force_terms = gpu_force_terms();
  p.seed = (uint64_t)(int64_t)(-100 - run);
  return p;
}

// Bead types from the vdw candidates' type columns (params.cpp:186-197): the
// engine keeps one type per bead, so a bead listed with two types is refused.
static void bead_types(std::vector<int>& type) {
  type.assign(nbead, 0);
  auto put = [&](int bead, int t) {
    if (bead < 1 || bead > nbead || t < 1 || t > 2) fail("vdw candidate with a bead or type out of range");
    int& slot = type[bead - 1];
    if (slot && slot != t) fail("a bead carries two different types in the vdw file");
    slot = t;
  };
  for (int k = 1; k <= ncon_att; k++) {
    put(ibead_lj_nat[k], itype_lj_nat[k]);
    put(jbead_lj_nat[k], jtype_lj_nat[k]);
  }
  for (int k = 1; k <= ncon_rep; k++) {
    put(ibead_lj_non_nat[k], itype_lj_non_nat[k]);
    put(jbead_lj_non_nat[k], jtype_lj_non_nat[k]);
  }
  for (int& t : type)
    if (!t) t = 1;  // a bead in no candidate pair: its type is never read
}

// The engine's candidate set is implicit (every pair with |i-j| > 2 that is
// not native); pairs of it the vdw file does not list never interact in the
// reference, so they go to the engine as exclusions.  A listed non-native
// with |i-j| <= 2 has no place in that set and is refused.
static void exclusions(std::vector<int>& ie, std::vector<int>& je) {
  const long long n = nbead;
  std::unordered_set<long long> listed;
  listed.reserve(2 * (size_t)(ncon_att + ncon_rep) + 1);
  auto key = [n](int a, int b) { return (long long)std::min(a, b) * n + std::max(a, b); };
  for (int k = 1; k <= ncon_att; k++) listed.insert(key(ibead_lj_nat[k] - 1, jbead_lj_nat[k] - 1));
  for (int k = 1; k <= ncon_rep; k++) {
    const int i = ibead_lj_non_nat[k] - 1, j = jbead_lj_non_nat[k] - 1;
    if (std::abs(i - j) <= 2) fail("a non-native vdw candidate with |i-j| <= 2 is not supported");
    listed.insert(key(i, j));
  }
  for (int i = 0; i < nbead; i++)
    for (int j = i + 3; j < nbead; j++)
      if (!listed.count(key(i, j))) {
        ie.push_back(i);
        je.push_back(j);
      }
}

// After load bonds/angles/vdw/init and the set commands (params.cpp:12-260):
// create the engine and upload the system; builds its lists at X0
// (sop.cpp:117-125).
void gpu_attach() {
  std::vector<double> xyz(3 * (size_t)nbead);
  for (int i = 1; i <= nbead; i++) {
    xyz[3 * i - 3] = unc_pos[i].x; xyz[3 * i - 2] = unc_pos[i].y; xyz[3 * i - 1] = unc_pos[i].z;
  }
  std::vector<int> type, in(ncon_att), jn(ncon_att), ib(nbnd), jb(nbnd), ia(nang), ka(nang), ie, je;
  std::vector<double> rn(ncon_att), r0(nbnd);
  bead_types(type);
  for (int k = 1; k <= ncon_att; k++) {
    in[k - 1] = ibead_lj_nat[k] - 1; jn[k - 1] = jbead_lj_nat[k] - 1; rn[k - 1] = lj_nat_pdb_dist[k];
  }
  for (int k = 1; k <= nbnd; k++) { ib[k - 1] = ibead_bnd[k] - 1; jb[k - 1] = jbead_bnd[k] - 1; r0[k - 1] = pdb_dist[k]; }
  for (int k = 1; k <= nang; k++) { ia[k - 1] = ibead_ang[k] - 1; ka[k - 1] = kbead_ang[k] - 1; }
  exclusions(ie, je);

  sop_system_desc d = {};
  d.nbead = nbead; d.xyz = xyz.data(); d.bead_type = type.data();
  d.nbnd = nbnd; d.ib = ib.data(); d.jb = jb.data(); d.r0 = r0.data();
  d.nang = nang; d.ia = ia.data(); d.ka = ka.data();
  d.nnat = ncon_att; d.in_ = in.data(); d.jn = jn.data(); d.rn = rn.data();
  d.nexcl = (int)ie.size(); d.ie = ie.data(); d.je = je.data();
  d.params = current_params();

  sop_engine_config cfg;
  sop_engine_config_default(&cfg);
  // the per-bead arenas also hold the exclusions (24 entries per bead slot)
  cfg.max_beads = std::max({2 * nbead, 4096, (int)std::min<long long>(2LL * ie.size() / 24 + 1, 1 << 30)});
  cfg.max_replicas = 4;
  cfg.max_list_entries = (int64_t)nbead * 512 + 65536;
  check(sop_engine_create(&cfg, &g_eng), "sop_engine_create");
  check(sop_replica_add(g_eng, &d, &g_rep), "sop_replica_add");
}

// the reference's globals may have changed since the last call (set
// commands, force_term_on edits): the engine takes them before each call
static void sync_params() {
  const sop_params p = current_params();
  check(sop_replica_set_params(g_eng, g_rep, &p), "sop_replica_set_params");
}

void gpu_read_state();

// ---- the reference's entry points, forwarded (neighbor_list.h, cell_list.h,
// ---- sop.h, energy.h) ---------------------------------------------------------
void update_neighbor_list() { check(sop_update_neighbor_list(g_eng, g_rep), "sop_update_neighbor_list"); }
void update_cell_list() { check(sop_update_cell_list(g_eng, g_rep), "sop_update_cell_list"); }
void update_pair_list() { check(sop_update_pair_list(g_eng, g_rep), "sop_update_pair_list"); }

void force_eval() {
  sync_params();
  std::vector<double> f(3 * (size_t)nbead);
  check(sop_force_eval(g_eng, g_rep, f.data()), "sop_force_eval");
  for (int i = 1; i <= nbead; i++) { force[i].x = f[3 * i - 3]; force[i].y = f[3 * i - 2]; force[i].z = f[3 * i - 1]; }
}

void energy_eval() {
  double e[6];
  check(sop_energy_eval(g_eng, g_rep, e), "sop_energy_eval");
  e_bnd = e[0]; e_ang_ss = e[1]; e_vdw_rr = e[2]; e_vdw_rr_att = e[3]; e_vdw_rr_rep = e[4]; rna_etot = e[5];
}

// underdamped_iteration (sop.cpp:282-329) / overdamped_iteration
// (sop.cpp:331-363): one step of the replica's integrator on the device, then
// pos, unc_pos and vel back into the globals.  The position increment stays
// on the device (the reference's callers read it only in
// calculate_observables, which gpu_output covers).
static void iteration() {
  sync_params();
  check(sop_underdamped_iteration(g_eng, g_rep), "sop_underdamped_iteration");
  gpu_read_state();
}
void underdamped_iteration(coord*) { iteration(); }
void overdamped_iteration(coord*) { iteration(); }

// underdamped_ctrl's loop (sop.cpp:153-189) on the device: one run window of
// nstep steps, advanced in chunks that end right after each nup step
void gpu_begin(long long nstep) {
  sync_params();
  check(sop_replica_start(g_eng, g_rep, nstep), "sop_replica_start");
}
void gpu_steps(long long launches) {
  int fin[1], nfin = 0;
  check(sop_run_chunk(g_eng, launches, fin, 1, &nfin), "sop_run_chunk");
}

// at an nup step: the energies the step itself computed (with the pair list
// its force used), the observables and the state
void gpu_output() {
  double e[6], o[5];
  check(sop_replica_outputs(g_eng, g_rep, e, nullptr), "sop_replica_outputs");
  check(sop_observables(g_eng, g_rep, o), "sop_observables");
  e_bnd = e[0]; e_ang_ss = e[1]; e_vdw_rr = e[2]; e_vdw_rr_att = e[3]; e_vdw_rr_rep = e[4]; rna_etot = e[5];
  Q = o[0]; contct_nat = (int)o[1]; rgsq = o[2]; kinT = o[3];
}

void gpu_read_state() {
  std::vector<double> p(3 * (size_t)nbead), u(3 * (size_t)nbead), v(3 * (size_t)nbead);
  check(sop_replica_get_state(g_eng, g_rep, p.data(), u.data(), v.data()), "sop_replica_get_state");
  for (int i = 1; i <= nbead; i++) {  // coord has a constructor: set the fields
    pos[i].x = p[3 * i - 3]; pos[i].y = p[3 * i - 2]; pos[i].z = p[3 * i - 1];
    unc_pos[i].x = u[3 * i - 3]; unc_pos[i].y = u[3 * i - 2]; unc_pos[i].z = u[3 * i - 1];
    vel[i].x = v[3 * i - 3]; vel[i].y = v[3 * i - 2]; vel[i].z = v[3 * i - 1];
  }
}

// end of run: the engine and its device memory
void gpu_detach() {
  if (g_eng) check(sop_engine_destroy(g_eng), "sop_engine_destroy");
  g_eng = nullptr;
  g_rep = -1;
}
