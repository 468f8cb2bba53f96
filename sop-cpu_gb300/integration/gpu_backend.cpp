// gpu_backend.cpp -- the file a SOP-CPU maintainer adds to the reference's
// tree to run its entry points on the GB300 engine.  Compiled with the
// reference's own sources (whose CPU definitions of the forwarded functions
// are then left out, e.g. behind -DSOP_GPU) and linked with -lsopgpu.  The
// reference's globals stay the source of truth between calls; state moves
// only when the reference's code reads it (every nup steps).
//
// make -C sop-cpu_gb300/integration check compiles it against the reference's
// headers and links it with the reference's globals and libsopgpu.so.
#include <cstddef>  // size_t: global.h uses it without including it
#include <cstdint>
#include <vector>

#include "global.h"
#include "sop_gpu.h"

static sop_engine* g_eng;
static int g_rep = -1;

// after load bonds/angles/vdw/init and the set commands (params.cpp:12-260)
void gpu_attach() {
  sop_engine_create(nullptr, &g_eng);
  std::vector<double> xyz(3 * nbead);
  for (int i = 1; i <= nbead; i++) { xyz[3*i-3] = unc_pos[i].x; xyz[3*i-2] = unc_pos[i].y; xyz[3*i-1] = unc_pos[i].z; }
  // natives from the vdw candidates (r < rcut_nat, params.cpp:197), 0-based
  std::vector<int> in(ncon_att), jn(ncon_att), ib(nbnd), jb(nbnd), ia(nang), ka(nang);
  std::vector<double> rn(ncon_att), r0(nbnd);
  for (int k = 1; k <= ncon_att; k++) { in[k-1] = ibead_lj_nat[k]-1; jn[k-1] = jbead_lj_nat[k]-1; rn[k-1] = lj_nat_pdb_dist[k]; }
  for (int k = 1; k <= nbnd; k++) { ib[k-1] = ibead_bnd[k]-1; jb[k-1] = jbead_bnd[k]-1; r0[k-1] = pdb_dist[k]; }
  for (int k = 1; k <= nang; k++) { ia[k-1] = ibead_ang[k]-1; ka[k-1] = kbead_ang[k]-1; }
  sop_system_desc d = {};
  d.nbead = nbead; d.xyz = xyz.data();
  d.nbnd = nbnd; d.ib = ib.data(); d.jb = jb.data(); d.r0 = r0.data();
  d.nang = nang; d.ia = ia.data(); d.ka = ka.data();
  d.nnat = ncon_att; d.in_ = in.data(); d.jn = jn.data(); d.rn = rn.data();
  sop_params_default(&d.params);
  d.params.T = T; d.params.zeta = zeta; d.params.h = h;
  d.params.a1 = a1; d.params.a2 = a2; d.params.a3 = a3; d.params.a4 = a4;
  d.params.boxl = boxl; d.params.lcell = lcell; d.params.ncell = ncell;
  d.params.nnlup = nnlup; d.params.nup = nup;
  d.params.list_mode = neighborlist ? SOP_LIST_NEIGHBOR : celllist ? SOP_LIST_CELL : SOP_LIST_NONE;
  d.params.seed = (uint64_t)(int64_t)(-100 - run);
  sop_replica_add(g_eng, &d, &g_rep);          // builds the lists at X0 (sop.cpp:119-125)
}

// the reference's entry points, forwarded (energy.h, neighbor_list.h, cell_list.h, sop.h)
void update_neighbor_list() { sop_update_neighbor_list(g_eng, g_rep); }
void update_cell_list()     { sop_update_cell_list(g_eng, g_rep); }
void update_pair_list()     { sop_update_pair_list(g_eng, g_rep); }
void force_eval() {
  std::vector<double> f(3 * nbead);
  sop_force_eval(g_eng, g_rep, f.data());
  for (int i = 1; i <= nbead; i++) { force[i].x = f[3*i-3]; force[i].y = f[3*i-2]; force[i].z = f[3*i-1]; }
}
void energy_eval() {
  double e[6]; sop_energy_eval(g_eng, g_rep, e);
  e_bnd = e[0]; e_ang_ss = e[1]; e_vdw_rr = e[2]; e_vdw_rr_att = e[3]; e_vdw_rr_rep = e[4]; rna_etot = e[5];
}
// underdamped_ctrl's loop (sop.cpp:153-189) on the device: one run window of
// nstep steps, advanced in chunks that end right after each nup step
void gpu_begin(long long nstep) { sop_replica_start(g_eng, g_rep, nstep); }
void gpu_steps(long long launches) { int fin[1], nfin; sop_run_chunk(g_eng, launches, fin, 1, &nfin); }
// at an nup step: the energies the step itself computed (with the pair list
// its force used), the observables and the state
void gpu_output() {
  double e[6], o[5];
  sop_replica_outputs(g_eng, g_rep, e, nullptr);
  sop_observables(g_eng, g_rep, o);
  e_bnd = e[0]; e_ang_ss = e[1]; e_vdw_rr = e[2]; rna_etot = e[5];
  Q = o[0]; contct_nat = (int)o[1]; rgsq = o[2]; kinT = o[3];
}
void gpu_read_state() {
  std::vector<double> p(3*nbead), u(3*nbead), v(3*nbead);
  sop_replica_get_state(g_eng, g_rep, p.data(), u.data(), v.data());
  for (int i = 1; i <= nbead; i++) {  // coord has a constructor: set the fields
    pos[i].x = p[3*i-3]; pos[i].y = p[3*i-2]; pos[i].z = p[3*i-1];
    unc_pos[i].x = u[3*i-3]; unc_pos[i].y = u[3*i-2]; unc_pos[i].z = u[3*i-1];
    vel[i].x = v[3*i-3]; vel[i].y = v[3*i-2]; vel[i].z = v[3*i-1];
  }
}
