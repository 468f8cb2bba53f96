/* Test infrastructure only: CPU oracle for the SOP hot path (see sop_oracle.h).
 * Each function cites the SOP-CPU file:line whose algorithm it restates; the
 * FP64 expressions keep the reference's operation order so that, compiled
 * with -ffp-contract=off, the results equal the reference's bit for bit.
 */
#include "sop_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* Pair-type tables (global.cpp:60-92), index 0 unused. */
static const double k_coeff_att[3][3] = {{0, 0, 0}, {0, 0.7, 0.8}, {0, 0.8, 1.0}};
static const double k_coeff_rep[3][3] = {{0, 0, 0}, {0, 1.0, 1.0}, {0, 1.0, 1.0}};
static const double k_force_coeff_att[3][3] = {
    {0, 0, 0}, {0, -12.0 * 1.0, -12.0 * 0.8}, {0, -12.0 * 0.8, -12.0 * 0.7}};
static const double k_force_coeff_rep[3][3] = {
    {0, 0, 0}, {0, -6.0 * 1.0, -6.0 * 1.0}, {0, -6.0 * 1.0, -6.0 * 1.0}};
static const double k_sigma_rep[3][3] = {{0, 0, 0}, {0, 3.8, 5.4}, {0, 5.4, 7.0}};
static const double k_rcut_nat[3][3] = {{0, 0, 0}, {0, 8.0, 11.0}, {0, 11.0, 14.0}};

struct sopo_sys {
  int nbead;
  double *pos, *unc_pos, *vel, *force, *incr;
  /* bonds / angles */
  int nbnd, *ib, *jb;
  double* r0b;
  int nang, *ia, *ja, *ka;
  /* candidates: natives (c) and non-natives (r) */
  int nnat, *ci, *cj, *cti, *ctj;
  double *cr, *cr2, *cr6, *cr12;
  int nrep, *ri, *rj, *rti, *rtj;
  /* lists hold candidate indices */
  int nnl_att, nnl_rep, nil_att, nil_rep;
  int *nl_att, *nl_rep, *pl_att, *pl_rep;
  /* parameters (params.cpp:262-400 defaults) */
  double k_bnd, R0, R0sq, e_bnd_coeff;
  double sigma_ss, sigma_ss6, epsilon_ss, e_ang_ss_coeff, f_ang_ss_coeff;
  double sigma_rep2[3][3], sigma_rep6[3][3], sigma_rep12[3][3];
  double T, boxl, ncell, lcell, zeta, nstep, h, halfh, a1, a2, a3, a4, a5;
  int nup, nnlup, run, sim_type, neighborlist, celllist;
  uint64_t seed;
  uint64_t force_evals; /* noise counter: one per force_eval */
  int force_on[4];      /* random, fene, angle, vdw */
  /* constant pulling force on two beads (no reference term) */
  double pull_f;        /* kcal/mol/A; 0 = off */
  int pull_i, pull_j;   /* pulled beads; pull_j < 0 = the last bead */
  int inlup;
  /* energies / observables */
  double e_bnd, e_ang_ss, e_vdw_att, e_vdw_rep, e_vdw, etot;
  double Q, rgsq, kinT;
  int contct_nat;
};

static double rnd(double x) { return (x > 0) ? floor(x + 0.5) : ceil(x - 0.5); } /* global.cpp:223-227 */

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  if (!p) { fprintf(stderr, "sop_oracle: out of memory\n"); abort(); }
  return p;
}

static void set_integrator_defaults(sopo_sys* s) {
  s->h = 2.5e-3;
  s->halfh = s->h / 2.0;
  s->a1 = s->h * (1.0 - s->zeta * s->halfh);
  s->a2 = s->h * s->halfh;
  s->a3 = (1.0 - s->h * s->zeta / 2.0 + (s->h * s->zeta) * (s->h * s->zeta) / 4.0) / s->h;
  s->a4 = s->halfh * (1.0 - s->h * s->zeta / 2.0);
  s->a5 = s->h / s->zeta;
}

sopo_sys* sopo_create(void) {
  sopo_sys* s = (sopo_sys*)xcalloc(1, sizeof(sopo_sys));
  /* params.cpp:268-293 */
  s->k_bnd = 20.0;
  s->R0 = 2.0;
  s->R0sq = s->R0 * s->R0;
  s->e_bnd_coeff = s->k_bnd * s->R0sq / 2.0;
  s->sigma_ss = 3.5;
  s->sigma_ss6 = pow(s->sigma_ss, 6.0);
  s->epsilon_ss = 1.0;
  s->e_ang_ss_coeff = s->epsilon_ss * s->sigma_ss6;
  s->f_ang_ss_coeff = 6.0 * s->e_ang_ss_coeff;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      s->sigma_rep2[i][j] = k_sigma_rep[i][j] * k_sigma_rep[i][j];
      s->sigma_rep6[i][j] = s->sigma_rep2[i][j] * s->sigma_rep2[i][j] * s->sigma_rep2[i][j];
      s->sigma_rep12[i][j] = s->sigma_rep6[i][j] * s->sigma_rep6[i][j];
    }
  /* params.cpp:367-392 */
  s->run = 1;
  s->seed = (uint64_t)(int64_t)(-100 - s->run);
  s->T = 0.6;
  s->boxl = 500.0;
  s->ncell = 55.0;
  s->lcell = s->boxl / s->ncell;
  s->zeta = 5.0e-2;
  s->nstep = 5e7;
  s->nup = 1000;
  s->nnlup = 50;
  s->sim_type = 1;
  set_integrator_defaults(s);
  /* global.cpp:200-202: random, bonds, angles, vdw on */
  s->force_on[0] = s->force_on[1] = s->force_on[2] = s->force_on[3] = 1;
  s->inlup = 1;
  s->pull_f = 0.0;
  s->pull_i = 0;
  s->pull_j = -1;
  return s;
}

static void free_topology(sopo_sys* s) {
  free(s->pos); free(s->unc_pos); free(s->vel); free(s->force); free(s->incr);
  free(s->ib); free(s->jb); free(s->r0b);
  free(s->ia); free(s->ja); free(s->ka);
  free(s->ci); free(s->cj); free(s->cti); free(s->ctj);
  free(s->cr); free(s->cr2); free(s->cr6); free(s->cr12);
  free(s->ri); free(s->rj); free(s->rti); free(s->rtj);
  free(s->nl_att); free(s->nl_rep); free(s->pl_att); free(s->pl_rep);
  s->pos = s->unc_pos = s->vel = s->force = s->incr = NULL;
  s->ib = s->jb = s->ia = s->ja = s->ka = NULL;
  s->r0b = NULL;
  s->ci = s->cj = s->cti = s->ctj = s->ri = s->rj = s->rti = s->rtj = NULL;
  s->cr = s->cr2 = s->cr6 = s->cr12 = NULL;
  s->nl_att = s->nl_rep = s->pl_att = s->pl_rep = NULL;
}

void sopo_destroy(sopo_sys* s) {
  if (!s) return;
  free_topology(s);
  free(s);
}

static void alloc_beads(sopo_sys* s, int nbead) {
  free(s->pos); free(s->unc_pos); free(s->vel); free(s->force); free(s->incr);
  s->nbead = nbead;
  s->pos = (double*)xcalloc(3 * (size_t)nbead, sizeof(double));
  s->unc_pos = (double*)xcalloc(3 * (size_t)nbead, sizeof(double));
  s->vel = (double*)xcalloc(3 * (size_t)nbead, sizeof(double));
  s->force = (double*)xcalloc(3 * (size_t)nbead, sizeof(double));
  s->incr = (double*)xcalloc(3 * (size_t)nbead, sizeof(double));
}

static void set_bonds(sopo_sys* s, int nbnd, const int* ib, const int* jb, const double* r0) {
  free(s->ib); free(s->jb); free(s->r0b);
  s->nbnd = nbnd;
  s->ib = (int*)xcalloc(nbnd, sizeof(int));
  s->jb = (int*)xcalloc(nbnd, sizeof(int));
  s->r0b = (double*)xcalloc(nbnd, sizeof(double));
  if (nbnd) {
    memcpy(s->ib, ib, nbnd * sizeof(int));
    memcpy(s->jb, jb, nbnd * sizeof(int));
    memcpy(s->r0b, r0, nbnd * sizeof(double));
  }
}

static void set_angles(sopo_sys* s, int nang, const int* ia, const int* ja, const int* ka) {
  free(s->ia); free(s->ja); free(s->ka);
  s->nang = nang;
  s->ia = (int*)xcalloc(nang, sizeof(int));
  s->ja = (int*)xcalloc(nang, sizeof(int));
  s->ka = (int*)xcalloc(nang, sizeof(int));
  if (nang) {
    memcpy(s->ia, ia, nang * sizeof(int));
    if (ja) memcpy(s->ja, ja, nang * sizeof(int));
    memcpy(s->ka, ka, nang * sizeof(int));
  }
}

static void alloc_candidates(sopo_sys* s, int nnat, int nrep) {
  free(s->ci); free(s->cj); free(s->cti); free(s->ctj);
  free(s->cr); free(s->cr2); free(s->cr6); free(s->cr12);
  free(s->ri); free(s->rj); free(s->rti); free(s->rtj);
  free(s->nl_att); free(s->nl_rep); free(s->pl_att); free(s->pl_rep);
  s->nnat = nnat;
  s->nrep = nrep;
  s->ci = (int*)xcalloc(nnat, sizeof(int));
  s->cj = (int*)xcalloc(nnat, sizeof(int));
  s->cti = (int*)xcalloc(nnat, sizeof(int));
  s->ctj = (int*)xcalloc(nnat, sizeof(int));
  s->cr = (double*)xcalloc(nnat, sizeof(double));
  s->cr2 = (double*)xcalloc(nnat, sizeof(double));
  s->cr6 = (double*)xcalloc(nnat, sizeof(double));
  s->cr12 = (double*)xcalloc(nnat, sizeof(double));
  s->ri = (int*)xcalloc(nrep, sizeof(int));
  s->rj = (int*)xcalloc(nrep, sizeof(int));
  s->rti = (int*)xcalloc(nrep, sizeof(int));
  s->rtj = (int*)xcalloc(nrep, sizeof(int));
  s->nl_att = (int*)xcalloc(nnat, sizeof(int));
  s->pl_att = (int*)xcalloc(nnat, sizeof(int));
  s->nl_rep = (int*)xcalloc(nrep, sizeof(int));
  s->pl_rep = (int*)xcalloc(nrep, sizeof(int));
}

/* One native candidate, with the powers computed as params.cpp:201-205. */
static void put_native(sopo_sys* s, int k, int i, int j, double r, int ti, int tj) {
  s->ci[k] = i; s->cj[k] = j; s->cti[k] = ti; s->ctj[k] = tj;
  s->cr[k] = r;
  s->cr2[k] = r * r;
  s->cr6[k] = s->cr2[k] * s->cr2[k] * s->cr2[k];
  s->cr12[k] = s->cr6[k] * s->cr6[k];
}

/* load vdw seeds both pair lists with every candidate (params.cpp:210-230). */
static void seed_pair_lists(sopo_sys* s) {
  s->nil_att = s->nnat;
  for (int k = 0; k < s->nnat; k++) s->pl_att[k] = k;
  s->nil_rep = s->nrep;
  for (int k = 0; k < s->nrep; k++) s->pl_rep[k] = k;
  s->nnl_att = s->nnl_rep = 0;
}

/* Split candidates into natives and non-natives by r < rcut_nat
 * (params.cpp:197), in candidate order, and seed the pair lists. */
static void set_candidates(sopo_sys* s, int ncand, const int* ic, const int* jc, const double* rc,
                           const int* ti, const int* tj) {
  int nn = 0, nr = 0;
  for (int k = 0; k < ncand; k++) {
    if (rc[k] < k_rcut_nat[ti[k]][tj[k]]) nn++;
    else nr++;
  }
  alloc_candidates(s, nn, nr);
  nn = nr = 0;
  for (int k = 0; k < ncand; k++) {
    if (rc[k] < k_rcut_nat[ti[k]][tj[k]]) {
      put_native(s, nn++, ic[k], jc[k], rc[k], ti[k], tj[k]);
    } else {
      s->ri[nr] = ic[k]; s->rj[nr] = jc[k]; s->rti[nr] = ti[k]; s->rtj[nr] = tj[k];
      nr++;
    }
  }
  seed_pair_lists(s);
}

int sopo_set_topology(sopo_sys* s, int nbead, int nbnd, const int* ib, const int* jb,
                      const double* r0, int nang, const int* ia, const int* ja, const int* ka,
                      int ncand, const int* ic, const int* jc, const double* rc, const int* ti,
                      const int* tj) {
  alloc_beads(s, nbead);
  set_bonds(s, nbnd, ib, jb, r0);
  set_angles(s, nang, ia, ja, ka);
  set_candidates(s, ncand, ic, jc, rc, ti, tj);
  return 0;
}

static int cmp_pair(const void* a, const void* b) {
  const int* x = (const int*)a;
  const int* y = (const int*)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
  return 0;
}

int sopo_set_topology_implicit(sopo_sys* s, int nbead, const int* type, const int* chain,
                               int nbnd, const int* ib, const int* jb, const double* r0,
                               int nang, const int* ia, const int* ja, const int* ka,
                               int nnat, const int* in_, const int* jn, const double* rn) {
  alloc_beads(s, nbead);
  set_bonds(s, nbnd, ib, jb, r0);
  set_angles(s, nang, ia, ja, ka);
  /* natives sorted (i,j) with their distances, so that membership is a merge */
  int* nat = (int*)xcalloc(3 * (size_t)nnat, sizeof(int));
  for (int k = 0; k < nnat; k++) { nat[3 * k] = in_[k]; nat[3 * k + 1] = jn[k]; nat[3 * k + 2] = k; }
  qsort(nat, nnat, 3 * sizeof(int), cmp_pair);
  long long ncand = 0;
  for (int i = 0; i < nbead; i++)
    for (int j = i + 1; j < nbead; j++)
      if ((chain && chain[i] != chain[j]) || j - i > 2) ncand++;
  int nnative = 0;
  for (int k = 0; k < nnat; k++) {
    int t_i = type ? type[in_[k]] : 1, t_j = type ? type[jn[k]] : 1;
    if (rn[k] < k_rcut_nat[t_i][t_j]) nnative++;
  }
  if (ncand - nnative > 0x7fffffffLL) { free(nat); return -1; }
  alloc_candidates(s, nnative, (int)(ncand - nnative));
  int nn = 0, nr = 0, p = 0;
  for (int i = 0; i < nbead; i++) {
    for (int j = i + 1; j < nbead; j++) {
      if (!((chain && chain[i] != chain[j]) || j - i > 2)) continue;
      int ti = type ? type[i] : 1, tj = type ? type[j] : 1;
      while (p < nnat && (nat[3 * p] < i || (nat[3 * p] == i && nat[3 * p + 1] < j))) p++;
      if (p < nnat && nat[3 * p] == i && nat[3 * p + 1] == j &&
          rn[nat[3 * p + 2]] < k_rcut_nat[ti][tj]) {
        put_native(s, nn++, i, j, rn[nat[3 * p + 2]], ti, tj);
      } else {
        s->ri[nr] = i; s->rj[nr] = j; s->rti[nr] = ti; s->rtj[nr] = tj;
        nr++;
      }
    }
  }
  free(nat);
  s->nnat = nn;
  s->nrep = nr;
  seed_pair_lists(s);
  return 0;
}

static int cmp_ll(const void* a, const void* b) {
  const long long x = *(const long long*)a, y = *(const long long*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

int sopo_set_topology_pruned(sopo_sys* s, int nbead, const int* type, const int* chain,
                             int nbnd, const int* ib, const int* jb, const double* r0,
                             int nang, const int* ia, const int* ja, const int* ka,
                             int nnat, const int* in_, const int* jn, const double* rn,
                             const double* xyz, double cutoff) {
  if (nbead <= 0 || !(cutoff > 0)) return -1;
  /* close pairs (i<j) through a uniform grid of edge `cutoff` */
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < nbead; i++)
    for (int c = 0; c < 3; c++) {
      if (xyz[3 * i + c] < lo[c]) lo[c] = xyz[3 * i + c];
      if (xyz[3 * i + c] > hi[c]) hi[c] = xyz[3 * i + c];
    }
  long long dim[3];
  double edge = cutoff;
  for (;;) {
    for (int c = 0; c < 3; c++) dim[c] = (long long)((hi[c] - lo[c]) / edge) + 1;
    if (dim[0] * dim[1] * dim[2] <= 4LL * nbead + 4096) break;
    edge *= 1.25;
  }
  const long long ncell = dim[0] * dim[1] * dim[2];
  long long* cid = (long long*)xcalloc((size_t)nbead, sizeof(long long));
  long long* start = (long long*)xcalloc((size_t)ncell + 1, sizeof(long long));
  int* sorted = (int*)xcalloc((size_t)nbead, sizeof(int));
  for (int i = 0; i < nbead; i++) {
    long long q[3];
    for (int c = 0; c < 3; c++) {
      q[c] = (long long)((xyz[3 * i + c] - lo[c]) / edge);
      if (q[c] >= dim[c]) q[c] = dim[c] - 1;
    }
    cid[i] = q[0] + dim[0] * (q[1] + dim[1] * q[2]);
    start[cid[i] + 1]++;
  }
  for (long long c = 0; c < ncell; c++) start[c + 1] += start[c];
  {
    long long* fill = (long long*)xcalloc((size_t)ncell, sizeof(long long));
    for (int i = 0; i < nbead; i++) sorted[start[cid[i]] + fill[cid[i]]++] = i;
    free(fill);
  }
  size_t cap = 1024, np = 0;
  long long* pairs = (long long*)xcalloc(cap, sizeof(long long));
  const double c2 = cutoff * cutoff;
  for (int i = 0; i < nbead; i++) {
    const long long qx = cid[i] % dim[0], qy = (cid[i] / dim[0]) % dim[1], qz = cid[i] / (dim[0] * dim[1]);
    for (long long z = qz - 1; z <= qz + 1; z++)
      for (long long y = qy - 1; y <= qy + 1; y++)
        for (long long x = qx - 1; x <= qx + 1; x++) {
          if (x < 0 || y < 0 || z < 0 || x >= dim[0] || y >= dim[1] || z >= dim[2]) continue;
          const long long cc = x + dim[0] * (y + dim[1] * z);
          for (long long k = start[cc]; k < start[cc + 1]; k++) {
            const int j = sorted[k];
            if (j <= i) continue;
            if (!((chain && chain[i] != chain[j]) || j - i > 2)) continue;
            const double dx = xyz[3 * j] - xyz[3 * i], dy = xyz[3 * j + 1] - xyz[3 * i + 1],
                         dz = xyz[3 * j + 2] - xyz[3 * i + 2];
            if (dx * dx + dy * dy + dz * dz >= c2) continue;
            if (np == cap) {
              cap *= 2;
              pairs = (long long*)realloc(pairs, cap * sizeof(long long));
              if (!pairs) { fprintf(stderr, "oracle: out of memory\n"); exit(1); }
            }
            pairs[np++] = (long long)i * nbead + j;
          }
        }
  }
  free(cid);
  free(start);
  free(sorted);
  /* every native pair (i<j) is a candidate whatever its distance */
  for (int k = 0; k < nnat; k++) {
    if (np == cap) {
      cap *= 2;
      pairs = (long long*)realloc(pairs, cap * sizeof(long long));
      if (!pairs) { fprintf(stderr, "oracle: out of memory\n"); exit(1); }
    }
    pairs[np++] = (long long)in_[k] * nbead + jn[k];
  }
  qsort(pairs, np, sizeof(long long), cmp_ll);
  size_t u = 0;
  for (size_t k = 0; k < np; k++)
    if (u == 0 || pairs[k] != pairs[u - 1]) pairs[u++] = pairs[k];
  np = u;

  alloc_beads(s, nbead);
  set_bonds(s, nbnd, ib, jb, r0);
  set_angles(s, nang, ia, ja, ka);
  int* nat = (int*)xcalloc(3 * (size_t)(nnat > 0 ? nnat : 1), sizeof(int));
  for (int k = 0; k < nnat; k++) { nat[3 * k] = in_[k]; nat[3 * k + 1] = jn[k]; nat[3 * k + 2] = k; }
  qsort(nat, nnat, 3 * sizeof(int), cmp_pair);
  int nnative = 0;
  for (int k = 0; k < nnat; k++) {
    int t_i = type ? type[in_[k]] : 1, t_j = type ? type[jn[k]] : 1;
    if (rn[k] < k_rcut_nat[t_i][t_j]) nnative++;
  }
  alloc_candidates(s, nnative, (int)(np - (size_t)nnative));
  int nn = 0, nr = 0, p = 0;
  for (size_t k = 0; k < np; k++) {
    const int i = (int)(pairs[k] / nbead), j = (int)(pairs[k] % nbead);
    if (!((chain && chain[i] != chain[j]) || j - i > 2)) continue;  /* not a candidate */
    int ti = type ? type[i] : 1, tj = type ? type[j] : 1;
    while (p < nnat && (nat[3 * p] < i || (nat[3 * p] == i && nat[3 * p + 1] < j))) p++;
    if (p < nnat && nat[3 * p] == i && nat[3 * p + 1] == j &&
        rn[nat[3 * p + 2]] < k_rcut_nat[ti][tj]) {
      put_native(s, nn++, i, j, rn[nat[3 * p + 2]], ti, tj);
    } else {
      s->ri[nr] = i; s->rj[nr] = j; s->rti[nr] = ti; s->rtj[nr] = tj;
      nr++;
    }
  }
  free(nat);
  free(pairs);
  s->nnat = nn;
  s->nrep = nr;
  seed_pair_lists(s);
  return 0;
}

static double* coord_ptr(const sopo_sys* s, int which) {
  switch (which) {
    case 0: return s->pos;
    case 1: return s->unc_pos;
    case 2: return s->vel;
    case 3: return s->force;
    case 4: return s->incr;
    default: return NULL;
  }
}

int sopo_set_coords(sopo_sys* s, int which, const double* xyz) {
  double* p = coord_ptr(s, which);
  if (!p) return -1;
  memcpy(p, xyz, 3 * (size_t)s->nbead * sizeof(double));
  return 0;
}

int sopo_get_coords(const sopo_sys* s, int which, double* xyz) {
  const double* p = coord_ptr(s, which);
  if (!p) return -1;
  memcpy(xyz, p, 3 * (size_t)s->nbead * sizeof(double));
  return 0;
}

int sopo_set_param(sopo_sys* s, const char* name, double v) {
  if (!strcmp(name, "T")) s->T = v;
  else if (!strcmp(name, "zeta")) s->zeta = v;
  else if (!strcmp(name, "h")) s->h = v;
  else if (!strcmp(name, "halfh")) s->halfh = v;
  else if (!strcmp(name, "a1")) s->a1 = v;
  else if (!strcmp(name, "a2")) s->a2 = v;
  else if (!strcmp(name, "a3")) s->a3 = v;
  else if (!strcmp(name, "a4")) s->a4 = v;
  else if (!strcmp(name, "a5")) s->a5 = v;
  else if (!strcmp(name, "boxl")) s->boxl = v;
  else if (!strcmp(name, "ncell")) s->ncell = v;
  else if (!strcmp(name, "lcell")) s->lcell = v;
  else if (!strcmp(name, "nstep")) s->nstep = v;
  else if (!strcmp(name, "nup")) s->nup = (int)v;
  else if (!strcmp(name, "nnlup")) s->nnlup = (int)v;
  else if (!strcmp(name, "seed")) s->seed = (uint64_t)(int64_t)v;
  else if (!strcmp(name, "neighborlist")) s->neighborlist = (int)v;
  else if (!strcmp(name, "celllist")) s->celllist = (int)v;
  else if (!strcmp(name, "force_evals")) s->force_evals = (uint64_t)v;
  else if (!strcmp(name, "pull_force")) s->pull_f = v;
  else if (!strcmp(name, "pull_i")) s->pull_i = (int)v;
  else if (!strcmp(name, "pull_j")) s->pull_j = (int)v;
  else return -1;
  return 0;
}

double sopo_get_param(const sopo_sys* s, const char* name) {
  if (!strcmp(name, "T")) return s->T;
  if (!strcmp(name, "zeta")) return s->zeta;
  if (!strcmp(name, "h")) return s->h;
  if (!strcmp(name, "halfh")) return s->halfh;
  if (!strcmp(name, "a1")) return s->a1;
  if (!strcmp(name, "a2")) return s->a2;
  if (!strcmp(name, "a3")) return s->a3;
  if (!strcmp(name, "a4")) return s->a4;
  if (!strcmp(name, "a5")) return s->a5;
  if (!strcmp(name, "boxl")) return s->boxl;
  if (!strcmp(name, "ncell")) return s->ncell;
  if (!strcmp(name, "lcell")) return s->lcell;
  if (!strcmp(name, "nstep")) return s->nstep;
  if (!strcmp(name, "nup")) return s->nup;
  if (!strcmp(name, "nnlup")) return s->nnlup;
  if (!strcmp(name, "run")) return s->run;
  if (!strcmp(name, "seed")) return (double)(int64_t)s->seed;
  if (!strcmp(name, "neighborlist")) return s->neighborlist;
  if (!strcmp(name, "celllist")) return s->celllist;
  if (!strcmp(name, "sim_type")) return s->sim_type;
  if (!strcmp(name, "k_bnd")) return s->k_bnd;
  if (!strcmp(name, "R0")) return s->R0;
  if (!strcmp(name, "force_evals")) return (double)s->force_evals;
  if (!strcmp(name, "pull_force")) return s->pull_f;
  if (!strcmp(name, "pull_i")) return s->pull_i;
  if (!strcmp(name, "pull_j")) return s->pull_j;
  return NAN;
}

/* set_params (params.cpp:12-101), keyword by keyword, same side effects. */
int sopo_set_command(sopo_sys* s, const char* key, const char* value) {
  if (!strcmp(key, "dynamics")) {
    if (value && !strcmp(value, "underdamped")) {
      s->sim_type = 1;
      s->h = 2.5e-3;
      s->halfh = s->h / 2.0;
      s->a1 = s->h * (1.0 - s->zeta * s->halfh);
      s->a2 = s->h * s->halfh;
      s->a3 = (1.0 - s->h * s->zeta / 2.0 + (s->h * s->zeta) * (s->h * s->zeta) / 4.0) / s->h;
      s->a4 = s->halfh * (1.0 - s->h * s->zeta / 2.0);
    } else if (value && !strcmp(value, "overdamped")) {
      s->sim_type = 2;
      s->h = 0.02;
      s->a5 = s->h / s->zeta;
    }
  } else if (!strcmp(key, "temp")) {
    s->T = atof(value);
  } else if (!strcmp(key, "nstep")) {
    s->nstep = atof(value);
  } else if (!strcmp(key, "nup")) {
    s->nup = atoi(value);
  } else if (!strcmp(key, "run")) {
    s->run = atoi(value);
    s->seed = (uint64_t)(int64_t)(-100 - s->run);
  } else if (!strcmp(key, "cutofftype")) {
    if (!strcmp(value, "neighborlist")) s->neighborlist = 1;
    else if (!strcmp(value, "celllist")) s->celllist = 1;
  } else if (!strcmp(key, "nnlup")) {
    s->nnlup = atoi(value);
  } else if (!strcmp(key, "boxl")) {
    s->boxl = atof(value);
  } else if (!strcmp(key, "ncell")) {
    s->ncell = atof(value);
    s->lcell = s->boxl / s->ncell;
  } else if (!strcmp(key, "t_step")) {
    s->h = atof(value);
    s->halfh = s->h / 2.0;
    s->a1 = s->h * (1.0 - s->zeta * s->halfh);
    s->a2 = s->h * s->halfh;
    s->a3 = (1.0 - s->h * s->zeta / 2.0 + (s->h * s->zeta) * (s->h * s->zeta) / 4.0) / s->h;
    s->a4 = s->halfh * (1.0 - s->h * s->zeta / 2.0);
    s->a5 = s->h / s->zeta;
  } else if (!strcmp(key, "zeta")) {
    /* resets h but not halfh or a2 (params.cpp:91-98) */
    if (s->sim_type == 1) s->h = 2.5e-3;
    else if (s->sim_type == 2) s->h = 0.02;
    s->zeta = atof(value);
    s->a1 = s->h * (1.0 - s->zeta * s->halfh);
    s->a3 = (1.0 - s->h * s->zeta / 2.0 + (s->h * s->zeta) * (s->h * s->zeta) / 4.0) / s->h;
    s->a4 = s->halfh * (1.0 - s->h * s->zeta / 2.0);
    s->a5 = s->h / s->zeta;
  } else {
    /* file names, restart switches, istep_restart: no effect on the path */
    return 1;
  }
  return 0;
}

/* ---- input files (params.cpp:110-260) ---------------------------------- */

static char* slurp(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  char* buf = (char*)xcalloc((size_t)n + 1, 1);
  if (fread(buf, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(buf); return NULL; }
  buf[n] = 0;
  fclose(f);
  return buf;
}

/* Next line of a buffer (newline replaced by NUL); NULL at the end. */
static char* next_line(char** cur) {
  char* p = *cur;
  if (!p || !*p) return NULL;
  char* e = strchr(p, '\n');
  if (e) { *e = 0; *cur = e + 1; }
  else *cur = p + strlen(p);
  return p;
}

static int nth_token_int(char* line, int n) {
  char* save = NULL;
  char* t = strtok_r(line, " \t\r", &save);
  for (int k = 1; k < n && t; k++) t = strtok_r(NULL, " \t\r", &save);
  return t ? atoi(t) : -1;
}

static int load_file(sopo_sys* s, const char* what, const char* path) {
  char* buf = slurp(path);
  if (!buf) { fprintf(stderr, "sop_oracle: cannot open %s\n", path); return -1; }
  char* cur = buf;
  char* line = next_line(&cur);
  int rc = 0;
  if (!line) { free(buf); return -1; }
  if (!strcmp(what, "bonds")) {
    int n = nth_token_int(line, 2);
    int* ib = (int*)xcalloc(n, sizeof(int));
    int* jb = (int*)xcalloc(n, sizeof(int));
    double* r0 = (double*)xcalloc(n, sizeof(double));
    for (int k = 0; k < n; k++) {
      line = next_line(&cur);
      if (!line || sscanf(line, "%d %d %lf", &ib[k], &jb[k], &r0[k]) != 3) { rc = -1; break; }
      ib[k]--; jb[k]--;
    }
    if (!rc) set_bonds(s, n, ib, jb, r0);
    free(ib); free(jb); free(r0);
  } else if (!strcmp(what, "angles")) {
    int n = nth_token_int(line, 2);
    int* ia = (int*)xcalloc(n, sizeof(int));
    int* ja = (int*)xcalloc(n, sizeof(int));
    int* ka = (int*)xcalloc(n, sizeof(int));
    for (int k = 0; k < n; k++) {
      double a0;
      line = next_line(&cur);
      if (!line || sscanf(line, "%d %d %d %lf", &ia[k], &ja[k], &ka[k], &a0) != 4) { rc = -1; break; }
      ia[k]--; ja[k]--; ka[k]--;
    }
    if (!rc) set_angles(s, n, ia, ja, ka);
    free(ia); free(ja); free(ka);
  } else if (!strcmp(what, "vdw")) {
    char hdr[4096];
    strncpy(hdr, line, sizeof(hdr) - 1);
    hdr[sizeof(hdr) - 1] = 0;
    int natt = nth_token_int(line, 2);
    int nrep = nth_token_int(hdr, 4);
    int ntot = natt + nrep;
    int* ic = (int*)xcalloc(ntot, sizeof(int));
    int* jc = (int*)xcalloc(ntot, sizeof(int));
    int* ti = (int*)xcalloc(ntot, sizeof(int));
    int* tj = (int*)xcalloc(ntot, sizeof(int));
    double* rc_ = (double*)xcalloc(ntot, sizeof(double));
    for (int k = 0; k < ntot; k++) {
      line = next_line(&cur);
      if (!line || sscanf(line, "%d %d %lf %d %d", &ic[k], &jc[k], &rc_[k], &ti[k], &tj[k]) != 5) {
        rc = -1;
        break;
      }
      ic[k]--; jc[k]--;
    }
    if (!rc) {
      set_candidates(s, ntot, ic, jc, rc_, ti, tj);
      if (s->nnat != natt || s->nrep != nrep) rc = -2; /* header disagrees with the rcut split */
    }
    free(ic); free(jc); free(ti); free(tj); free(rc_);
  } else if (!strcmp(what, "init")) {
    int n = nth_token_int(line, 2);
    alloc_beads(s, n);
    for (int k = 0; k < n; k++) {
      int idx;
      double x, y, z;
      line = next_line(&cur);
      if (!line || sscanf(line, "%d %lf %lf %lf", &idx, &x, &y, &z) != 4) { rc = -1; break; }
      s->pos[3 * k] = s->unc_pos[3 * k] = x;
      s->pos[3 * k + 1] = s->unc_pos[3 * k + 1] = y;
      s->pos[3 * k + 2] = s->unc_pos[3 * k + 2] = z;
    }
  } else {
    rc = 1;
  }
  free(buf);
  return rc;
}

/* Command script: whitespace tokens; a token containing ';' ends a command,
 * and ';' characters are dropped (io.cpp:9-89). */
int sopo_load_script(sopo_sys* s, const char* path) {
  char* buf = slurp(path);
  if (!buf) return -1;
  char* toks[64];
  int nt = 0, rc = 0;
  char* save = NULL;
  for (char* t = strtok_r(buf, " \t\r\n", &save); t; t = strtok_r(NULL, " \t\r\n", &save)) {
    int ends = strchr(t, ';') != NULL;
    char* w = t;
    for (char* r = t; *r; r++)
      if (*r != ';') *w++ = *r;
    *w = 0;
    if (nt < 64) toks[nt++] = t;
    if (ends) {
      if (nt >= 1 && !strcmp(toks[0], "load") && nt >= 3) {
        int r = load_file(s, toks[1], toks[2]);
        if (r < 0) rc = r;
      } else if (nt >= 1 && !strcmp(toks[0], "set") && nt >= 2) {
        sopo_set_command(s, toks[1], nt >= 3 ? toks[2] : NULL);
      }
      nt = 0;
    }
  }
  free(buf);
  return rc;
}

void sopo_set_force_terms(sopo_sys* s, int random_on, int fene_on, int ang_on, int vdw_on) {
  s->force_on[0] = random_on;
  s->force_on[1] = fene_on;
  s->force_on[2] = ang_on;
  s->force_on[3] = vdw_on;
}

/* ---- pair search ------------------------------------------------------- */

static inline double pair_d2(const sopo_sys* s, int i, int j) {
  const double* u = s->unc_pos;
  double dx = u[3 * j] - u[3 * i];
  double dy = u[3 * j + 1] - u[3 * i + 1];
  double dz = u[3 * j + 2] - u[3 * i + 2];
  dx -= s->boxl * rnd(dx / s->boxl);
  dy -= s->boxl * rnd(dy / s->boxl);
  dz -= s->boxl * rnd(dz / s->boxl);
  return dx * dx + dy * dy + dz * dz;
}

/* neighbor_list.cpp:17-116 */
void sopo_neighbor_list(sopo_sys* s) {
  s->nnl_att = 0;
  for (int c = 0; c < s->nnat; c++) {
    double d2 = pair_d2(s, s->ci[c], s->cj[c]);
    double rcut = 3.2 * s->cr[c];
    double rcut2 = rcut * rcut;
    if (d2 < rcut2) s->nl_att[s->nnl_att++] = c;
  }
  s->nnl_rep = 0;
  for (int c = 0; c < s->nrep; c++) {
    double d2 = pair_d2(s, s->ri[c], s->rj[c]);
    double rcut = 3.2 * k_sigma_rep[s->rti[c]][s->rtj[c]];
    double rcut2 = rcut * rcut;
    if (d2 < rcut2) s->nl_rep[s->nnl_rep++] = c;
  }
}

static inline int cell_adjacent(const sopo_sys* s, int i, int j) {
  const double* u = s->unc_pos;
  double imx = floor(u[3 * i] / s->lcell), imy = floor(u[3 * i + 1] / s->lcell),
         imz = floor(u[3 * i + 2] / s->lcell);
  double jmx = floor(u[3 * j] / s->lcell), jmy = floor(u[3 * j + 1] / s->lcell),
         jmz = floor(u[3 * j + 2] / s->lcell);
  double cx = imx - jmx, cy = imy - jmy, cz = imz - jmz;
  cx -= s->ncell * rnd(cx / s->ncell);
  cy -= s->ncell * rnd(cy / s->ncell);
  cz -= s->ncell * rnd(cz / s->ncell);
  return cx >= -1.0 && cx <= 1.0 && cy >= -1.0 && cy <= 1.0 && cz >= -1.0 && cz <= 1.0;
}

/* cell_list.cpp:15-97 */
void sopo_cell_list(sopo_sys* s) {
  s->nnl_att = 0;
  for (int c = 0; c < s->nnat; c++)
    if (cell_adjacent(s, s->ci[c], s->cj[c])) s->nl_att[s->nnl_att++] = c;
  s->nnl_rep = 0;
  for (int c = 0; c < s->nrep; c++)
    if (cell_adjacent(s, s->ri[c], s->rj[c])) s->nl_rep[s->nnl_rep++] = c;
}

/* sop.cpp:486-552 */
void sopo_pair_list(sopo_sys* s) {
  s->nil_att = 0;
  for (int k = 0; k < s->nnl_att; k++) {
    int c = s->nl_att[k];
    double d2 = pair_d2(s, s->ci[c], s->cj[c]);
    double rcut = 2.5 * s->cr[c];
    double rcut2 = rcut * rcut;
    if (d2 < rcut2) s->pl_att[s->nil_att++] = c;
  }
  s->nil_rep = 0;
  for (int k = 0; k < s->nnl_rep; k++) {
    int c = s->nl_rep[k];
    double d2 = pair_d2(s, s->ri[c], s->rj[c]);
    double rcut = 2.5 * k_sigma_rep[s->rti[c]][s->rtj[c]];
    double rcut2 = rcut * rcut;
    if (d2 < rcut2) s->pl_rep[s->nil_rep++] = c;
  }
}

/* ---- noise: Philox-4x32-10 + Box-Muller --------------------------------- */

void sopo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Three standard normals for (bead, force evaluation) from one Philox block. */
static void bead_normals(uint64_t seed, uint64_t step, int bead, double g[3]) {
  uint32_t ctr[4] = {(uint32_t)bead, (uint32_t)step, (uint32_t)(step >> 32), 0u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  sopo_philox4x32_10(ctr, key, o);
  const double two_m32 = 2.3283064365386963e-10; /* 2^-32 */
  double u0 = ((double)o[0] + 0.5) * two_m32, u1 = ((double)o[1] + 0.5) * two_m32;
  double u2 = ((double)o[2] + 0.5) * two_m32, u3 = ((double)o[3] + 0.5) * two_m32;
  double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
  const double twopi = 6.283185307179586;
  g[0] = r0 * cos(twopi * u1);
  g[1] = r0 * sin(twopi * u1);
  g[2] = r1 * cos(twopi * u3);
}

/* ---- force terms (energy.cpp:259-465) ----------------------------------- */

static void clear_forces(sopo_sys* s) { memset(s->force, 0, 3 * (size_t)s->nbead * sizeof(double)); }

static void random_force(sopo_sys* s) {
  double var = sqrt(2.0 * s->T * s->zeta / s->h);
  for (int i = 0; i < s->nbead; i++) {
    double g[3];
    bead_normals(s->seed, s->force_evals, i, g);
    s->force[3 * i] += var * g[0];
    s->force[3 * i + 1] += var * g[1];
    s->force[3 * i + 2] += var * g[2];
  }
}

static void fene_forces(sopo_sys* s) {
  const double* u = s->unc_pos;
  double* f = s->force;
  for (int b = 0; b < s->nbnd; b++) {
    int i = s->ib[b], j = s->jb[b];
    double dx = u[3 * j] - u[3 * i];
    double dy = u[3 * j + 1] - u[3 * i + 1];
    double dz = u[3 * j + 2] - u[3 * i + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    double dev = d - s->r0b[b];
    double dev2 = dev * dev;
    double temp = -s->k_bnd * dev / d / (1.0 - dev2 / s->R0sq);
    double fx = temp * dx, fy = temp * dy, fz = temp * dz;
    f[3 * i] -= fx; f[3 * i + 1] -= fy; f[3 * i + 2] -= fz;
    f[3 * j] += fx; f[3 * j + 1] += fy; f[3 * j + 2] += fz;
  }
}

static void soft_sphere_angular_forces(sopo_sys* s) {
  const double* u = s->unc_pos;
  double* f = s->force;
  for (int a = 0; a < s->nang; a++) {
    int i = s->ia[a], k = s->ka[a];
    double dx = u[3 * k] - u[3 * i];
    double dy = u[3 * k + 1] - u[3 * i + 1];
    double dz = u[3 * k + 2] - u[3 * i + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    double d8 = pow(d, 8.0);
    double co1 = s->f_ang_ss_coeff / d8;
    double fx = co1 * dx, fy = co1 * dy, fz = co1 * dz;
    f[3 * i] -= fx; f[3 * i + 1] -= fy; f[3 * i + 2] -= fz;
    f[3 * k] += fx; f[3 * k + 1] += fy; f[3 * k + 2] += fz;
  }
}

static void vdw_forces(sopo_sys* s) {
  const double* u = s->unc_pos;
  double* f = s->force;
  const double tol = 1.0e-7;
  double rep_tol = 0.0; /* the reference leaves it unset when nil_att == 0 */
  for (int k = 0; k < s->nil_att; k++) {
    int c = s->pl_att[k];
    int i = s->ci[c], j = s->cj[c], ti = s->cti[c], tj = s->ctj[c];
    double dx = u[3 * j] - u[3 * i];
    double dy = u[3 * j + 1] - u[3 * i + 1];
    double dz = u[3 * j + 2] - u[3 * i + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d2 = dx * dx + dy * dy + dz * dz;
    rep_tol = s->sigma_rep2[ti][tj] * tol;
    /* energy.cpp:293 tests against the UNFILTERED native array at the pair-list
     * position (lj_nat_pdb_dist2[i] with i the pair-list index) */
    if (d2 < tol * s->cr2[k]) continue;
    double d6 = d2 * d2 * d2;
    double d12 = d6 * d6;
    double co1 = k_force_coeff_att[ti][tj] / d2 * ((s->cr12[c] / d12) - (s->cr6[c] / d6));
    double fx = co1 * dx, fy = co1 * dy, fz = co1 * dz;
    f[3 * i] += fx; f[3 * i + 1] += fy; f[3 * i + 2] += fz;
    f[3 * j] -= fx; f[3 * j + 1] -= fy; f[3 * j + 2] -= fz;
  }
  for (int k = 0; k < s->nil_rep; k++) {
    int c = s->pl_rep[k];
    int i = s->ri[c], j = s->rj[c], ti = s->rti[c], tj = s->rtj[c];
    double dx = u[3 * j] - u[3 * i];
    double dy = u[3 * j + 1] - u[3 * i + 1];
    double dz = u[3 * j + 2] - u[3 * i + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < rep_tol) continue;
    double d6 = d2 * d2 * d2;
    double d12 = d6 * d6;
    double co1 = k_force_coeff_rep[ti][tj] / d2 *
                 (2.0 * s->sigma_rep12[ti][tj] / d12 + s->sigma_rep6[ti][tj] / d6);
    double fx = co1 * dx, fy = co1 * dy, fz = co1 * dz;
    f[3 * i] += fx; f[3 * i + 1] += fy; f[3 * i + 2] += fz;
    f[3 * j] -= fx; f[3 * j + 1] -= fy; f[3 * j + 2] -= fz;
  }
}

/* Constant-force pulling of two beads apart along their separation, the
 * served workload's optional term.  The reference has no such term (its
 * tension switch is off by default, global.cpp:200, and has no force
 * routine), so this restates the engine's definition: with u = x_j - x_i
 * (unwrapped positions, no minimum image), bead i gets -f u/|u| and bead j
 * +f u/|u|, f in kcal/mol/A (1 pN = 1/69.48 kcal/mol/A).  Independent of the
 * force-term switches; applied after them. */
static void pull_force(sopo_sys* s) {
  const int i = s->pull_i, j = s->pull_j < 0 ? s->nbead - 1 : s->pull_j;
  if (i < 0 || i >= s->nbead || j < 0 || j >= s->nbead || i == j) return;
  const double* u = s->unc_pos;
  double ux = u[3 * j] - u[3 * i], uy = u[3 * j + 1] - u[3 * i + 1], uz = u[3 * j + 2] - u[3 * i + 2];
  double d = sqrt(ux * ux + uy * uy + uz * uz);
  double fx = s->pull_f * ux / d, fy = s->pull_f * uy / d, fz = s->pull_f * uz / d;
  s->force[3 * i] -= fx; s->force[3 * i + 1] -= fy; s->force[3 * i + 2] -= fz;
  s->force[3 * j] += fx; s->force[3 * j + 1] += fy; s->force[3 * j + 2] += fz;
}

/* energy.cpp:21-45 with the term order of set_forces (energy.cpp:78-113),
 * then the pulling term when one is set. */
void sopo_force_eval(sopo_sys* s) {
  clear_forces(s);
  if (s->force_on[0]) random_force(s);
  if (s->force_on[1]) fene_forces(s);
  if (s->force_on[2]) soft_sphere_angular_forces(s);
  if (s->force_on[3]) vdw_forces(s);
  if (s->pull_f != 0.0) pull_force(s);
  s->force_evals++;
}

/* ---- energy terms (energy.cpp:115-257) ---------------------------------- */

void sopo_energy_eval(sopo_sys* s) {
  const double* u = s->unc_pos;
  double e = 0.0;
  for (int b = 0; b < s->nbnd; b++) {
    int i = s->ib[b], j = s->jb[b];
    double dx = u[3 * j] - u[3 * i];
    double dy = u[3 * j + 1] - u[3 * i + 1];
    double dz = u[3 * j + 2] - u[3 * i + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    double dev = d - s->r0b[b];
    e += log1p(-dev * dev / s->R0sq);
  }
  e *= -s->e_bnd_coeff;
  s->e_bnd = e;

  e = 0.0;
  for (int a = 0; a < s->nang; a++) {
    int i = s->ia[a], k = s->ka[a];
    double rx = u[3 * k] - u[3 * i];
    double ry = u[3 * k + 1] - u[3 * i + 1];
    double rz = u[3 * k + 2] - u[3 * i + 2];
    rx -= s->boxl * rnd(rx / s->boxl);
    ry -= s->boxl * rnd(ry / s->boxl);
    rz -= s->boxl * rnd(rz / s->boxl);
    double d = sqrt(rx * rx + ry * ry + rz * rz);
    double d6 = pow(d, 6.0);
    e += s->e_ang_ss_coeff / d6;
  }
  s->e_ang_ss = e;

  double ea = 0.0, er = 0.0;
  for (int k = 0; k < s->nil_att; k++) {
    int c = s->pl_att[k];
    int ti = s->cti[c], tj = s->ctj[c];
    double d2 = pair_d2(s, s->ci[c], s->cj[c]);
    double d6 = d2 * d2 * d2;
    double d12 = d6 * d6;
    /* energy.cpp:224: the coefficient multiplies only the r^-12 term */
    ea += k_coeff_att[ti][tj] * (s->cr12[c] / d12) - 2.0 * (s->cr6[c] / d6);
  }
  for (int k = 0; k < s->nil_rep; k++) {
    int c = s->pl_rep[k];
    int ti = s->rti[c], tj = s->rtj[c];
    double d2 = pair_d2(s, s->ri[c], s->rj[c]);
    double d6 = d2 * d2 * d2;
    double d12 = d6 * d6;
    er += k_coeff_rep[ti][tj] * (s->sigma_rep12[ti][tj] / d12 + s->sigma_rep6[ti][tj] / d6);
  }
  s->e_vdw_att = ea;
  s->e_vdw_rep = er;
  s->e_vdw = ea + er;
  s->etot = s->e_bnd + s->e_ang_ss + s->e_vdw;
}

/* ---- observables (sop.cpp:200-279) -------------------------------------- */

void sopo_observables(sopo_sys* s) {
  const double* u = s->unc_pos;
  int cnt = 0;
  for (int c = 0; c < s->nnat; c++) {
    int i = s->ci[c], j = s->cj[c];
    float r_ij = (float)s->cr[c];
    double dx = u[3 * i] - u[3 * j];
    double dy = u[3 * i + 1] - u[3 * j + 1];
    double dz = u[3 * i + 2] - u[3 * j + 2];
    dx -= s->boxl * rnd(dx / s->boxl);
    dy -= s->boxl * rnd(dy / s->boxl);
    dz -= s->boxl * rnd(dz / s->boxl);
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d / r_ij < 1.25) cnt++;
  }
  s->contct_nat = cnt;
  s->Q = (double)cnt / s->nnat;
  double rg = 0.0;
  for (int i = 0; i < s->nbead - 1; i++) {
    for (int j = i + 1; j < s->nbead; j++) {
      double dx = u[3 * i] - u[3 * j];
      double dy = u[3 * i + 1] - u[3 * j + 1];
      double dz = u[3 * i + 2] - u[3 * j + 2];
      dx -= s->boxl * rnd(dx / s->boxl);
      dy -= s->boxl * rnd(dy / s->boxl);
      dz -= s->boxl * rnd(dz / s->boxl);
      rg += (dx * dx + dy * dy + dz * dz);
    }
  }
  rg /= (double)(s->nbead * s->nbead);
  s->rgsq = rg;
  double sv = 0.0;
  if (s->sim_type == 2) {  /* overdamped: from the last increments (sop.cpp:270-278) */
    for (int i = 0; i < s->nbead; i++) {
      const double* v = s->incr + 3 * i;
      sv += v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
    sv *= s->zeta / (2.0 * s->h);
  } else {
    for (int i = 0; i < s->nbead; i++) {
      const double* v = s->vel + 3 * i;
      sv += v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
  }
  s->kinT = sv / (3.0 * (double)s->nbead);
}

/* ---- integrator and step loop ------------------------------------------- */

/* sop.cpp:282-329 */
void sopo_iteration(sopo_sys* s) {
  const double eps = 1.0e-5;
  double *pos = s->pos, *unc = s->unc_pos, *vel = s->vel, *f = s->force, *inc = s->incr;
  if (s->sim_type == 2) {  /* overdamped_iteration (sop.cpp:331-363) */
    for (int q = 0; q < 3 * s->nbead; q++) {
      inc[q] = s->a5 * f[q];
      unc[q] += inc[q];
      pos[q] += inc[q];
      pos[q] -= s->boxl * rnd(pos[q] / s->boxl);
    }
    sopo_force_eval(s);
    return;
  }
  for (int q = 0; q < 3 * s->nbead; q++) {
    inc[q] = s->a1 * vel[q] + s->a2 * f[q];
    pos[q] += inc[q];
    pos[q] -= s->boxl * rnd(pos[q] / s->boxl);
    unc[q] += inc[q];
  }
  sopo_force_eval(s);
  if (s->T < eps) return;
  for (int q = 0; q < 3 * s->nbead; q++) vel[q] = s->a3 * inc[q] + s->a4 * f[q];
}

/* underdamped_ctrl set-up (sop.cpp:106-147). */
void sopo_setup(sopo_sys* s, int do_initial_eval) {
  memset(s->vel, 0, 3 * (size_t)s->nbead * sizeof(double));
  memset(s->force, 0, 3 * (size_t)s->nbead * sizeof(double));
  if (s->neighborlist == 1) { sopo_neighbor_list(s); sopo_pair_list(s); }
  else if (s->celllist == 1) { sopo_cell_list(s); sopo_pair_list(s); }
  if (do_initial_eval) { sopo_energy_eval(s); sopo_force_eval(s); }
  s->inlup = 1;
}

/* The loop body of underdamped_ctrl (sop.cpp:153-172). */
void sopo_run(sopo_sys* s, int nsteps) {
  for (int n = 0; n < nsteps; n++) {
    if ((s->inlup % s->nnlup) == 0) {
      if (s->neighborlist == 1) sopo_neighbor_list(s);
      else if (s->celllist == 1) sopo_cell_list(s);
      s->inlup = 0;
    }
    s->inlup++;
    if (s->neighborlist == 1 || s->celllist == 1) sopo_pair_list(s);
    sopo_iteration(s);
  }
}

int sopo_get_list(const sopo_sys* s, int which, int* ii, int* jj) {
  int n;
  const int* L;
  const int *A, *B;
  switch (which) {
    case 0: n = s->nnl_att; L = s->nl_att; A = s->ci; B = s->cj; break;
    case 1: n = s->nnl_rep; L = s->nl_rep; A = s->ri; B = s->rj; break;
    case 2: n = s->nil_att; L = s->pl_att; A = s->ci; B = s->cj; break;
    case 3: n = s->nil_rep; L = s->pl_rep; A = s->ri; B = s->rj; break;
    default: return -1;
  }
  if (ii && jj)
    for (int k = 0; k < n; k++) { ii[k] = A[L[k]] + 1; jj[k] = B[L[k]] + 1; }
  return n;
}

int sopo_get_count(const sopo_sys* s, const char* name) {
  if (!strcmp(name, "nbead")) return s->nbead;
  if (!strcmp(name, "nbnd")) return s->nbnd;
  if (!strcmp(name, "nang")) return s->nang;
  if (!strcmp(name, "ncon_att")) return s->nnat;
  if (!strcmp(name, "ncon_rep")) return s->nrep;
  if (!strcmp(name, "nnl_att")) return s->nnl_att;
  if (!strcmp(name, "nnl_rep")) return s->nnl_rep;
  if (!strcmp(name, "nil_att")) return s->nil_att;
  if (!strcmp(name, "nil_rep")) return s->nil_rep;
  if (!strcmp(name, "contct_nat")) return s->contct_nat;
  if (!strcmp(name, "inlup")) return s->inlup;
  return -1;
}

double sopo_get_energy(const sopo_sys* s, const char* name) {
  if (!strcmp(name, "e_bnd")) return s->e_bnd;
  if (!strcmp(name, "e_ang_ss")) return s->e_ang_ss;
  if (!strcmp(name, "e_vdw_rr")) return s->e_vdw;
  if (!strcmp(name, "e_vdw_rr_att")) return s->e_vdw_att;
  if (!strcmp(name, "e_vdw_rr_rep")) return s->e_vdw_rep;
  if (!strcmp(name, "rna_etot")) return s->etot;
  if (!strcmp(name, "Q")) return s->Q;
  if (!strcmp(name, "rgsq")) return s->rgsq;
  if (!strcmp(name, "kinT")) return s->kinT;
  return NAN;
}

/* ---- multi-threaded runner (CPU baseline) ------------------------------- */

typedef struct {
  sopo_sys** sys;
  int n, nsteps;
  int next;
  pthread_mutex_t mu;
} run_pool;

static void* run_worker(void* arg) {
  run_pool* p = (run_pool*)arg;
  for (;;) {
    pthread_mutex_lock(&p->mu);
    int k = p->next++;
    pthread_mutex_unlock(&p->mu);
    if (k >= p->n) break;
    sopo_run(p->sys[k], p->nsteps);
  }
  return NULL;
}

double sopo_run_many(sopo_sys** systems, int n, int nsteps, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  run_pool p;
  p.sys = systems;
  p.n = n;
  p.nsteps = nsteps;
  p.next = 0;
  pthread_mutex_init(&p.mu, NULL);
  pthread_t th[256];
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, run_worker, &p);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  pthread_mutex_destroy(&p.mu);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
