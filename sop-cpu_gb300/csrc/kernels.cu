// GB300 kernels of the SOP hot path.
//
//   k_prep      one cooperative launch per step: K0 per-replica step
//               bookkeeping (phase, noise counter, the reference's nnlup
//               cadence or the displacement trigger) that publishes the
//               step's due work units, K1 the cell binning of every replica
//               whose lists are rebuilt this step (one CTA per replica:
//               shared-memory counting sort into global bins, bead order
//               within a cell), and, in the same CTAs as consumers, K2
//               neighbor/pair-list enumeration in slices of beads over the
//               binned stencil (one warp per bead, cutoffs decided bit-exactly
//               against the reference's FP64 arithmetic), output-step
//               energies and observables.
//   k_step      K3+K4 fused: pair/bond/angle forces in FP32 from positions
//               staged in shared memory by TMA bulk copies, lane partials to
//               int64 fixed point and reduced with warp shuffles, counter-
//               based Langevin noise drawn in-kernel, the underdamped update
//               with FP64 position accumulation, next step's pair-list bits.
//   k_step_w    the same step with warps as independent workers over L1/L2.
//   k_energy    K5 energy terms in FP64 with a fixed-order reduction.
//   k_obs       K6 observables (Q, Rg^2, kinT) in FP64.
//   k_pairlist  update_pair_list at the current positions.
//   k_export    pair lists as (i<j) pairs for checking.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/sop_gpu.h"
#include "kernels.cuh"
#include "sop_common.cuh"

namespace sop {

__constant__ FFTables c_ff;

void upload_tables(const FFTables& t, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_ff, &t, sizeof(FFTables), 0, cudaMemcpyHostToDevice, s);
}

// ---------------------------------------------------------------------------------
// small helpers

// Checked build (-DSOP_CHECKED): every partner index read from a list row,
// cell bin, native, bond or angle record is tested against its replica's
// bead range before the gather; one outside it is recorded in the engine's
// error word (kErrIndex, reported by the call as SOP_ERR_INDEX) and the entry
// is skipped.  compute-sanitizer is not available on the GPUs this engine is
// tested on, so this build stands in for its bounds checks.  The default
// build compiles the checks out.
#ifdef SOP_CHECKED
__device__ __forceinline__ bool gather_ok(const DevArrays& A, int j, int n) {
  if ((unsigned)j < (unsigned)n) return true;
  atomicOr(A.err, kErrIndex);
  return false;
}
#define SOP_GATHER_OK(A, j, n) gather_ok((A), (j), (n))
#else
#define SOP_GATHER_OK(A, j, n) true
#endif

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ float rnd_f(float v) { return v > 0.f ? floorf(v + 0.5f) : ceilf(v - 0.5f); }

// A staged difference x_j - x_i in two floats (s + t): s = hj - hi rounded,
// t = its rounding error plus lj - li.  With IMG, the minimum image: the box
// shift k Lh comes off s exactly (|s - k Lh| <= boxl/2 is a multiple of the
// coarser ulp of the two, so the single rounding of the fma is exact) and
// k Ll off the small part, so an image keeps the accuracy of a plain pair.
struct BoxF {
  float Lh, Ll, invL;
};
template <bool IMG>
__device__ __forceinline__ void staged_diff(float hj, float lj, float hi, float lo, const BoxF& B,
                                            float& s, float& t) {
  float e;
  two_sum(hj, -hi, s, e);
  t = e + (lj - lo);
  if (IMG) {
    const float k = rnd_f(s * B.invL);
    s = fmaf(-k, B.Lh, s);
    t = fmaf(-k, B.Ll, t);
  }
}

// d^2 - r0^2 between two staged beads, in two-float arithmetic (Knuth's
// TwoSum, Dekker's exact product via FMA), accurate to ~2^-46 of d^2; also
// returns dx (float, i -> j) and d^2 (float).  r0^2 = r0h + r0l.  IMG: the
// minimum image of the difference (staged_diff).
template <bool IMG = false>
__device__ __forceinline__ float d2_minus(const float4& hi, const float4& lo, const float4& hj,
                                          const float4& lj, float r0h, float r0l, float& dx,
                                          float& dy, float& dz, float& d2, const BoxF& B = BoxF{}) {
  float sx, tx, sy, ty, sz, tz;
  staged_diff<IMG>(hj.x, lj.x, hi.x, lo.x, B, sx, tx);
  staged_diff<IMG>(hj.y, lj.y, hi.y, lo.y, B, sy, ty);
  staged_diff<IMG>(hj.z, lj.z, hi.z, lo.z, B, sz, tz);
  const float px = sx * sx, py = sy * sy, pz = sz * sz;
  const float pex = fmaf(sx, sx, -px), pey = fmaf(sy, sy, -py), pez = fmaf(sz, sz, -pz);
  float a, ea, bb, eb, c, ec;
  two_sum(px, py, a, ea);
  two_sum(a, pz, bb, eb);
  two_sum(bb, -r0h, c, ec);
  const float tail = ea + eb + ec + pex + pey + pez + 2.0f * (sx * tx + sy * ty + sz * tz) - r0l;
  dx = sx + tx;
  dy = sy + ty;
  dz = sz + tz;
  d2 = bb;
  return c + tail;
}

// FP64 squared distance with the reference's operation order and no FMA
// (neighbor_list.cpp:27-37, sop.cpp:496-507).  Callers guarantee the minimum
// image is the identity (extent checked at every build), as rnd(dx/boxl) = 0.
__device__ __forceinline__ double exact_d2(const double* X, long long cap, long long gi,
                                           long long gj) {
  double dx = __dsub_rn(X[gj], X[gi]);
  double dy = __dsub_rn(X[cap + gj], X[cap + gi]);
  double dz = __dsub_rn(X[2 * cap + gj], X[2 * cap + gi]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// The reference's minimum image of one FP64 difference, d - boxl rnd(d/boxl)
// (global.cpp:223-227, applied to every pair, bond and angle: energy.cpp,
// neighbor_list.cpp:27-37), in its operation order, no FMA.  The image of -d
// is minus the image of d (rnd rounds half away from zero), so the direction
// of the difference does not change d^2.
__device__ __forceinline__ double image_d(double d, double L) {
  const double q = __ddiv_rn(d, L);
  const double k = q > 0.0 ? floor(__dadd_rn(q, 0.5)) : ceil(__dsub_rn(q, 0.5));
  return __dsub_rn(d, __dmul_rn(L, k));
}

// exact_d2 with minimum images when L > 0 (replicas in image mode).
__device__ __forceinline__ double exact_d2i(const double* X, long long cap, long long gi,
                                            long long gj, double L) {
  double dx = __dsub_rn(X[gj], X[gi]);
  double dy = __dsub_rn(X[cap + gj], X[cap + gi]);
  double dz = __dsub_rn(X[2 * cap + gj], X[2 * cap + gi]);
  if (L > 0.0) {
    dx = image_d(dx, L);
    dy = image_d(dy, L);
    dz = image_d(dz, L);
  }
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// The reference's cell-list predicate (cell_list.cpp:24-41): cells
// floor(x / lcell), their index differences wrapped by ncell, adjacent when
// every wrapped difference lies in [-1, 1].  For replicas in image mode, whose
// grid is a single cell.
__device__ __forceinline__ bool cell_adjacent_ref(const double* X, long long cap, long long gi,
                                                  long long gj, double lc, double nc) {
  for (int c = 0; c < 3; c++) {
    const double ci = floor(__ddiv_rn(X[c * cap + gi], lc));
    const double cj = floor(__ddiv_rn(X[c * cap + gj], lc));
    const double cd = image_d(__dsub_rn(ci, cj), nc);
    if (!(cd >= -1.0 && cd <= 1.0)) return false;
  }
  return true;
}

// FP32 minimum image of a relative-position difference (screens only).
__device__ __forceinline__ float image_f(float d, float L, float invL) {
  return fmaf(-rnd_f(d * invL), L, d);
}

// d2 < rc2, screened in FP32 and re-decided in FP64 inside a relative band.
template <class Exact>
__device__ __forceinline__ bool within(float d2, float rc2f, float margin, Exact exact) {
  if (d2 < rc2f * (1.0f - margin)) return true;
  if (d2 > rc2f * (1.0f + margin)) return false;
  return exact();
}

__device__ __forceinline__ void bead_normals(unsigned seed_lo, unsigned seed_hi,
                                             long long t, int bead, float n[3]) {
  uint32_t ctr[4] = {(uint32_t)bead, (uint32_t)t, (uint32_t)((unsigned long long)t >> 32), 0u};
  uint32_t key[2] = {seed_lo, seed_hi};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  const float k32 = 2.3283064365386963e-10f, k33 = 1.1641532182693481e-10f;
  float u0 = fmaf(__uint2float_rn(o[0]), k32, k33);
  float u1 = fmaf(__uint2float_rn(o[1]), k32, k33);
  float u2 = fmaf(__uint2float_rn(o[2]), k32, k33);
  float u3 = fmaf(__uint2float_rn(o[3]), k32, k33);
  float r0 = sqrtf(-2.0f * logf(u0));
  float r1 = sqrtf(-2.0f * logf(u2));
  float s0, c0, s1, c1;
  sincospif(2.0f * u1, &s0, &c0);
  sincospif(2.0f * u3, &s1, &c1);
  n[0] = r0 * c0;
  n[1] = r0 * s0;
  n[2] = r1 * c1;
}

__device__ __forceinline__ bool finite3(float a, float b, float c) {
  return isfinite(a) && isfinite(b) && isfinite(c);
}

// ---- mbarrier + TMA bulk copy (cp.async.bulk) ------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                             unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------------------------
// K1: cell binning of one replica by one CTA into global memory
// K2: neighbor/pair-list enumeration of a slice of beads (build units)

constexpr int kWarpNat = 64;       // native partners per bead staged per warp

struct BuildSmem {
  int wnat[kBuildThreads / 32][kWarpNat];
  int wseg[kBuildThreads / 32][32];
  int s_maxrow, s_status;
};

__device__ __forceinline__ int bsearch_sorted(const int* a, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    int v = a[mid];
    if (v == key) return mid;
    if (v < key) lo = mid + 1;
    else hi = mid;
  }
  return -1;
}

// largest non-native list cutoff over the bead types present in replica R
__device__ __forceinline__ float list_cutoff_max(const RepDev* R, int mode) {
  float rl_max = 0.f;
  const int tmask = R->type_mask ? R->type_mask : 0x6;
  for (int a = 1; a < kMaxTypes; a++)
    for (int b = 1; b < kMaxTypes; b++) {
      if (!((tmask >> a) & 1) || !((tmask >> b) & 1)) continue;
      float rl = (mode == SOP_LIST_SKIN) ? (float)(2.5 * c_ff.sigma_rep[a][b]) + R->skin
                                         : (float)(3.2 * c_ff.sigma_rep[a][b]);
      rl_max = fmaxf(rl_max, rl);
    }
  return rl_max;
}

// Bin replica r's beads (positions of buffer `src`) into a cell grid held in
// global memory: relative positions + type/chain code, cell of each bead, the
// bead ids sorted by cell (bead order within a cell) and the cell starts.
// Cutoff modes use cells half a list cutoff wide (125-cell stencil); cell mode
// the reference's floor(x / lcell) cells (cell_list.cpp:24-31, 27-cell
// stencil); mode "none" one cell.  One CTA.
__device__ void bin_replica(const DevArrays& A, int r, int src, int mode, int* smem, int smem_ints) {
  __shared__ float red[6][32];
  __shared__ int wsum[32];
  __shared__ BinHdr H;
  RepDev* R = &A.rep[r];
  const int n = R->n, off = R->off, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const float4* S = A.stage[src] + 2 * (long long)off;
  const double* X = A.X[src];
  const long long cap = A.cap;
  int* cst = A.cstart + R->cell_base;
  int* ccur = A.ccur + R->cell_base;

  // 1. bounding box of the hi positions
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int i = tid; i < n; i += nt) {
    float4 h = S[2 * i];
    mn[0] = fminf(mn[0], h.x); mn[1] = fminf(mn[1], h.y); mn[2] = fminf(mn[2], h.z);
    mx[0] = fmaxf(mx[0], h.x); mx[1] = fmaxf(mx[1], h.y); mx[2] = fmaxf(mx[2], h.z);
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 3; c++) {
      mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
      mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
    }
  if (lane == 0)
    for (int c = 0; c < 3; c++) { red[c][warp] = mn[c]; red[3 + c][warp] = mx[c]; }
  __syncthreads();
  if (tid == 0) {
    float m0[3] = {3.4e38f, 3.4e38f, 3.4e38f}, m1[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int w = 0; w < nwarp; w++)
      for (int c = 0; c < 3; c++) {
        m0[c] = fminf(m0[c], red[c][w]);
        m1[c] = fmaxf(m1[c], red[3 + c][w]);
      }
    BinHdr h;
    h.ok = 0; h.status = 0; h.img = 0; h.nx = h.ny = h.nz = 1; h.K = 0; h.ncell = 1;
    h.edge = 3.0e38f; h.ox = m0[0]; h.oy = m0[1]; h.oz = m0[2]; h.cx0 = h.cy0 = h.cz0 = 0;
    h.margin = 1e-5f;
    const float rl_max = list_cutoff_max(R, mode);
    bool finite_box = true;
    for (int c = 0; c < 3; c++)
      finite_box = finite_box && isfinite(m0[c]) && isfinite(m1[c]) && m1[c] >= m0[c] &&
                   fabsf(m0[c]) < 1e6f && fabsf(m1[c]) < 1e6f;
    if (!finite_box) {  // non-finite or runaway positions: no grid can be built
      h.status = SOP_ST_NONFINITE;
    } else {
      const float ext = fmaxf(m1[0] - m0[0], fmaxf(m1[1] - m0[1], m1[2] - m0[2]));
      // minimum images (global.cpp:223-227) are the identity for every pair
      // while the extent stays below half the box by two list cutoffs; past
      // that, and always in mode none (no later build re-checks it), the
      // replica runs in image mode
      h.img = mode == SOP_LIST_NONE || (double)ext + 2.0 * rl_max >= 0.5 * R->boxl;
      // FP32 screening band: relative positions carry ~ext * 2^-24 of error
      if (rl_max > 0.f) h.margin = 1e-5f + 16.0f * ext * 5.9604645e-8f / rl_max;
      const long long ccap = R->cell_cap;
      if (mode == SOP_LIST_CELL) {
        const double lc = R->lcell;
        int c0[3], c1[3];
        for (int c = 0; c < 3; c++) {
          c0[c] = (int)floor(__ddiv_rn((double)m0[c] - 1e-3 * fabs((double)m0[c]) - 1e-3, lc));
          c1[c] = (int)floor(__ddiv_rn((double)m1[c] + 1e-3 * fabs((double)m1[c]) + 1e-3, lc));
        }
        h.cx0 = c0[0]; h.cy0 = c0[1]; h.cz0 = c0[2];
        h.nx = c1[0] - c0[0] + 1; h.ny = c1[1] - c0[1] + 1; h.nz = c1[2] - c0[2] + 1;
        if (2.0 * (double)(max(h.nx, max(h.ny, h.nz)) + 1) >= R->ncell) h.img = 1;  // cells wrap
        h.edge = (float)lc;
        h.K = 1;
        if ((long long)h.nx * h.ny * h.nz > ccap) h.status |= SOP_ST_GRID;
      } else if (mode != SOP_LIST_NONE) {
        // cells of the replica's cell edge, at least half a list cutoff wide
        // (0 = exactly half): K cells each way reach one cutoff, a 5x5x5
        // stencil below the cutoff, 3x3x3 from the cutoff up
        const float rcut = rl_max * 1.0001f + 1e-3f;
        float e = fmaxf(R->cell_edge, 0.5f * rcut);
        for (;;) {
          const long long nx = (long long)((m1[0] - m0[0]) / e) + 1;
          const long long ny = (long long)((m1[1] - m0[1]) / e) + 1;
          const long long nz = (long long)((m1[2] - m0[2]) / e) + 1;
          if (nx * ny * nz <= ccap) {
            h.nx = (int)nx; h.ny = (int)ny; h.nz = (int)nz;
            h.edge = e;
            break;
          }
          e *= 1.25f;
        }
        h.K = e >= rcut ? 1 : 2;
      }
      if (h.img) {
        // every bead a candidate of every other: one cell, decisions with images
        h.nx = h.ny = h.nz = 1;
        h.K = 0;
        h.edge = 3.0e38f;
        h.status &= ~SOP_ST_GRID;
      }
      h.ncell = h.nx * h.ny * h.nz;
      h.ok = !(h.status & SOP_ST_GRID);
    }
    // the replica's cutoffs, once per binning instead of once per listed bead.
    // Band width w: half the skin (skin lists), else 0.35 of the smallest
    // sigma present (half the 3.2 - 2.5 sigma gap of neighbor lists; any w
    // is exact, it only sets how many entries are far)
    double sig_min = 1e30;
    const int tm = R->type_mask ? R->type_mask : 0x6;
    for (int a = 1; a < kMaxTypes; a++)
      for (int b = 1; b < kMaxTypes; b++)
        if (((tm >> a) & 1) && ((tm >> b) & 1)) sig_min = fmin(sig_min, c_ff.sigma_rep[a][b]);
    const double band_w = (mode == SOP_LIST_SKIN) ? 0.5 * (double)R->skin : 0.35 * sig_min;
    for (int a = 0; a < kMaxTypes; a++)
      for (int b = 0; b < 2; b++) {
        const int ta = a ? a : 1, tb = b + 1;
        const double rl = 2.5 * c_ff.sigma_rep[ta][tb] + (double)R->skin;
        h.rl2d[a][b] = (mode == SOP_LIST_SKIN) ? rl * rl : c_ff.rc2_nl[ta][tb];
        h.pl2d[a][b] = c_ff.rc2_pl[ta][tb];  // (2.5 sigma)^2, sop.cpp:539-541
        h.rl2f[a][b] = (float)h.rl2d[a][b];
        h.pl2f[a][b] = (float)h.pl2d[a][b];
        const double bd = 2.5 * c_ff.sigma_rep[ta][tb] + band_w;
        h.bandf[a][b] = A.row_bands ? (float)(bd * bd) : 3.0e38f;  // off: nothing is far
      }
    R->band_w = (mode != SOP_LIST_NONE && A.row_bands) ? (float)band_w : 0.f;
    H = h;
  }
  __syncthreads();
  if (!H.ok) {
    if (tid == 0) {
      A.bin_hdr[r] = H;
      atomicOr(&R->status, H.status);
    }
    return;
  }
  const int nx = H.nx, ny = H.ny, nz = H.nz, ncell = H.ncell;
  const float edge = H.edge, ox = H.ox, oy = H.oy, oz = H.oz;

  // working arrays (counts / starts, cursors, sorted ids) in shared memory
  // when they fit, else directly in the replica's global bins
  int* const gsorted = A.bin_sorted + off;
  const bool local = 2LL * (ncell + 1) + n <= smem_ints;
  int* const wc = local ? smem : cst;
  int* const wq = local ? smem + ncell + 1 : ccur;
  int* const sorted = local ? smem + 2 * (ncell + 1) : gsorted;

  // 2. cell counts
  for (int c = tid; c <= ncell; c += nt) { wc[c] = 0; wq[c] = 0; }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const float4 hq = S[2 * i], lq = S[2 * i + 1];
    float4 p;
    p.x = (hq.x - ox) + lq.x;
    p.y = (hq.y - oy) + lq.y;
    p.z = (hq.z - oz) + lq.z;
    p.w = u2f(f2u(hq.w) | (f2u(lq.w) << 2));  // type | chain << 2
    A.bin_p[off + i] = p;
    int cx, cy, cz;
    if (H.img) {
      cx = cy = cz = 0;
    } else if (mode == SOP_LIST_CELL) {
      const double lc = R->lcell;
      cx = (int)floor(__ddiv_rn(X[off + i], lc)) - H.cx0;
      cy = (int)floor(__ddiv_rn(X[cap + off + i], lc)) - H.cy0;
      cz = (int)floor(__ddiv_rn(X[2 * cap + off + i], lc)) - H.cz0;
    } else if (mode == SOP_LIST_NONE) {
      cx = cy = cz = 0;
    } else {
      cx = (int)(p.x / edge);
      cy = (int)(p.y / edge);
      cz = (int)(p.z / edge);
    }
    cx = min(max(cx, 0), nx - 1); cy = min(max(cy, 0), ny - 1); cz = min(max(cz, 0), nz - 1);
    const int c = cx + nx * (cy + ny * cz);
    A.bin_cell[off + i] = c;
    atomicAdd(&wc[c], 1);
  }
  __syncthreads();

  // 3. exclusive scan of the ncell + 1 counts (contiguous chunk per thread)
  {
    const int N = ncell + 1, C = (N + nt - 1) / nt, a = min(N, tid * C), b = min(N, a + C);
    int s = 0;
    for (int k = a; k < b; k++) s += wc[k];
    int x = s;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int v = lane < nwarp ? wsum[lane] : 0, z = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, z, o);
        if (lane >= o) z += y;
      }
      if (lane < nwarp) wsum[lane] = z - v;
    }
    __syncthreads();
    int run = wsum[warp] + x - s;
    for (int k = a; k < b; k++) {
      const int v = wc[k];
      wc[k] = run;
      run += v;
    }
  }
  __syncthreads();

  // 4. scatter, then bead order inside every cell (deterministic rows)
  if (mode == SOP_LIST_NONE || H.img) {
    for (int i = tid; i < n; i += nt) sorted[i] = i;
  } else {
    for (int i = tid; i < n; i += nt) {
      const int c = A.bin_cell[off + i];
      sorted[wc[c] + atomicAdd(&wq[c], 1)] = i;
    }
    __syncthreads();
    for (int c = tid; c < ncell; c += nt) {
      const int a = wc[c], b = wc[c + 1];
      for (int k = a + 1; k < b; k++) {  // insertion sort (cells hold a few beads)
        const int v = sorted[k];
        int m = k - 1;
        while (m >= a && sorted[m] > v) {
          sorted[m + 1] = sorted[m];
          m--;
        }
        sorted[m + 1] = v;
      }
    }
  }
  __syncthreads();
  if (local) {
    for (int c = tid; c <= ncell; c += nt) cst[c] = wc[c];
    for (int i = tid; i < n; i += nt) gsorted[i] = sorted[i];
  }
  if (tid == 0) {
    A.bin_hdr[r] = H;
    R->img = H.img;
    if (H.status) atomicOr(&R->status, H.status);
  }
}

// Enumerate the list rows of beads [b0, b1) of replica r from its bins (one
// warp per bead).  The bins are copied into shared memory when they fit in
// `dyn_bytes`, else read from global memory (L2).  The lanes test 32
// stencil candidates at a time and ballot-compact the survivors, so each row
// holds its partners in stencil order, bead order within a cell.
template <bool IMG>
__device__ void build_slice(const DevArrays& A, int r, int src, int mode, int b0, int b1,
                            BuildSmem& B, unsigned char* dyn, int dyn_bytes) {
  RepDev* R = &A.rep[r];
  const BinHdr* H = A.bin_hdr + r;
  if (!H->ok) return;  // the binning recorded why
  const int n = R->n, off = R->off, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nx = H->nx, ny = H->ny, nz = H->nz, ncell = H->ncell, K = H->K, SK = 2 * K + 1;
  const int ncs = SK * SK * SK;
  const float4* S = A.stage[src] + 2 * (long long)off;
  const double* X = A.X[src];
  const long long cap = A.cap;
  // image mode: minimum images in every screen and decision, and in cell
  // mode the reference's wrapped cell predicate per pair
  const bool img = IMG;  // (the caller dispatches on the replica's binning)
  const float Lf = R->Lh, invLf = R->invL;
  const double Limg = IMG ? R->boxl : 0.0, lcell = R->lcell, ncellref = R->ncell;

  const float4* P = A.bin_p + off;
  const int* sorted = A.bin_sorted + off;
  const int* cell = A.bin_cell + off;
  const int* cst = A.cstart + R->cell_base;
  if ((long long)n * 24 + (long long)(ncell + 1) * 4 <= dyn_bytes) {
    float4* Ps = reinterpret_cast<float4*>(dyn);
    int* ss = reinterpret_cast<int*>(Ps + n);
    int* cs = ss + n;
    int* ts = cs + n;
    for (int i = tid; i < n; i += nt) {
      Ps[i] = P[i];
      ss[i] = sorted[i];
      cs[i] = cell[i];
    }
    for (int c = tid; c <= ncell; c += nt) ts[c] = cst[c];
    __syncthreads();
    P = Ps; sorted = ss; cell = cs; cst = ts;
  }
  if (tid == 0) { B.s_maxrow = 0; B.s_status = 0; }
  __syncthreads();

  const long long nl_base = R->nl_base;
  const int L = R->L;
  const float margin = H->margin;
  int my_status = 0, my_max = 0;
  int* wnat = B.wnat[warp];
  int* wseg = B.wseg[warp];  // per window position: sorted slot - candidate index of its cell
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nwarp = nt >> 5;
  // this lane's stencil cells 4 lane + q as packed offsets (dx+K | dy+K << 4 |
  // dz+K << 8), -1 past the stencil
  int soff[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int k = 4 * lane + q;
    soff[q] = k < ncs ? (k % SK) | (((k / SK) % SK) << 4) | ((k / (SK * SK)) << 8) : -1;
  }
  for (int i = b0 + warp; i < b1; i += nwarp) {
    const float4 pi = P[i];
    const int code_i = __float_as_int(pi.w), ti = code_i & 3, chi = code_i >> 2;
    const int c = cell[i];
    const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
    const int4 tp = A.topo[off + i];
    const int nat_cnt = tp.w & 0xFFFF;
    const int2 er = A.exc_rng[off + i];
    const long long row = nl_base + (long long)i * L;
    const long long gi = off + i;
    // the bead's native partners (sorted) staged for the exclusion test
    const bool nat_in_smem = nat_cnt <= kWarpNat;
    if (nat_in_smem)
      for (int k = lane; k < nat_cnt; k += 32) wnat[k] = A.nat[tp.x + k].x & (int)kIdx;
    __syncwarp();
    // list and pair cutoffs^2 against partner types 1 and 2
    const float rl2f1 = H->rl2f[ti][0], rl2f2 = H->rl2f[ti][1];
    const float pl2f1 = H->pl2f[ti][0], pl2f2 = H->pl2f[ti][1];
    // the stencil cells (dz, dy, dx from -K to K) flattened into one candidate
    // range: lane l owns stencil cells 4l..4l+3, a warp scan gives offsets
    int cnt4[4], beg4[4], lsum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      cnt4[q] = 0;
      beg4[q] = 0;
      if (soff[q] >= 0) {
        const int xx = cx + (soff[q] & 15) - K, yy = cy + ((soff[q] >> 4) & 15) - K,
                  zz = cz + (soff[q] >> 8) - K;
        if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) {
          const int cc = xx + nx * (yy + ny * zz);
          beg4[q] = cst[cc];
          cnt4[q] = cst[cc + 1] - beg4[q];
        }
      }
      lsum += cnt4[q];
    }
    int incl = lsum;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int pre0 = incl - lsum;  // candidate index of this lane's first cell
    int carry = 0;  // sorted slot - candidate index of the cell running into the window
    int cnt = 0;    // warp-uniform
    // pair-list entries fill the row from the front, the rest from the back, so
    // the step kernel's warps pass the force code of a row's skin entries in
    // step (the sums are exact, so entry order does not change any result)
    int cntp = 0;   // warp-uniform: entries in the pair list
    for (int base = 0; base < total; base += 32) {
      // every non-empty cell that starts inside the window marks its first
      // position; a lane's cell is the last mark at or before it
      unsigned bits = 0;
      {
        int pre = pre0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int at = pre - base;
          if (cnt4[q] > 0 && at >= 0 && at < 32) {
            bits |= 1u << at;
            wseg[at] = beg4[q] - pre;
          }
          pre += cnt4[q];
        }
      }
      const unsigned marks = __reduce_or_sync(0xffffffffu, bits);
      __syncwarp();
      const unsigned upto = marks & (0xffffffffu >> (31 - lane));
      const int segoff = upto ? wseg[31 - __clz(upto)] : carry;
      if (marks) carry = wseg[31 - __clz(marks)];
      __syncwarp();
      const int f = base + lane;
      bool pass = f < total;
      int j = 0, tj = 1;
      float d2 = 0.f;
      if (pass) {
        const int slot = segoff + f;
        j = SOP_GATHER_OK(A, slot, n) ? sorted[slot] : i;
        if (!SOP_GATHER_OK(A, j, n)) j = i;  // (dropped below)
        const float4 pj = P[j];
        const int code_j = __float_as_int(pj.w), chj = code_j >> 2;
        tj = code_j & 3;
        pass = j != i && !(chi == chj && abs(i - j) <= 2);
        float ddx = pj.x - pi.x, ddy = pj.y - pi.y, ddz = pj.z - pi.z;
        if (img) {
          ddx = image_f(ddx, Lf, invLf);
          ddy = image_f(ddy, Lf, invLf);
          ddz = image_f(ddz, Lf, invLf);
        }
        d2 = ddx * ddx + ddy * ddy + ddz * ddz;
      }
      const long long gj = off + j;
      if (pass && mode != SOP_LIST_NONE && mode != SOP_LIST_CELL) {
        const float rl2f = tj == 2 ? rl2f2 : rl2f1;
        pass = d2 <= rl2f * (1.0f + margin) &&
               within(d2, rl2f, margin,
                      [&] { return exact_d2i(X, cap, gi, gj, Limg) < H->rl2d[ti][tj == 2]; });
      } else if (pass && mode == SOP_LIST_CELL && img) {
        // cell adjacency is the whole predicate in cell mode (cell_list.cpp:86-88);
        // with a single cell it is decided per pair
        pass = cell_adjacent_ref(X, cap, gi, gj, lcell, ncellref);
      }
      if (pass) {  // natives are listed separately (sorted by partner)
        int lo = 0, hi = nat_cnt;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          const int v = nat_in_smem ? wnat[mid] : (A.nat[tp.x + mid].x & (int)kIdx);
          if (v == j) { pass = false; break; }
          if (v < j) lo = mid + 1;
          else hi = mid;
        }
      }
      if (pass && er.y > 0 && bsearch_sorted(A.exc + er.x, er.y, j) >= 0) pass = false;
      bool inp = false;
      if (pass) {
        if (mode == SOP_LIST_NONE) {
          inp = true;  // no pair-list filter without a cutoff type
        } else {
          inp = within(d2, tj == 2 ? pl2f2 : pl2f1, margin,
                       [&] { return exact_d2i(X, cap, gi, gj, Limg) < H->pl2d[ti][tj == 2]; });
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, pass);
      const unsigned mp = __ballot_sync(0xffffffffu, pass && inp);
      const int pos = inp ? cntp + __popc(mp & lt_mask)
                          : L - 1 - ((cnt - cntp) + __popc(m & ~mp & lt_mask));
      if (pass && pos >= 0 && pos < L) A.nl[row + pos] = j | (inp ? (int)kPL : 0);
      cnt += __popc(m);
      cntp += __popc(mp);
    }
    int near_end = min(cnt, L);  // row entries [near_end, cnt) are far
    const int nsk = cnt - cntp;
    if (cnt <= L && nsk > 0) {
      const long long src = row + L - nsk, dst = row + cntp;
      __syncwarp();
      if (mode != SOP_LIST_NONE && cnt + nsk <= L) {
        // the skin block [L - nsk, L) does not overlap [cntp, cnt): copy its
        // near entries down first, then its far ones (farther than the pair
        // cutoff plus the band width at these positions, with the screen's
        // relative band as a margin: an entry in doubt counts as near)
        int w0 = cntp;
        for (int pass = 0; pass < 2; pass++) {
          if (pass == 1) near_end = w0;
          for (int k0 = 0; k0 < nsk; k0 += 32) {
            const int k = k0 + lane;
            bool take = false;
            int v = 0;
            if (k < nsk) {
              v = A.nl[src + k];
              const int j = v & (int)kIdx;
              const float4 pj = P[j];
              float ddx = pj.x - pi.x, ddy = pj.y - pi.y, ddz = pj.z - pi.z;
              if (img) {
                ddx = image_f(ddx, Lf, invLf);
                ddy = image_f(ddy, Lf, invLf);
                ddz = image_f(ddz, Lf, invLf);
              }
              const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
              const int tj = __float_as_int(pj.w) & 3;
              const bool far = d2 > H->bandf[ti][tj == 2] * (1.0f + margin);
              take = pass == 0 ? !far : far;
            }
            const unsigned m = __ballot_sync(0xffffffffu, take);
            if (take) A.nl[dst - cntp + w0 + __popc(m & lt_mask)] = v;
            w0 += __popc(m);
          }
        }
      } else {
        // move the back block down to cntp (dest <= src, 32 entries at a
        // time, each chunk read before it is written); no far part
        for (int k0 = 0; k0 < nsk; k0 += 32) {
          const int k = k0 + lane;
          const int v = k < nsk ? A.nl[src + k] : 0;
          __syncwarp();
          if (k < nsk) A.nl[dst + k] = v;
          __syncwarp();
        }
      }
    }
    if (lane == 0) {
      if (cnt > L) my_status |= SOP_ST_LIST_OVERFLOW;
      my_max = max(my_max, cnt);
      A.nl_cnt[off + i] = min(cnt, L);
      A.nl_near[off + i] = near_end;
      const float4 h = S[2 * i];
      A.xb[off + i] = make_float4(h.x, h.y, h.z, 0.f);
    }
    __syncwarp();
    // natives: neighbor-list and pair-list bits, one lane per native entry
    for (int k = lane; k < nat_cnt; k += 32) {
      int4 e = A.nat[tp.x + k];
      int j = e.x & (int)kIdx;
      if (!SOP_GATHER_OK(A, j, n)) continue;
      float4 pj = P[j];
      float ddx = pj.x - pi.x, ddy = pj.y - pi.y, ddz = pj.z - pi.z;
      if (img) {
        ddx = image_f(ddx, Lf, invLf);
        ddy = image_f(ddy, Lf, invLf);
        ddz = image_f(ddz, Lf, invLf);
      }
      float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
      const float r0sq = __int_as_float(e.y);  // r0^2 rounded to FP32: the screen's cutoffs
      const long long gj = off + j;
      bool nlb, plb;
      if (mode == SOP_LIST_NEIGHBOR) {
        nlb = within(d2, 10.24f * r0sq, margin, [&] {
          const double rc = 3.2 * A.nat_r0[tp.x + k];  // neighbor_list.cpp:44-47
          return exact_d2i(X, cap, gi, gj, Limg) < rc * rc;
        });
      } else if (mode == SOP_LIST_CELL) {
        if (img) {
          nlb = cell_adjacent_ref(X, cap, gi, gj, lcell, ncellref);
        } else {
          int c2 = cell[j];
          int jx = c2 % nx, jy = (c2 / nx) % ny, jz = c2 / (nx * ny);
          nlb = abs(jx - cx) <= 1 && abs(jy - cy) <= 1 && abs(jz - cz) <= 1;
        }
      } else {
        nlb = true;
      }
      if (mode == SOP_LIST_NONE) {
        plb = true;
      } else if (nlb) {
        plb = within(d2, 6.25f * r0sq, margin, [&] {
          const double rc = 2.5 * A.nat_r0[tp.x + k];  // sop.cpp:504-506
          return exact_d2i(X, cap, gi, gj, Limg) < rc * rc;
        });
      } else {
        plb = false;
      }
      A.nat[tp.x + k].x = j | (nlb ? (int)kNL : 0) | (plb ? (int)kPL : 0);
    }
    __syncwarp();
  }
  atomicMax(&B.s_maxrow, my_max);
  if (my_status) atomicOr(&B.s_status, my_status);
  __syncthreads();
  if (tid == 0) {
    atomicMax(&R->max_row, B.s_maxrow);
    if (B.s_status) atomicOr(&R->status, B.s_status);
  }
}

__device__ void replica_energy(const DevArrays& A, RepDev* R, int buf, double* red);
__device__ void replica_obs(const DevArrays& A, RepDev* R, int buf, double* red);

// Work units of a step's preparation: {replica, kind | mode << 8, slice,
// buffer}.  A slot becomes valid when its replica id (x >= 0) is stored after
// the other fields and a fence; the consumer resets x to -1.
enum UnitKind : int { U_OBS = 1, U_BUILD = 2, U_ENERGY = 3 };

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void publish_unit(int4* slot, int r, int kind_mode, int slice, int buf) {
  slot->y = kind_mode;
  slot->z = slice;
  slot->w = buf;
  __threadfence();
  atomicExch(&slot->x, r);
}

__device__ __forceinline__ void push_units(const DevArrays& A, int r, int kind, int mode, int nsl,
                                           int buf) {
  const int base = atomicAdd(A.unit_cnt, nsl);
  for (int s = 0; s < nsl; s++)
    if (base + s < A.unit_cap) publish_unit(&A.units[base + s], r, kind | (mode << 8), s, buf);
}

// Per-replica step bookkeeping, one thread per replica: phase, noise counter,
// the reference's nnlup cadence or the displacement trigger, output steps.
// Due work goes to the unit queue, in this order of meaning:
//   observables of the previous output step (positions X_{t-1}, velocities v_{t-1}),
//   the list build from X_{t-1} in slices (sop.cpp:156-170: rebuild before the step),
//   the energies of this output step at X_t with pair list PL_t (after the build,
//   before the step kernel rewrites the pair-list bits).
// Returns -1, or the build due now as mode | buffer << 8 (its counters reset;
// the caller bins the replica, then publishes the build's slices).
// group: some replica's displacement trigger fired in the last step.
__device__ int decide_one(const DevArrays& A, int r, int force_build, int build_mode, int group) {
  RepDev* R = &A.rep[r];
  RepDev Q = *R;  // one pipelined copy; decide in registers, store back
  if (force_build) {  // build_mode < 0: the replica's own list mode
    const int mode = build_mode >= 0 ? build_mode : Q.mode;
    R->en_after = 0;
    A.slice_done[r] = 0;
    R->max_row = 0;
    return mode | (Q.cur << 8);
  }
  if (Q.obs_pending) {
    push_units(A, r, U_OBS, 0, 1, Q.cur);
    R->obs_pending = 0;
  }
  if (!Q.active || !Q.running ||
      (Q.status & (SOP_ST_NONFINITE | SOP_ST_LIST_OVERFLOW | SOP_ST_PERIODIC | SOP_ST_GRID))) {
    R->phase = PH_SKIP;
    R->out = 0;
    return -1;
  }
  bool need = false;
  const int prev = Q.cur;
  if (Q.moved) {
    if (Q.mode == SOP_LIST_NEIGHBOR || Q.mode == SOP_LIST_CELL) {
      // underdamped_ctrl cadence (sop.cpp:156-165), local inlup from 1
      if (Q.inlup % Q.nnlup == 0) { need = true; Q.inlup = 0; }
      Q.inlup++;
      R->inlup = Q.inlup;
    } else if (Q.mode == SOP_LIST_SKIN) {
      // its own trigger, or another replica's while this one is near its own
      need = Q.rebuild != 0 || (group && Q.near != 0);
    }
    Q.cur ^= 1;
    Q.moved = 0;
  }
  int ph;
  if (Q.first_pending) { ph = PH_FIRST; R->first_pending = 0; }
  else if (Q.t >= Q.t_end) ph = PH_FINAL;
  else ph = PH_NORMAL;
  R->t_cur = Q.t;
  if (ph == PH_FINAL) {
    R->running = 0;
    const int slot = atomicAdd(A.done_cnt, 1);
    if (slot < A.done_cap) A.done_list[slot] = r;
  } else {
    R->t = Q.t + 1;
    Q.moved = 1;
  }
  R->cur = Q.cur;
  R->moved = Q.moved;
  R->phase = ph;
  const int out = (ph == PH_NORMAL || ph == PH_FINAL) && Q.nup > 0 && Q.t > 0 && (Q.t % Q.nup) == 0;
  R->out = out;
  if (out) R->obs_pending = 1;
  R->en_after = need && out;
  if (need) {
    A.slice_done[r] = 0;
    R->max_row = 0;
  }
  if (out && !need) push_units(A, r, U_ENERGY, 0, 1, Q.cur);
  // work this replica may queue at the next step: the observables of this
  // output step, the energies of an output step, a cadence build.  (A skin
  // trigger raises any_rebuild in the step kernel; host-side changes make the
  // next k_prep a full one.)
  if (out || (ph != PH_FINAL &&
              ((Q.nup > 0 && (Q.t + 1) % Q.nup == 0) ||
               ((Q.mode == SOP_LIST_NEIGHBOR || Q.mode == SOP_LIST_CELL) &&
                (Q.nnlup <= 1 || Q.inlup % Q.nnlup == 0)))))
    A.prep_flag[1] = 1;
  return need ? (Q.mode | (prev << 8)) : -1;
}

// One unit: observables, energies, or a list-build slice.  The CTA that
// finishes the last slice of a build closes it (counters, displacement flag)
// and, on an output step, computes the energies with the new pair list.
__device__ void run_unit(const DevArrays& A, int4 w, BuildSmem& B, unsigned char* dyn, int dyn_bytes,
                         int* s_last) {
  double* red = reinterpret_cast<double*>(dyn);
  const int r = w.x, kind = w.y & 0xFF, mode = w.y >> 8;
  RepDev* R = &A.rep[r];
  if (kind == U_OBS) {
    replica_obs(A, R, w.w, red);
  } else if (kind == U_ENERGY) {
    replica_energy(A, R, w.w, red);
  } else if (kind == U_BUILD) {
    const int sb = A.slice_beads;
    const int n = R->n, nsl = (n + sb - 1) / sb;
    const int b0 = w.z * sb, b1 = min(n, b0 + sb);
    if (A.bin_hdr[r].img) build_slice<true>(A, r, w.w, mode, b0, b1, B, dyn, dyn_bytes);
    else build_slice<false>(A, r, w.w, mode, b0, b1, B, dyn, dyn_bytes);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      *s_last = atomicAdd(&A.slice_done[r], 1) == nsl - 1;
    }
    __syncthreads();
    if (*s_last) {
      __threadfence();
      if (threadIdx.x == 0) {
        R->builds += 1;
        R->rebuild = 0;
        R->near = 0;
        R->dmax2 = 0.f;
      }
      if (R->en_after) replica_energy(A, R, R->cur, red);
    }
  }
}

// After a staging wait ran out: how long the CTA lets its copy in flight land
// before it leaves (a copy of at most 227 KB takes microseconds).
constexpr unsigned long long kDrainNs = 10000000ULL;  // 10 ms

// K0 + K1 + K2 of a step in one cooperative launch (every CTA resident).
// Producers: CTA b owns the replicas k = b, b + grid, ...; its threads do
// their bookkeeping in parallel (one thread per replica, observables and
// energy units published at once), then the CTA bins, one after another, the
// replicas that rebuild and publishes each one's build slices.  Consumers:
// every CTA, once its own replicas are done, takes units in ticket order
// until all producers have finished and the queue is drained, so builds start
// while other replicas are still being binned.  nrep comes from device memory
// when nrep_dev is set, so a captured graph keeps working when replicas are
// admitted or retired.  The last CTA out resets the queue and clears the
// grouped-rebuild signal (every CTA has read it by then).
__global__ void __launch_bounds__(kBuildThreads, 2) k_prep(DevArrays A, const int* rep_ids,
                                                          const int* nrep_dev, int nrep_host,
                                                          int force_build, int build_mode,
                                                          int force_full, int dyn_bytes) {
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ BuildSmem B;
  __shared__ int s_build[kBuildThreads];
  __shared__ int s_base, s_last;
  __shared__ int4 s_unit;
  int* const bsm = reinterpret_cast<int*>(dyn);
  const int nrep = nrep_dev ? *nrep_dev : nrep_host;
  const int group = *A.any_rebuild;
  const int sb = A.slice_beads;
  // lean launch: no replica can queue work this step (no skin trigger, no
  // output, observables or cadence build flagged by the last k_prep), so the
  // CTAs skip the consumer phase and its wait for every producer
  const bool full = force_full || force_build || group || A.prep_flag[0];

  // A. producers
  const int mine = nrep > (int)blockIdx.x ? (nrep - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
  for (int m0 = 0; m0 < mine; m0 += (int)blockDim.x) {
    const int cnt = min(mine - m0, (int)blockDim.x);
    if ((int)threadIdx.x < cnt) {
      const int r = rep_ids[blockIdx.x + (m0 + threadIdx.x) * gridDim.x];
      s_build[threadIdx.x] = decide_one(A, r, force_build, build_mode, group);
    }
    __syncthreads();
    for (int q = 0; q < cnt; q++) {
      const int b = s_build[q];
      if (b < 0) continue;
      const int r = rep_ids[blockIdx.x + (m0 + q) * gridDim.x];
      bin_replica(A, r, b >> 8, b & 0xFF, bsm, dyn_bytes / 4);
      // the bins (written by the whole CTA) before the slices that read them
      __threadfence();
      __syncthreads();
      if (A.publish_delay_ns > 0) {  // diagnostics: a host-requested stall (bounded)
        if (threadIdx.x == 0) {
          const unsigned long long t0 = globaltimer_ns();
          while (globaltimer_ns() - t0 < (unsigned long long)A.publish_delay_ns) __nanosleep(1000);
        }
        __syncthreads();
      }
      const int nsl = (A.rep[r].n + sb - 1) / sb;
      if (threadIdx.x == 0) s_base = atomicAdd(A.unit_cnt, nsl);
      __syncthreads();
      for (int s = threadIdx.x; s < nsl; s += blockDim.x)
        if (s_base + s < A.unit_cap)
          publish_unit(&A.units[s_base + s], r, U_BUILD | ((b & 0xFF) << 8), s, b >> 8);
      __syncthreads();
    }
    __syncthreads();
  }
  // one fence after the barrier orders every unit this CTA queued (and the
  // descriptor fields its threads wrote) before the producer-done signal
  __syncthreads();
  if (full && threadIdx.x == 0) {
    __threadfence();
    atomicAdd(A.pro_done, 1);
  }

  // B. consumers (a lean launch has none; see below)
  bool consume = full;
  for (;;) {
    for (; consume;) {
      if (threadIdx.x == 0) {
        const int t = atomicAdd(A.unit_take, 1);
        int4 w = make_int4(-1, 0, 0, 0);
        const unsigned long long t0 = globaltimer_ns();
        for (;;) {
          if (t < min(ld_volatile(A.unit_cnt), A.unit_cap)) {
            const int x = ld_volatile(&A.units[t].x);
            if (x >= 0) {
              __threadfence();
              w = make_int4(x, ld_volatile(&A.units[t].y), ld_volatile(&A.units[t].z),
                            ld_volatile(&A.units[t].w));
              A.units[t].x = -1;  // free for the next step
              break;
            }
          } else if (ld_volatile(A.pro_done) == (int)gridDim.x) {
            __threadfence();
            if (t >= min(ld_volatile(A.unit_cnt), A.unit_cap)) break;  // drained
            continue;
          }
          if (globaltimer_ns() - t0 > (unsigned long long)A.queue_wait_ns) {
            atomicOr(A.err, 2);  // never expected: record and stop waiting
            break;
          }
        }
        s_unit = w;
      }
      __syncthreads();
      const int4 w = s_unit;
      if (w.x < 0) break;
      run_unit(A, w, B, dyn, dyn_bytes, &s_last);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(A.unit_exit, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (consume || ld_volatile(A.unit_cnt) == 0) break;
    // a lean launch that found work all the same (never expected): every
    // producer is done, so the last CTA out becomes the queue's only consumer
    // and results stay exact
    if (threadIdx.x == 0) {
      *A.pro_done = (int)gridDim.x;
      *A.unit_exit = (int)gridDim.x - 1;
      atomicAdd(A.prep_flag + 2, 1);
    }
    consume = true;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *A.unit_cnt = 0;
    *A.unit_take = 0;
    *A.pro_done = 0;
    *A.unit_exit = 0;
    if (!force_build) {
      *A.any_rebuild = 0;
      A.prep_flag[0] = ld_volatile(A.prep_flag + 1);
      A.prep_flag[1] = 0;
    }
  }
}

// ---------------------------------------------------------------------------------
// K3 + K4: fused force + underdamped step

struct ItemCtx {
  int r, off, n, cur, phase, terms, mode, out, ti_dummy;
  long long nl_base, t_cur;
  int L;
  float a1, a2, a3, a4, a5, amp, T, kbnd, inv_R0sq, fang, half_skin2, pull_f;
  int dyn;
  int pull_i, pull_j;
  unsigned seed_lo, seed_hi;
  int img;        // minimum images apply (the box itself is read per bead)
  float band_lim; // a bead displaced less than this since the build skips its
                  // row's far band (band width - largest displacement - 0.01 A;
                  // <= 0: rows are scanned whole)
  float dmax2;    // the replica's largest squared displacement (RepDev::dmax2)
};

// The box of an image-mode replica: FP32 two-float for the staged
// differences, FP64 for the exact decisions (0 = no image).
struct BoxCtx {
  BoxF f;
  double L;
};
template <bool IMG>
__device__ __forceinline__ BoxCtx box_ctx(const DevArrays& A, int r) {
  BoxCtx b{};
  if (IMG) {
    const RepDev* R = &A.rep[r];
    b.f = BoxF{R->Lh, R->Ll, R->invL};
    b.L = R->boxl;
  }
  return b;
}

// The step's view of replica r.
__device__ __forceinline__ ItemCtx load_ctx(const DevArrays& A, int r) {
  const RepDev* R = &A.rep[r];
  ItemCtx C;
  C.r = r; C.off = R->off; C.n = R->n; C.cur = R->cur; C.phase = R->phase;
  C.terms = R->terms; C.mode = R->mode; C.out = R->out;
  C.nl_base = R->nl_base; C.t_cur = R->t_cur; C.L = R->L;
  C.a1 = R->a1; C.a2 = R->a2; C.a3 = R->a3; C.a4 = R->a4; C.a5 = R->a5; C.dyn = R->dyn;
  C.amp = R->noise_amp; C.T = R->T; C.kbnd = R->kbnd; C.inv_R0sq = R->inv_R0sq; C.fang = R->fang;
  C.half_skin2 = R->half_skin2; C.pull_f = R->pull_f; C.pull_i = R->pull_i;
  C.img = R->img;
  C.dmax2 = R->dmax2;
  C.band_lim = R->band_w - 0.01f - sqrtf(C.dmax2);
  C.pull_j = R->pull_j; C.seed_lo = R->seed_lo; C.seed_hi = R->seed_hi;
  // a list build of this step that failed (row overflow, grid, periodic
  // image) leaves the replica frozen: no step on incomplete lists
  if (R->status & (SOP_ST_LIST_OVERFLOW | SOP_ST_PERIODIC | SOP_ST_GRID)) C.phase = PH_SKIP;
  return C;
}

template <bool ST>
__device__ __forceinline__ float4 ldp(const float4* S, int k) {
  if (ST) return S[k];
  return __ldg(S + k);
}

// Exact force accumulator of one bead (a lane's or a thread's share): every
// pair / bond / angle contribution is added in int64 fixed point, so the force
// is an exact integer sum, independent of list order, of how the entries are
// split among lanes or threads and of when the lists were built.
struct FixAcc {
  long long x = 0, y = 0, z = 0;
  float mag = 0.f;  // sum of |contributions|: bounds the int64 sums, carries NaN/inf
  int st = 0;
  __device__ __forceinline__ void add(float cx, float cy, float cz) {
    x += fixed_from_float(cx);
    y += fixed_from_float(cy);
    z += fixed_from_float(cz);
    mag += fabsf(cx) + fabsf(cy) + fabsf(cz);
  }
  // NaN, inf or a share out of the fixed-point range
  __device__ __forceinline__ int range_status() const { return mag <= kFixMax ? 0 : SOP_ST_NONFINITE; }
};

// The bead the contributions act on.
struct BeadRef {
  float4 hi, lo;  // staged position (hi, lo) with the type / chain codes
  int i, ti;      // index in the replica, bead type
  long long g;    // packed index
};

template <bool ST>
__device__ __forceinline__ BeadRef bead_ref(const ItemCtx& C, const float4* S, int i) {
  BeadRef b;
  b.hi = ldp<ST>(S, 2 * i);
  b.lo = ldp<ST>(S, 2 * i + 1);
  b.i = i;
  b.ti = (int)f2u(b.hi.w);
  b.g = (long long)C.off + i;
  return b;
}

// Native 12-6 attraction (energy.cpp:274-311) of native entry k (record e) of
// bead b, and its pair-list bit for the next step.  The force vanishes at the
// native distance, so (r0/d)^12 - (r0/d)^6 is formed from r0^2 - d^2 in
// two-float arithmetic: with u = r0^2/d^2 - 1, s^3 - 1 = u (u^2 + 3u + 3).
template <bool ST, bool IMG>
__device__ __forceinline__ void native_entry(const DevArrays& A, const ItemCtx& C, const float4* S,
                                             const BeadRef& b, int4 e, int k, bool upd,
                                             FixAcc& acc, const BoxCtx& bx) {
  const int j = e.x & (int)kIdx;
  if (!SOP_GATHER_OK(A, j, C.n)) return;
  const float4 hj = ldp<ST>(S, 2 * j), lj = ldp<ST>(S, 2 * j + 1);
  const float r0sq = __int_as_float(e.y);
  float dx, dy, dz, d2;
  const float diff = d2_minus<IMG>(b.hi, b.lo, hj, lj, r0sq, __int_as_float(e.z), dx, dy, dz, d2,
                                   bx.f);
  if (e.x & (int)kPL) {
    if (d2 >= (float)kTol * r0sq) {
      const int tj = (int)f2u(hj.w);
      const float inv = __fdividef(1.0f, d2);
      const float u = -diff * inv;                     // s - 1, s = r0^2/d^2
      const float s3m1 = u * fmaf(u, u + 3.0f, 3.0f);  // s^3 - 1
      const float s3 = 1.0f + s3m1;
      const float co = c_ff.fca[b.ti][tj] * inv * (s3 * s3m1);
      acc.add(co * dx, co * dy, co * dz);
    }
  }
  if (upd) {
    bool plb = false;
    if (e.x & (int)kNL) {
      plb = within(d2, 6.25f * r0sq, kScreenMargin, [&] {
        double rc = 2.5 * A.nat_r0[k], rc2 = rc * rc;
        return exact_d2i(A.X[C.cur], A.cap, b.g, (long long)C.off + j, bx.L) < rc2;
      });
    }
    if (plb != ((e.x & (int)kPL) != 0)) A.nat[k].x = e.x ^ (int)kPL;
  }
}

// Non-native repulsion (energy.cpp:313-350) of list entry e at row slot idx,
// and its pair-list bit for the next step.
template <bool IMG>
__device__ __forceinline__ void pair_delta(const BeadRef& b, const float4& hj, const float4& lj,
                                           const BoxF& B, float& dx, float& dy, float& dz) {
  if (!IMG) {
    dx = (hj.x - b.hi.x) + (lj.x - b.lo.x);
    dy = (hj.y - b.hi.y) + (lj.y - b.lo.y);
    dz = (hj.z - b.hi.z) + (lj.z - b.lo.z);
  } else {
    float s, t;
    staged_diff<true>(hj.x, lj.x, b.hi.x, b.lo.x, B, s, t);
    dx = s + t;
    staged_diff<true>(hj.y, lj.y, b.hi.y, b.lo.y, B, s, t);
    dy = s + t;
    staged_diff<true>(hj.z, lj.z, b.hi.z, b.lo.z, B, s, t);
    dz = s + t;
  }
}

template <bool ST, bool IMG>
__device__ __forceinline__ void nonnative_entry(const DevArrays& A, const ItemCtx& C, const float4* S,
                                                const BeadRef& b, int e, long long idx, bool upd,
                                                FixAcc& acc, const BoxCtx& bx) {
  const int j = e & (int)kIdx;
  if (!SOP_GATHER_OK(A, j, C.n)) return;
  const float4 hj = ldp<ST>(S, 2 * j), lj = ldp<ST>(S, 2 * j + 1);
  float dx, dy, dz;
  pair_delta<IMG>(b, hj, lj, bx.f, dx, dy, dz);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const int tj = (int)f2u(hj.w);
  const float s2 = c_ff.s2[b.ti][tj];
  if (e & (int)kPL) {
    if (d2 >= s2 * (float)kTol) {
      const float inv = __fdividef(1.0f, d2);
      const float s = s2 * inv, s3 = s * s * s;
      const float co = c_ff.fcr[b.ti][tj] * inv * (2.0f * s3 * s3 + s3);
      acc.add(co * dx, co * dy, co * dz);
    }
  }
  if (upd) {
    const bool plb = within(d2, c_ff.rc2_pl_f[b.ti][tj], kScreenMargin, [&] {
      return exact_d2i(A.X[C.cur], A.cap, b.g, (long long)C.off + j, bx.L) < c_ff.rc2_pl[b.ti][tj];
    });
    if (plb != ((e & (int)kPL) != 0)) A.nl[idx] = e ^ (int)kPL;
  }
}

// FENE (energy.cpp:402-447) of bond record bd; d^2 - r0^2 in two-float
// arithmetic so the stretch dev = (d^2 - r0^2)/(d + r0) keeps FP32 relative
// accuracy.
template <bool ST, bool IMG>
__device__ __forceinline__ void bond_entry(const ItemCtx& C, const float4* S, const BeadRef& b, int4 bd,
                                           FixAcc& acc, const BoxCtx& bx) {
  const int j = bd.x;
  const float r0 = __int_as_float(bd.y), r0h = __int_as_float(bd.z), r0l = __int_as_float(bd.w);
  const float4 hj = ldp<ST>(S, 2 * j), lj = ldp<ST>(S, 2 * j + 1);
  float dx, dy, dz, d2;
  const float diff = d2_minus<IMG>(b.hi, b.lo, hj, lj, r0h, r0l, dx, dy, dz, d2, bx.f);  // d^2 - r0^2
  const float d = sqrtf(d2);
  const float dev = __fdividef(diff, d + r0);
  const float den = 1.0f - dev * dev * C.inv_R0sq;
  if (!(den > 0.f)) acc.st |= SOP_ST_FENE;
  const float temp = __fdividef(-C.kbnd * dev, d * den);
  acc.add(-temp * dx, -temp * dy, -temp * dz);
}

// i,i+2 soft-sphere repulsion (energy.cpp:354-400) with partner j.
template <bool ST, bool IMG>
__device__ __forceinline__ void angle_entry(const ItemCtx& C, const float4* S, const BeadRef& b, int j,
                                            FixAcc& acc, const BoxCtx& bx) {
  const float4 hj = ldp<ST>(S, 2 * j), lj = ldp<ST>(S, 2 * j + 1);
  float dx, dy, dz;
  pair_delta<IMG>(b, hj, lj, bx.f, dx, dy, dz);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float d4 = d2 * d2, d8 = d4 * d4;
  const float co = __fdividef(C.fang, d8);
  acc.add(-co * dx, -co * dy, -co * dz);
}

// The bead's update from its exact force sum: noise, pulling force, the
// underdamped / overdamped step (FP64 position accumulation), the next
// staging, the skin trigger, status bits.
template <bool ST>
__device__ __forceinline__ void bead_tail(const DevArrays& A, const ItemCtx& C, const float4* S,
                                          const BeadRef& b, long long Fx, long long Fy, long long Fz,
                                          int st) {
  const long long cap = A.cap, g = b.g;
  const int i = b.i;
  const double* Xc = A.X[C.cur];
  float F[3] = {float_from_fixed(Fx), float_from_fixed(Fy), float_from_fixed(Fz)};
  if ((C.terms & SOP_TERM_RANDOM) && C.amp > 0.f) {
    float nrm[3];
    bead_normals(C.seed_lo, C.seed_hi, C.t_cur, i, nrm);
    F[0] += C.amp * nrm[0]; F[1] += C.amp * nrm[1]; F[2] += C.amp * nrm[2];
  }
  if (C.pull_f != 0.f && (i == C.pull_i || i == C.pull_j)) {
    const int o = (i == C.pull_i) ? C.pull_j : C.pull_i;
    const float4 ho = ldp<ST>(S, 2 * o), lo2 = ldp<ST>(S, 2 * o + 1);
    float ux = (ho.x - b.hi.x) + (lo2.x - b.lo.x), uy = (ho.y - b.hi.y) + (lo2.y - b.lo.y),
          uz = (ho.z - b.hi.z) + (lo2.z - b.lo.z);
    float inv = rsqrtf(ux * ux + uy * uy + uz * uz);
    F[0] -= C.pull_f * ux * inv; F[1] -= C.pull_f * uy * inv; F[2] -= C.pull_f * uz * inv;
  }
  if (C.phase == PH_FORCE || C.phase == PH_FINAL) {
    for (int c = 0; c < 3; c++) A.force[c * cap + g] = f2d_exact(F[c]);
  }
  if (C.phase != PH_FORCE) {
    float inc3[3];
    if (C.dyn == SOP_DYN_OVERDAMPED) {
      // overdamped_iteration (sop.cpp:331-363): incr = a5 F, no velocities; at
      // output steps the velocity array keeps the finished iteration's
      // increment, which calculate_observables reads (sop.cpp:270-278)
      if (C.phase != PH_FIRST && (C.out || C.phase == PH_FINAL))
        for (int c = 0; c < 3; c++) A.vel[c * cap + g] = f2d_exact(A.incr[c * cap + g]);
      for (int c = 0; c < 3; c++) inc3[c] = C.a5 * F[c];
    } else {
      const bool keepv = (C.phase == PH_FIRST) || (C.T < (float)kEpsT);
      float v[3];
      for (int c = 0; c < 3; c++) {
        if (keepv) {
          float h, l;
          split_double(A.vel[c * cap + g], h, l);
          v[c] = h;
        } else {
          v[c] = C.a3 * A.incr[c * cap + g] + C.a4 * F[c];
        }
      }
      if (!keepv && (C.out || C.phase == PH_FINAL))
        for (int c = 0; c < 3; c++) A.vel[c * cap + g] = f2d_exact(v[c]);
      for (int c = 0; c < 3; c++) inc3[c] = C.a1 * v[c] + C.a2 * F[c];
    }
    if (C.phase != PH_FINAL) {
      const int nb = C.cur ^ 1;
      float h[3], l[3];
      double xn[3];
      for (int c = 0; c < 3; c++) {
        const float inc = inc3[c];
        xn[c] = Xc[c * cap + g] + f2d_exact(inc);  // the FP64 accumulation
        A.X[nb][c * cap + g] = xn[c];
        A.incr[c * cap + g] = inc;
        split_double(xn[c], h[c], l[c]);
      }
      A.stage[nb][2 * g] = make_float4(h[0], h[1], h[2], b.hi.w);
      A.stage[nb][2 * g + 1] = make_float4(l[0], l[1], l[2], b.lo.w);
      if (C.mode != SOP_LIST_NONE) {  // displacement since the last list build
        const float4 xb = A.xb[g];
        const float ex = h[0] - xb.x, ey = h[1] - xb.y, ez = h[2] - xb.z;
        const float d2 = ex * ex + ey * ey + ez * ez;
        // the replica's largest displacement, read by the next step's band
        // test (h and xb are rounded to float: coordinates so large that two
        // ulps exceed the 0.01 A slack there make it unknown)
        const float ulp2 = 2.4e-7f * fmaxf(fabsf(h[0]), fmaxf(fabsf(h[1]), fabsf(h[2])));
        const float dd2 = ulp2 > 0.005f ? 3.0e38f : d2;
        if (dd2 > C.dmax2) atomicMax(reinterpret_cast<int*>(&A.rep[C.r].dmax2), __float_as_int(dd2));
        if (C.mode == SOP_LIST_SKIN) {
          if (d2 > C.half_skin2) {
            A.rep[C.r].rebuild = 1;
            *A.any_rebuild = 1;
          } else if (d2 > C.half_skin2 * A.group_frac2) {
            A.rep[C.r].near = 1;  // may rebuild with the next replica that must
          }
        }
      }
      if (!(isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]))) st |= SOP_ST_NONFINITE;
    }
  }
  if (!finite3(F[0], F[1], F[2])) st |= SOP_ST_NONFINITE;
  if (st) atomicOr(&A.rep[C.r].status, st);
}

// One bead on a group of G lanes: each lane takes every G-th native entry,
// list quad, bond and angle (loaded one iteration ahead), the lanes' exact
// partial sums are reduced with shuffles and lane 0 updates the bead.  IMG:
// the replica is in image mode (minimum images on every difference).
template <int G, bool ST, bool IMG = false>
__device__ __forceinline__ void step_bead(const DevArrays& A, const ItemCtx& C, const float4* S,
                                          int i, int lane, unsigned gmask) {
  const BeadRef b = bead_ref<ST>(C, S, i);
  const BoxCtx bx = box_ctx<IMG>(A, C.r);
  const int4 tp = A.topo[b.g];
  // the non-native row: rows start 32-byte aligned and hold a multiple of 8
  // entries, so a lane reads four entries with one 16-byte load (never past
  // the row); the lane's first quad is in flight during the natives.  While
  // no bead of the replica has moved half the band width since the build,
  // the row's far entries (farther than the pair cutoff plus the band width
  // at the build) cannot be in the pair list: their bits stay 0 and they are
  // not scanned (the pair filter stays exact).  Precisely: a far pair was at
  // least the pair cutoff + w apart at the build and each bead moved at most
  // its displacement since, so it stays outside the cutoff while this bead's
  // displacement plus the replica's largest one is below w
  int cnt = A.nl_cnt[b.g];
  if (C.band_lim > 0.f) {
    const float4 xb = A.xb[b.g];
    const float ex = b.hi.x - xb.x, ey = b.hi.y - xb.y, ez = b.hi.z - xb.z;
    if (sqrtf(ex * ex + ey * ey + ez * ez) < C.band_lim) cnt = A.nl_near[b.g];
  }
  const long long row = C.nl_base + (long long)i * C.L;
  const int4* row4 = reinterpret_cast<const int4*>(A.nl + row);
  int4 e4n = make_int4(0, 0, 0, 0);
  if (4 * lane < C.L) e4n = row4[lane];
  const int nat_cnt = tp.w & 0xFFFF, bnd_cnt = (tp.w >> 16) & 0xFF, ang_cnt = (tp.w >> 24) & 0xFF;
  int4 bn = make_int4(0, 0, 0, 0);
  int an = 0;
  if (lane < bnd_cnt) bn = A.bnd[tp.y + lane];
  if (lane < ang_cnt) an = A.ang[tp.z + lane];
  const bool upd = (C.phase == PH_FIRST || C.phase == PH_NORMAL) && C.mode != SOP_LIST_NONE;
  FixAcc acc;
  if (C.terms & SOP_TERM_VDW) {
    int4 en = make_int4(0, 0, 0, 0);  // the lane's next native record, loaded one entry ahead
    if (lane < nat_cnt) en = A.nat[tp.x + lane];
    for (int k = lane; k < nat_cnt; k += G) {
      const int4 e = en;
      if (k + G < nat_cnt) en = A.nat[tp.x + k + G];
      native_entry<ST, IMG>(A, C, S, b, e, tp.x + k, upd, acc, bx);
    }
    for (int q = lane; 4 * q < cnt; q += G) {
      const int4 e4 = e4n;
      if (4 * (q + G) < cnt) e4n = row4[q + G];
      const int ev[4] = {e4.x, e4.y, e4.z, e4.w};
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int k = 4 * q + u;
        if (k >= cnt) break;
        nonnative_entry<ST, IMG>(A, C, S, b, ev[u], row + k, upd, acc, bx);
      }
    }
  }
  if (C.terms & SOP_TERM_FENE) {
    for (int k = lane; k < bnd_cnt; k += G) {
      const int4 bd = bn;
      if (k + G < bnd_cnt) bn = A.bnd[tp.y + k + G];
      if (SOP_GATHER_OK(A, bd.x, C.n)) bond_entry<ST, IMG>(C, S, b, bd, acc, bx);
    }
  }
  if (C.terms & SOP_TERM_ANGLE) {
    for (int k = lane; k < ang_cnt; k += G) {
      const int j = an;
      if (k + G < ang_cnt) an = A.ang[tp.z + k + G];
      if (SOP_GATHER_OK(A, j, C.n)) angle_entry<ST, IMG>(C, S, b, j, acc, bx);
    }
  }
  // exact cross-lane sum of the fixed-point partials
  int st = acc.st | acc.range_status();
  long long Fx = acc.x, Fy = acc.y, Fz = acc.z;
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    Fx += __shfl_xor_sync(gmask, Fx, o, G);
    Fy += __shfl_xor_sync(gmask, Fy, o, G);
    Fz += __shfl_xor_sync(gmask, Fz, o, G);
  }
  st |= __reduce_or_sync(gmask, st);
  if (lane != 0) return;
  bead_tail<ST>(A, C, S, b, Fx, Fy, Fz, st);
}

// TPB: largest block size (256, or 512 for the wide variants); MB: resident
// CTAs of TPB threads per SM the register allocation is sized for
template <int G, int MB, int TPB = 256>
__global__ void __launch_bounds__(TPB, MB) k_step(DevArrays A, const StepItem* items,
                                                 const int* nitems_dev, int nitems_host,
                                                 const int* cta_first) {
  const int nitems = nitems_dev ? *nitems_dev : nitems_host;
  extern __shared__ __align__(128) float4 sst[];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ ItemCtx sC;
  __shared__ int s_block;
  const int lane = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G, ngrp = blockDim.x / G;
  const unsigned gmask =
      (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  if (threadIdx.x == 0) mbar_init(&mbar, 1);
  fence_async_smem();
  __syncthreads();
  uint32_t parity = 0;
  // The CTA's work items: one contiguous block [cta_first[b], cta_first[b + 1])
  // when the host split the items by estimated cost (else equal item counts),
  // or (blk_dyn) blocks of about equal estimated cost: CTA b's first block is
  // block b, and the blocks past the grid are taken in turn from the queue
  // blk_q = {next block, CTAs done, blocks}, so that CTAs whose rows run
  // short take more of them; the last CTA to finish resets the queue for the
  // next launch.  Consecutive items of one replica merge into one bead range,
  // staged once.  (A CTA's time is set by its chain of items, each with a
  // fixed staging and row-latency cost on top of its beads.)
  const bool dyn = A.blk_dyn != 0;
  bool first = true;
  int it = 0, it_end = 0;
  if (!dyn) {
    const int per = (nitems + (int)gridDim.x - 1) / (int)gridDim.x;
    it = cta_first ? min(nitems, cta_first[blockIdx.x]) : (int)blockIdx.x * per;
    it_end = cta_first ? min(nitems, cta_first[blockIdx.x + 1]) : min(nitems, ((int)blockIdx.x + 1) * per);
  }
  for (;;) {
    if (it >= it_end) {
      if (!dyn) break;
      int k = (int)blockIdx.x;
      if (!first) {
        if (threadIdx.x == 0) s_block = (int)gridDim.x + atomicAdd(A.blk_q, 1);
        __syncthreads();
        k = s_block;
        __syncthreads();  // s_block is rewritten by the next take
      }
      first = false;
      if (k >= A.blk_q[2]) break;
      const int2 bk = A.blk[k];
      it = min(nitems, bk.x);
      it_end = min(nitems, bk.y);
      continue;
    }
    StepItem w = items[it];
    int nx = it + 1;
    for (; nx < it_end; ++nx) {
      const StepItem v = items[nx];
      if (v.r != w.r) break;
      w.b1 = v.b1;
    }
    it = nx;
    if (threadIdx.x == 0) {
      const ItemCtx C = load_ctx(A, w.r);
      sC = C;
      if (C.phase != PH_SKIP && w.staged) {
        const char* src = reinterpret_cast<const char*>(A.stage[C.cur] + 2 * (long long)C.off);
        const uint32_t bytes = (uint32_t)C.n * 32u;
        fence_async_smem();
        mbar_expect_tx(&mbar, bytes);
        if (!A.skip_stage_copy)  // (diagnostics: expected but not issued)
          for (uint32_t o = 0; o < bytes; o += 32768u) {
            const uint32_t b = (bytes - o < 32768u) ? bytes - o : 32768u;
            tma_bulk_g2s(reinterpret_cast<char*>(sst) + o, src + o, b, &mbar);
          }
      }
    }
    __syncthreads();
    const ItemCtx C = sC;
    if (C.phase != PH_SKIP) {
      if (w.staged) {
        const unsigned long long t0 = globaltimer_ns();
        bool late = false;
        while (!mbar_try_wait(&mbar, parity)) {
          if (globaltimer_ns() - t0 > (unsigned long long)A.stage_wait_ns) {
            late = true;
            break;
          }
        }
        if (__syncthreads_or(late)) {
          // never expected: record it, let the copy in flight land in this
          // CTA's shared memory (bounded), and leave the step
          if (threadIdx.x == 0) atomicOr(A.err, 1);
          const unsigned long long t1 = globaltimer_ns();
          while (!mbar_try_wait(&mbar, parity) && globaltimer_ns() - t1 < kDrainNs) {
          }
          break;
        }
        parity ^= 1u;
        if (C.img)
          for (int b = w.b0 + grp; b < w.b1; b += ngrp) step_bead<G, true, true>(A, C, sst, b, lane, gmask);
        else
          for (int b = w.b0 + grp; b < w.b1; b += ngrp) step_bead<G, true>(A, C, sst, b, lane, gmask);
      } else {
        const float4* S = A.stage[C.cur] + 2 * (long long)C.off;
        if (C.img)
          for (int b = w.b0 + grp; b < w.b1; b += ngrp) step_bead<G, false, true>(A, C, S, b, lane, gmask);
        else
          for (int b = w.b0 + grp; b < w.b1; b += ngrp) step_bead<G, false>(A, C, S, b, lane, gmask);
      }
    }
    __syncthreads();
  }
  // every CTA passes here (a late staging copy included), so the queue is
  // reset once all CTAs have taken their last block
  if (dyn && threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(A.blk_q + 1, 1) == (int)gridDim.x - 1) {
      A.blk_q[0] = 0;
      A.blk_q[1] = 0;
      __threadfence();
    }
  }
}

// The same step with warps as independent workers: each warp takes work items
// from a global counter and steps their beads 32/G at a time, gathering
// partner positions through L1/L2 (no shared-memory staging, no block
// barriers, dynamic balance).  Per-bead arithmetic is step_bead's, so results
// are bit-identical to k_step's.  ctr[0] hands out items, ctr[1] counts
// finished warps; the last warp resets both for the next launch.
template <int G, int MB>
__global__ void __launch_bounds__(256, MB) k_step_w(DevArrays A, const StepItem* items,
                                                   const int* nitems_dev, int nitems_host,
                                                   const int*) {
  const int nitems = nitems_dev ? *nitems_dev : nitems_host;
  const int l32 = threadIdx.x & 31;
  const int lane = l32 & (G - 1), grp = l32 / G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (l32 & ~(G - 1)));
  for (;;) {
    int it = 0;
    if (l32 == 0) it = atomicAdd(A.step_ctr, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const StepItem w = items[it];
    const ItemCtx C = load_ctx(A, w.r);
    if (C.phase == PH_SKIP) continue;
    const float4* S = A.stage[C.cur] + 2 * (long long)C.off;
    if (C.img)
      for (int b = w.b0 + grp; b < w.b1; b += 32 / G) step_bead<G, false, true>(A, C, S, b, lane, gmask);
    else
      for (int b = w.b0 + grp; b < w.b1; b += 32 / G) step_bead<G, false>(A, C, S, b, lane, gmask);
  }
  if (l32 == 0) {
    __threadfence();
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    if (atomicAdd(A.step_ctr + 1, 1) == warps - 1) {
      A.step_ctr[0] = 0;
      A.step_ctr[1] = 0;
    }
  }
}

// ---------------------------------------------------------------------------------
// K3+K4 in FP64 (replicas with precision SOP_PREC_FP64): one thread per bead,
// positions, forces and the update in double precision with the reference's
// formulas (energy.cpp:259-447, sop.cpp:282-363), pair-list decisions exact as
// in the mixed kernel, contributions summed in int64 fixed point (2^-40) so
// that the sums do not depend on list order.  The drift / force-error
// reference for the mixed-precision path.

__device__ __forceinline__ long long fix40(double v) { return __double2ll_rn(v * 1099511627776.0); }

__device__ void step_bead64(const DevArrays& A, const ItemCtx& C, const RepDev* R, int i) {
  const long long g = (long long)C.off + i, cap = A.cap;
  const double* X = A.X[C.cur];
  const double xi = X[g], yi = X[cap + g], zi = X[2 * cap + g];
  const int ti = (int)f2u(A.stage[C.cur][2 * g].w);
  const int4 tp = A.topo[g];
  const int nat_cnt = tp.w & 0xFFFF, bnd_cnt = (tp.w >> 16) & 0xFF, ang_cnt = (tp.w >> 24) & 0xFF;
  const bool upd = (C.phase == PH_FIRST || C.phase == PH_NORMAL) && C.mode != SOP_LIST_NONE;
  long long Fx = 0, Fy = 0, Fz = 0;
  double mag = 0.0;
  int st = 0;
  auto add = [&](double cx, double cy, double cz) {
    Fx += fix40(cx);
    Fy += fix40(cy);
    Fz += fix40(cz);
    mag += fabs(cx) + fabs(cy) + fabs(cz);
  };
  // the pair difference with the reference's minimum image (raw: without,
  // for the pulling term, which has no reference counterpart)
  auto delta_raw = [&](int j, double& dx, double& dy, double& dz) {
    const long long gj = (long long)C.off + j;
    dx = __dsub_rn(X[gj], xi);
    dy = __dsub_rn(X[cap + gj], yi);
    dz = __dsub_rn(X[2 * cap + gj], zi);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  };
  auto delta = [&](int j, double& dx, double& dy, double& dz) {
    const long long gj = (long long)C.off + j;
    dx = __dsub_rn(X[gj], xi);
    dy = __dsub_rn(X[cap + gj], yi);
    dz = __dsub_rn(X[2 * cap + gj], zi);
    if (C.img) {
      dx = image_d(dx, R->boxl);
      dy = image_d(dy, R->boxl);
      dz = image_d(dz, R->boxl);
    }
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  };
  if (C.terms & SOP_TERM_VDW) {
    for (int k = 0; k < nat_cnt; k++) {  // native attraction (energy.cpp:274-311)
      const int4 e = A.nat[tp.x + k];
      const int j = e.x & (int)kIdx;
      if (!SOP_GATHER_OK(A, j, C.n)) continue;
      double dx, dy, dz;
      const double d2 = delta(j, dx, dy, dz);
      const double r0 = A.nat_r0[tp.x + k], r2 = r0 * r0;
      if (e.x & (int)kPL) {
        if (!(d2 < kTol * r2)) {
          const int tj = (int)f2u(A.stage[C.cur][2 * ((long long)C.off + j)].w);
          const double r6 = r2 * r2 * r2, r12 = r6 * r6;
          const double d6 = d2 * d2 * d2, d12 = d6 * d6;
          const double co = c_ff.force_coeff_att[ti][tj] / d2 * ((r12 / d12) - (r6 / d6));
          add(co * dx, co * dy, co * dz);
        }
      }
      if (upd) {
        const double rc = 2.5 * r0;  // sop.cpp:504-506
        const bool plb = (e.x & (int)kNL) && d2 < rc * rc;
        if (plb != ((e.x & (int)kPL) != 0)) A.nat[tp.x + k].x = e.x ^ (int)kPL;
      }
    }
    const int cnt = A.nl_cnt[g];
    const long long row = C.nl_base + (long long)i * C.L;
    for (int k = 0; k < cnt; k++) {  // non-native repulsion (energy.cpp:313-350)
      const int e = A.nl[row + k];
      const int j = e & (int)kIdx;
      if (!SOP_GATHER_OK(A, j, C.n)) continue;
      double dx, dy, dz;
      const double d2 = delta(j, dx, dy, dz);
      const int tj = (int)f2u(A.stage[C.cur][2 * ((long long)C.off + j)].w);
      if (e & (int)kPL) {
        if (!(d2 < c_ff.sigma_rep2[ti][tj] * kTol)) {
          const double d6 = d2 * d2 * d2, d12 = d6 * d6;
          const double co = c_ff.force_coeff_rep[ti][tj] / d2 *
                            (2.0 * c_ff.sigma_rep12[ti][tj] / d12 + c_ff.sigma_rep6[ti][tj] / d6);
          add(co * dx, co * dy, co * dz);
        }
      }
      if (upd) {
        const bool plb = d2 < c_ff.rc2_pl[ti][tj];
        if (plb != ((e & (int)kPL) != 0)) A.nl[row + k] = e ^ (int)kPL;
      }
    }
  }
  if (C.terms & SOP_TERM_FENE) {
    for (int k = 0; k < bnd_cnt; k++) {  // FENE (energy.cpp:402-447)
      const int j = A.bnd[tp.y + k].x;
      if (!SOP_GATHER_OK(A, j, C.n)) continue;
      double dx, dy, dz;
      const double d = sqrt(delta(j, dx, dy, dz));
      const double dev = d - A.bnd_r0[tp.y + k];
      const double den = 1.0 - dev * dev / R->R0sq_d;
      if (!(den > 0.0)) st |= SOP_ST_FENE;
      const double temp = -R->kbnd_d * dev / d / den;
      add(-temp * dx, -temp * dy, -temp * dz);
    }
  }
  if (C.terms & SOP_TERM_ANGLE) {
    for (int k = 0; k < ang_cnt; k++) {  // i,i+2 soft sphere (energy.cpp:354-400)
      const int j = A.ang[tp.z + k];
      if (!SOP_GATHER_OK(A, j, C.n)) continue;
      double dx, dy, dz;
      const double d2 = delta(j, dx, dy, dz);
      const double d4 = d2 * d2, d8 = d4 * d4;
      const double co = R->fang_d / d8;
      add(-co * dx, -co * dy, -co * dz);
    }
  }
  if (!(mag <= (double)kFixMax)) st |= SOP_ST_NONFINITE;
  double F[3] = {(double)Fx * 9.094947017729282e-13, (double)Fy * 9.094947017729282e-13,
                 (double)Fz * 9.094947017729282e-13};  // 2^-40
  if ((C.terms & SOP_TERM_RANDOM) && R->noise_amp_d > 0.0) {
    float nrm[3];
    bead_normals(C.seed_lo, C.seed_hi, C.t_cur, i, nrm);
    for (int c = 0; c < 3; c++) F[c] += R->noise_amp_d * (double)nrm[c];
  }
  if (C.pull_f != 0.f && (i == C.pull_i || i == C.pull_j)) {
    const int o = (i == C.pull_i) ? C.pull_j : C.pull_i;
    double ux, uy, uz;
    const double inv = 1.0 / sqrt(delta_raw(o, ux, uy, uz));
    const double pf = R->pull_fd;
    F[0] -= pf * ux * inv; F[1] -= pf * uy * inv; F[2] -= pf * uz * inv;
  }
  if (C.phase == PH_FORCE || C.phase == PH_FINAL)
    for (int c = 0; c < 3; c++) A.force[c * cap + g] = F[c];
  if (C.phase != PH_FORCE) {
    double inc[3];
    if (C.dyn == SOP_DYN_OVERDAMPED) {
      if (C.phase != PH_FIRST && (C.out || C.phase == PH_FINAL))
        for (int c = 0; c < 3; c++) A.vel[c * cap + g] = A.incr64[c * cap + g];
      for (int c = 0; c < 3; c++) inc[c] = R->a5d * F[c];
    } else {
      const bool keepv = (C.phase == PH_FIRST) || (C.T < (float)kEpsT);
      double v[3];
      for (int c = 0; c < 3; c++)
        v[c] = keepv ? A.vel[c * cap + g] : R->a3d * A.incr64[c * cap + g] + R->a4d * F[c];
      if (!keepv && (C.out || C.phase == PH_FINAL))
        for (int c = 0; c < 3; c++) A.vel[c * cap + g] = v[c];
      for (int c = 0; c < 3; c++) inc[c] = R->a1d * v[c] + R->a2d * F[c];
    }
    if (C.phase != PH_FINAL) {
      const int nb = C.cur ^ 1;
      const double xo[3] = {xi, yi, zi};
      float h[3], l[3];
      double xn[3];
      for (int c = 0; c < 3; c++) {
        xn[c] = xo[c] + inc[c];
        A.X[nb][c * cap + g] = xn[c];
        A.incr64[c * cap + g] = inc[c];
        A.incr[c * cap + g] = (float)inc[c];
        split_double(xn[c], h[c], l[c]);
      }
      const float4 hi = A.stage[C.cur][2 * g], lo = A.stage[C.cur][2 * g + 1];
      A.stage[nb][2 * g] = make_float4(h[0], h[1], h[2], hi.w);
      A.stage[nb][2 * g + 1] = make_float4(l[0], l[1], l[2], lo.w);
      if (C.mode == SOP_LIST_SKIN) {
        const float4 b = A.xb[g];
        const float ex = h[0] - b.x, ey = h[1] - b.y, ez = h[2] - b.z;
        const float d2 = ex * ex + ey * ey + ez * ez;
        if (d2 > C.half_skin2) {
          A.rep[C.r].rebuild = 1;
          *A.any_rebuild = 1;
        } else if (d2 > C.half_skin2 * A.group_frac2) {
          A.rep[C.r].near = 1;
        }
      }
      if (!(isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]))) st |= SOP_ST_NONFINITE;
    }
  }
  if (!(isfinite(F[0]) && isfinite(F[1]) && isfinite(F[2]))) st |= SOP_ST_NONFINITE;
  if (st) atomicOr(&A.rep[C.r].status, st);
}

// One CTA per work item, one thread per bead.
__global__ void __launch_bounds__(256) k_step64(DevArrays A, const StepItem* items,
                                                const int* nitems_dev, int nitems_host) {
  const int nitems = nitems_dev ? *nitems_dev : nitems_host;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const StepItem w = items[it];
    const ItemCtx C = load_ctx(A, w.r);
    if (C.phase == PH_SKIP) continue;
    for (int b = w.b0 + (int)threadIdx.x; b < w.b1; b += (int)blockDim.x)
      step_bead64(A, C, &A.rep[w.r], b);
  }
}

// ---------------------------------------------------------------------------------
// K5: energies in FP64 (energy.cpp:115-257), deterministic fixed-order sums

__device__ void block_sum(double* v, int nv, double* red) {
  // red: [nv][blockDim], reduced in a fixed tree order
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int q = 0; q < nv; q++) red[q * nt + tid] = v[q];
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s)
      for (int q = 0; q < nv; q++) red[q * nt + tid] += red[q * nt + tid + s];
    __syncthreads();
  }
  for (int q = 0; q < nv; q++) v[q] = red[q * nt];
  __syncthreads();
}

// Energy sums of beads [b0, b1) of one replica at positions X[buf] with the
// current pair list, this thread's share (beads b0 + tid, b0 + tid + blockDim,
// ...; each pair counted once, from its lower-index bead): v = {FENE log sum,
// angle sum, native sum, repulsion}.
__device__ void energy_terms(const DevArrays& A, const RepDev* R, int buf, int b0, int b1,
                             double v[4]) {
  const int off = R->off;
  const long long cap = A.cap;
  const double* X = A.X[buf];
  const float4* S = A.stage[buf];
  const double Limg = R->img ? R->boxl : 0.0;  // minimum images (energy.cpp:137-139)
  double eb = 0, ea = 0, eatt = 0;
  long long erep_fx = 0;  // list-ordered sum: exact in fixed point (2^-40 kcal/mol)
  for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const long long gi = off + i;
    const int4 tp = A.topo[gi];
    const int nat_cnt = tp.w & 0xFFFF, bnd_cnt = (tp.w >> 16) & 0xFF, ang_cnt = (tp.w >> 24) & 0xFF;
    const int ti = (int)f2u(S[2 * gi].w);
    if (R->terms & SOP_TERM_FENE)
      for (int k = 0; k < bnd_cnt; k++) {
        const int j = A.bnd[tp.y + k].x;
        if (j <= i || !SOP_GATHER_OK(A, j, R->n)) continue;
        const double d = sqrt(exact_d2i(X, cap, gi, off + j, Limg));
        const double dev = d - A.bnd_r0[tp.y + k];
        eb += log1p(-dev * dev / R->R0sq_d);
      }
    if (R->terms & SOP_TERM_ANGLE)
      for (int k = 0; k < ang_cnt; k++) {
        const int j = A.ang[tp.z + k];
        if (j <= i || !SOP_GATHER_OK(A, j, R->n)) continue;
        const double d2 = exact_d2i(X, cap, gi, off + j, Limg);
        ea += R->e_ang_coeff / (d2 * d2 * d2);
      }
    if (R->terms & SOP_TERM_VDW) {
      for (int k = 0; k < nat_cnt; k++) {
        const int4 e = A.nat[tp.x + k];
        const int j = e.x & (int)kIdx;
        if (j <= i || !(e.x & (int)kPL) || !SOP_GATHER_OK(A, j, R->n)) continue;
        const int tj = (int)f2u(S[2 * (off + (long long)j)].w);
        const double r0 = A.nat_r0[tp.x + k];
        const double r2 = r0 * r0, r6 = r2 * r2 * r2, r12 = r6 * r6;
        const double d2 = exact_d2i(X, cap, gi, off + j, Limg);
        const double d6 = d2 * d2 * d2, d12 = d6 * d6;
        eatt += c_ff.coeff_att[ti][tj] * (r12 / d12) - 2.0 * (r6 / d6);  // energy.cpp:224
      }
      const int cnt = A.nl_cnt[gi];
      const long long row = R->nl_base + (long long)i * R->L;
      for (int k = 0; k < cnt; k++) {
        const int e = A.nl[row + k];
        const int j = e & (int)kIdx;
        if (j <= i || !(e & (int)kPL) || !SOP_GATHER_OK(A, j, R->n)) continue;
        const int tj = (int)f2u(S[2 * (off + (long long)j)].w);
        const double d2 = exact_d2i(X, cap, gi, off + j, Limg);
        const double d6 = d2 * d2 * d2, d12 = d6 * d6;
        const double ep = c_ff.coeff_rep[ti][tj] * (c_ff.sigma_rep12[ti][tj] / d12 + c_ff.sigma_rep6[ti][tj] / d6);
        erep_fx += __double2ll_rn(ep * 1099511627776.0);  // 2^40
      }
    }
  }
  v[0] = eb;
  v[1] = ea;
  v[2] = eatt;
  v[3] = (double)erep_fx * 9.094947017729282e-13;  // 2^-40
}

// The replica's energy terms from the summed v of energy_terms.
__device__ void energy_finish(RepDev* R, const double v[4]) {
  R->energy[0] = -R->e_bnd_coeff * v[0];
  R->energy[1] = v[1];
  R->energy[3] = v[2];
  R->energy[4] = v[3];
  R->energy[2] = v[2] + v[3];
  R->energy[5] = R->energy[0] + R->energy[1] + R->energy[2];
}

// Energy terms of one replica on one CTA (output steps, list-build closes).
__device__ void replica_energy(const DevArrays& A, RepDev* R, int buf, double* red) {
  double v[4];
  energy_terms(A, R, buf, 0, R->n, v);
  block_sum(v, 4, red);
  if (threadIdx.x == 0) energy_finish(R, v);
}

// K6: observables (sop.cpp:200-279) at positions X[buf] and the stored velocities.
__device__ void replica_obs(const DevArrays& A, RepDev* R, int buf, double* red) {
  const int n = R->n, off = R->off;
  const long long cap = A.cap;
  const double* X = A.X[buf];
  double s[4] = {0, 0, 0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long gi = off + i;
    s[0] += X[gi]; s[1] += X[cap + gi]; s[2] += X[2 * cap + gi];
  }
  block_sum(s, 3, red);
  const double mx = s[0] / n, my = s[1] / n, mz = s[2] / n;
  const double Limg = R->img ? R->boxl : 0.0;
  double q[4] = {0, 0, 0, 0};  // contacts, natives, sum |r - mean|^2, sum v^2
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long gi = off + i;
    if (R->img) {
      // with images the centroid identity does not hold: the pair sum of
      // sop.cpp:237-249 itself
      for (int j = i + 1; j < n; j++) q[2] += exact_d2i(X, cap, gi, off + j, Limg);
    } else {
      const double ax = X[gi] - mx, ay = X[cap + gi] - my, az = X[2 * cap + gi] - mz;
      q[2] += ax * ax + ay * ay + az * az;
    }
    const double vx = A.vel[gi], vy = A.vel[cap + gi], vz = A.vel[2 * cap + gi];
    q[3] += vx * vx + vy * vy + vz * vz;
    const int4 tp = A.topo[gi];
    const int nat_cnt = tp.w & 0xFFFF;
    for (int k = 0; k < nat_cnt; k++) {
      const int j = A.nat[tp.x + k].x & (int)kIdx;
      if (j <= i || !SOP_GATHER_OK(A, j, n)) continue;
      const float r_ij = (float)A.nat_r0[tp.x + k];  // sop.cpp:213 reads r0 into a float
      const double d = sqrt(exact_d2i(X, cap, off + j, gi, Limg));
      q[1] += 1.0;
      if (d / (double)r_ij < 1.25) q[0] += 1.0;
    }
  }
  block_sum(q, 4, red);
  if (threadIdx.x == 0) {
    R->obs[1] = q[0];
    R->obs[0] = q[1] > 0 ? q[0] / q[1] : 0.0;
    // sum_{i<j} d^2 / N^2, without images = sum |r - mean|^2 / N
    R->obs[2] = R->img ? q[2] / ((double)n * (double)n) : q[2] / n;
    // kinT (sop.cpp:262-279): overdamped from the last increments, kept in vel
    R->obs[3] = (R->dyn == SOP_DYN_OVERDAMPED ? q[3] * R->zeta_2h : q[3]) / (3.0 * n);
    R->obs[4] = sqrt(exact_d2i(X, cap, (long long)off, (long long)off + n - 1, Limg));
  }
}

// Energy terms of replicas rep_ids[0..nrep) on many CTAs: CTA (x, y) sums
// slice x (kEnergySlice beads) of replica rep_ids[y] into en_part[slice_base[y]
// + x]; the CTA that finishes the replica's last slice adds the slices' sums
// in slice order (deterministic) and stores the terms.
__global__ void __launch_bounds__(256) k_energy(DevArrays A, const int* rep_ids,
                                                const int* slice_base, int nrep) {
  __shared__ double red[4 * 256];
  __shared__ int s_last;
  const int y = blockIdx.y;
  RepDev* R = &A.rep[rep_ids[y]];
  const int n = R->n;
  const int nsl = (n + kEnergySlice - 1) / kEnergySlice;
  const int x = blockIdx.x;
  if (x >= nsl) return;  // the whole CTA: before any barrier
  double v[4];
  energy_terms(A, R, R->cur, x * kEnergySlice, min(n, (x + 1) * kEnergySlice), v);
  block_sum(v, 4, red);
  if (threadIdx.x == 0) {
    double* p = A.en_part + 4LL * (slice_base[y] + x);
    for (int q = 0; q < 4; q++) p[q] = v[q];
    __threadfence();
    s_last = atomicAdd(A.en_done + y, 1) == nsl - 1;
    if (s_last) {
      __threadfence();
      double t[4] = {0, 0, 0, 0};
      const volatile double* b = A.en_part + 4LL * slice_base[y];
      for (int k = 0; k < nsl; k++)
        for (int q = 0; q < 4; q++) t[q] += b[4 * k + q];
      energy_finish(R, t);
      A.en_done[y] = 0;
    }
  }
}

__global__ void __launch_bounds__(256) k_obs(DevArrays A, const int* rep_ids, int nrep) {
  __shared__ double red[4 * 256];
  RepDev* R = &A.rep[rep_ids[blockIdx.x]];
  replica_obs(A, R, R->cur, red);
  if (threadIdx.x == 0) R->obs_pending = 0;
}

// ---------------------------------------------------------------------------------
// update_pair_list (sop.cpp:473-553) at the current positions

__global__ void k_pairlist(DevArrays A, int r, int off, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  RepDev* R = &A.rep[r];
  if (R->mode == SOP_LIST_NONE) return;
  const long long gi = off + i, cap = A.cap;
  const double* X = A.X[R->cur];
  const float4* S = A.stage[R->cur] + 2 * (long long)off;
  const float4 hi = S[2 * i], lo = S[2 * i + 1];
  const int ti = (int)f2u(hi.w);
  const int4 tp = A.topo[gi];
  const BeadRef b{hi, lo, i, ti, gi};
  const BoxF box{R->Lh, R->Ll, R->invL};
  const double Limg = R->img ? R->boxl : 0.0;
  auto diff = [&](const float4& hj, const float4& lj, float& dx, float& dy, float& dz) {
    if (R->img) pair_delta<true>(b, hj, lj, box, dx, dy, dz);
    else pair_delta<false>(b, hj, lj, box, dx, dy, dz);
  };
  const int nat_cnt = tp.w & 0xFFFF;
  for (int k = 0; k < nat_cnt; k++) {
    const int4 e = A.nat[tp.x + k];
    const int j = e.x & (int)kIdx;
    if (!SOP_GATHER_OK(A, j, n)) continue;
    const float4 hj = S[2 * j], lj = S[2 * j + 1];
    float dx, dy, dz;
    diff(hj, lj, dx, dy, dz);
    const float d2 = dx * dx + dy * dy + dz * dz;
    bool plb = false;
    if (e.x & (int)kNL) {
      const double rc = 2.5 * A.nat_r0[tp.x + k], rc2 = rc * rc;
      plb = within(d2, (float)rc2, kScreenMargin, [&] { return exact_d2i(X, cap, gi, off + j, Limg) < rc2; });
    }
    A.nat[tp.x + k].x = (e.x & ~(int)kPL) | (plb ? (int)kPL : 0);
  }
  const int cnt = A.nl_cnt[gi];
  const long long row = R->nl_base + (long long)i * R->L;
  for (int k = 0; k < cnt; k++) {
    const int e = A.nl[row + k];
    const int j = e & (int)kIdx;
    if (!SOP_GATHER_OK(A, j, n)) continue;
    const float4 hj = S[2 * j], lj = S[2 * j + 1];
    float dx, dy, dz;
    diff(hj, lj, dx, dy, dz);
    const float d2 = dx * dx + dy * dy + dz * dz;
    const int tj = (int)f2u(hj.w);
    const double rc2 = c_ff.rc2_pl[ti][tj];
    const bool plb = within(d2, c_ff.rc2_pl_f[ti][tj], kScreenMargin,
                            [&] { return exact_d2i(X, cap, gi, off + j, Limg) < rc2; });
    A.nl[row + k] = (e & ~(int)kPL) | (plb ? (int)kPL : 0);
  }
}

// Packed host-order state (x y z per bead, replicas back to back at 3*poff[k])
// into replica k's device arrays: both position buffers, the staged float
// pairs, velocities, zero increments.  One CTA per replica.
__global__ void k_scatter_state(DevArrays A, const int* ids, const long long* poff,
                                const double* xyz, const double* vel) {
  const RepDev* R = &A.rep[ids[blockIdx.x]];
  const long long off = R->off, cap = A.cap, base = 3 * poff[blockIdx.x];
  for (int i = threadIdx.x; i < R->n; i += blockDim.x) {
    const long long g = off + i;
    float h[3], l[3];
    for (int c = 0; c < 3; c++) {
      const double x = xyz[base + 3 * i + c];
      A.X[0][c * cap + g] = x;
      A.X[1][c * cap + g] = x;
      split_double(x, h[c], l[c]);
      A.vel[c * cap + g] = vel ? vel[base + 3 * i + c] : 0.0;
      A.incr[c * cap + g] = 0.0f;
    }
    const float4 oh = A.stage[0][2 * g], ol = A.stage[0][2 * g + 1];  // keep type / chain
    const float4 nh = make_float4(h[0], h[1], h[2], oh.w), nl = make_float4(l[0], l[1], l[2], ol.w);
    A.stage[0][2 * g] = nh;
    A.stage[1][2 * g] = nh;
    A.stage[0][2 * g + 1] = nl;
    A.stage[1][2 * g + 1] = nl;
  }
}

// The reverse: current positions and velocities into the packed layout.
__global__ void k_gather_state(DevArrays A, const int* ids, const long long* poff, double* xyz,
                               double* vel) {
  const RepDev* R = &A.rep[ids[blockIdx.x]];
  const long long off = R->off, cap = A.cap, base = 3 * poff[blockIdx.x];
  const double* X = A.X[R->cur];
  for (int i = threadIdx.x; i < R->n; i += blockDim.x)
    for (int c = 0; c < 3; c++) {
      if (xyz) xyz[base + 3 * i + c] = X[c * cap + off + i];
      if (vel) vel[base + 3 * i + c] = A.vel[c * cap + off + i];
    }
}

cudaError_t launch_scatter_state(const DevArrays& A, const int* ids, int nrep, const long long* poff,
                                 const double* xyz, const double* vel, cudaStream_t s) {
  if (nrep <= 0) return cudaSuccess;
  k_scatter_state<<<nrep, 256, 0, s>>>(A, ids, poff, xyz, vel);
  return cudaGetLastError();
}

cudaError_t launch_gather_state(const DevArrays& A, const int* ids, int nrep, const long long* poff,
                                double* xyz, double* vel, cudaStream_t s) {
  if (nrep <= 0) return cudaSuccess;
  k_gather_state<<<nrep, 256, 0, s>>>(A, ids, poff, xyz, vel);
  return cudaGetLastError();
}

// which: 0 neighbor att, 1 neighbor rep, 2 pair att, 3 pair rep
__global__ void k_export(DevArrays A, int r, int off, int n, int which, int capacity) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RepDev* R = &A.rep[r];
  const long long gi = off + i;
  const int4 tp = A.topo[gi];
  if (which == 0 || which == 2) {
    const int nat_cnt = tp.w & 0xFFFF;
    const unsigned bit = (which == 0) ? kNL : kPL;
    for (int k = 0; k < nat_cnt; k++) {
      const int e = A.nat[tp.x + k].x;
      const int j = e & (int)kIdx;
      if (j <= i || !((unsigned)e & bit)) continue;
      const int slot = atomicAdd(A.pairs_cnt, 1);
      if (slot < capacity) A.pairs_out[slot] = ((unsigned long long)(i + 1) << 32) | (unsigned)(j + 1);
    }
  } else {
    const int cnt = A.nl_cnt[gi];
    const long long row = R->nl_base + (long long)i * R->L;
    for (int k = 0; k < cnt; k++) {
      const int e = A.nl[row + k];
      const int j = e & (int)kIdx;
      if (j <= i) continue;
      if (which == 3 && !((unsigned)e & kPL)) continue;
      const int slot = atomicAdd(A.pairs_cnt, 1);
      if (slot < capacity) A.pairs_out[slot] = ((unsigned long long)(i + 1) << 32) | (unsigned)(j + 1);
    }
  }
}

// ---------------------------------------------------------------------------------
// launchers

using StepKernel = void (*)(DevArrays, const StepItem*, const int*, int, const int*);

// The step kernel for a strategy (0: CTA items with shared-memory staging,
// 1: warp tasks), lane count (1, 2, 4, 8, 16) and occupancy target (2, 3,
// or 4 for CTA items: 64 registers, and 4 CTAs fit an SM when the stage
// limit is at most ~1700 beads).
template <int G>
static StepKernel step_kernel_g(int strategy, int min_blocks) {
  const bool two = min_blocks == 2;
  if (strategy == 1) return two ? k_step_w<G, 2> : k_step_w<G, 3>;
  if (min_blocks == 4) return k_step<G, 4>;
  return two ? k_step<G, 2> : k_step<G, 3>;
}
// 512-thread CTAs: the register budget of min_blocks 256-thread CTAs per SM
// (4 -> two 512-thread CTAs at 64 registers, 2 or 3 -> one at up to 128)
template <int G>
static StepKernel step_kernel_wide(int min_blocks) {
  return min_blocks == 4 ? k_step<G, 2, 512> : k_step<G, 1, 512>;
}
bool step_shape_supported(int lanes, int strategy, int threads) {
  if (threads % 32 || threads < 64 || threads > 512) return false;
  if (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16) return false;
  if (threads > 256) return strategy == 0 && lanes <= 4;
  return true;
}
static StepKernel step_kernel(int lanes, int min_blocks, int strategy, int threads = 256) {
  if (threads > 256) {
    switch (lanes) {
      case 1: return step_kernel_wide<1>(min_blocks);
      case 2: return step_kernel_wide<2>(min_blocks);
      default: return step_kernel_wide<4>(min_blocks);
    }
  }
  switch (lanes) {
    case 1: return step_kernel_g<1>(strategy, min_blocks);
    case 2: return step_kernel_g<2>(strategy, min_blocks);
    case 8: return step_kernel_g<8>(strategy, min_blocks);
    case 16: return step_kernel_g<16>(strategy, min_blocks);
    default: return step_kernel_g<4>(strategy, min_blocks);
  }
}

static int g_prep_dyn = 48 * 1024;  // k_prep dynamic shared memory (set by init_kernels)

// Opt a kernel into up to `optin_bytes` of dynamic shared memory per block
// (less its static shared memory and the per-block reservation).
template <class K>
static cudaError_t optin(K kernel, int optin_bytes, int* dyn_out = nullptr) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  int dyn = optin_bytes - (int)fa.sharedSizeBytes - 1024;
  if (dyn_out) *dyn_out = dyn;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
}

cudaError_t init_kernels(int optin_bytes, int sm_bytes) {
  cudaError_t e;
  // the prologue kernels run two CTAs per SM: half the SM's shared memory each
  const int half = std::min(optin_bytes, sm_bytes / 2);
  if ((e = optin(k_prep, half, &g_prep_dyn)) != cudaSuccess) return e;
  for (int lanes : {1, 2, 4, 8, 16})
    for (int mb : {2, 3, 4}) {
      if ((e = optin(step_kernel(lanes, mb, 0), optin_bytes)) != cudaSuccess) return e;
      if (lanes <= 4 && (e = optin(step_kernel(lanes, mb, 0, 512), optin_bytes)) != cudaSuccess)
        return e;
    }
  return cudaSuccess;
}

cudaError_t launch_prologue(const DevArrays& A, const int* rep_ids, int nrep, const int* nrep_dev,
                            int force_build, int build_mode, int full, int grid, cudaStream_t s,
                            cudaEvent_t after_decide, cudaEvent_t after_bin) {
  if (nrep <= 0) return cudaSuccess;
  cudaError_t e;
  if (after_decide && (e = cudaEventRecord(after_decide, s)) != cudaSuccess) return e;
  if (grid <= 0) grid = 1;
  // cooperative: the consumers wait for every producer CTA, so all must be resident
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBuildThreads);
  cfg.dynamicSmemBytes = (size_t)g_prep_dyn;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if ((e = cudaLaunchKernelEx(&cfg, k_prep, A, rep_ids, nrep_dev, nrep, force_build, build_mode,
                              full, g_prep_dyn)) != cudaSuccess)
    return e;
  if (after_bin && (e = cudaEventRecord(after_bin, s)) != cudaSuccess) return e;
  return cudaSuccess;
}

cudaError_t launch_step(const DevArrays& A, const StepItem* items, int nitems, const int* nitems_dev,
                        const int* cta_first, int queue, int max_staged, int lanes, int min_blocks,
                        int strategy, int threads, int grid, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  const size_t dyn = strategy == 1 ? 0 : (size_t)max_staged * 32 + 128;
  if (grid <= 0) grid = nitems;
  if (!step_shape_supported(lanes, strategy, threads)) return cudaErrorInvalidConfiguration;
  DevArrays B = A;
  B.blk_dyn = (queue && strategy != 1) ? 1 : 0;
  step_kernel(lanes, min_blocks, strategy, threads)<<<grid, threads, dyn, s>>>(B, items, nitems_dev,
                                                                              nitems, cta_first);
  return cudaGetLastError();
}

int step_kernel_max_smem() { return kStageMax * 32 + 128; }

int step_blocks_per_sm(int lanes, int min_blocks, int strategy, int threads, int max_staged) {
  const size_t dyn = strategy == 1 ? 0 : (size_t)max_staged * 32 + 128;
  int n = 0;
  if (!step_shape_supported(lanes, strategy, threads)) return 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel(lanes, min_blocks, strategy, threads),
                                                    threads, dyn) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_step64(const DevArrays& A, const StepItem* items, int nitems, const int* nitems_dev,
                          int grid, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  if (grid <= 0) grid = nitems;
  k_step64<<<grid, 256, 0, s>>>(A, items, nitems_dev, nitems);
  return cudaGetLastError();
}

cudaError_t launch_energy(const DevArrays& A, const int* rep_ids, const int* slice_base, int nrep,
                          int max_slices, cudaStream_t s) {
  if (nrep <= 0 || max_slices <= 0) return cudaSuccess;
  // the batch on grid y, at most 65535 replicas per launch (the launches run
  // in stream order, so the per-replica slice counters are reused safely)
  for (int y0 = 0; y0 < nrep; y0 += 65535) {
    const int ny = nrep - y0 < 65535 ? nrep - y0 : 65535;
    k_energy<<<dim3(max_slices, ny), 256, 0, s>>>(A, rep_ids + y0, slice_base + y0, ny);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_observables(const DevArrays& A, const int* rep_ids, int nrep, cudaStream_t s) {
  if (nrep <= 0) return cudaSuccess;
  k_obs<<<nrep, 256, 0, s>>>(A, rep_ids, nrep);
  return cudaGetLastError();
}

cudaError_t launch_pairlist(const DevArrays& A, int r, int off, int n, cudaStream_t s) {
  k_pairlist<<<(n + 127) / 128, 128, 0, s>>>(A, r, off, n);
  return cudaGetLastError();
}

cudaError_t launch_export(const DevArrays& A, int r, int off, int n, int which, int capacity,
                          cudaStream_t s) {
  k_export<<<(n + 127) / 128, 128, 0, s>>>(A, r, off, n, which, capacity);
  return cudaGetLastError();
}

}  // namespace sop
