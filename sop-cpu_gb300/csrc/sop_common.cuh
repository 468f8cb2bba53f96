// Shared definitions of the GB300 SOP engine: device data layout, the
// per-replica descriptor, constant force-field tables and small numerics
// helpers used by both host and device code.
//
// Data layout (all packed over replicas, bead g = replica.off + local i):
//   X[2]      double, SoA x|y|z blocks of `cap` each: unc_pos, double-buffered
//   stage[2]  float4 pairs per bead: {hi.xyz, type}, {lo.xyz, chain} with
//             hi = nearest float of X and lo = nearest float of X - hi, so
//             hi_j - hi_i + (lo_j - lo_i) is dx to ~1e-14 relative
//   incr      float, SoA: the position increment of the last step (internal)
//   vel       double, SoA: velocity (written at output / final steps)
//   xb        float4: positions at the last list build (displacement check)
//   topo      int4 per bead {nat_start, bond_start, angle_start, counts}
//   nl        int per neighbor-list entry, rows of L entries per bead:
//             local j in bits 0..29, bit 31 = in the pair list this step
//   nat       int2 per native entry {local j | bit30 NL | bit31 PL, r0^2 (f32)}
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define SOP_HD __host__ __device__ __forceinline__
#else
#define SOP_HD inline
#endif

namespace sop {

constexpr int kMaxTypes = 3;            // bead types 1 and 2 (index 0 unused)
constexpr unsigned kPL = 0x80000000u;   // entry bit: member of the pair list
constexpr unsigned kNL = 0x40000000u;   // native entry bit: member of the neighbor list
constexpr unsigned kIdx = 0x3FFFFFFFu;  // entry bits holding the local index
constexpr double kTol = 1.0e-7;         // vdw_forces skip tolerance (energy.cpp:268)
constexpr double kEpsT = 1.0e-5;        // "steepest descent" threshold (sop.cpp:286)
constexpr float kScreenMargin = 4e-6f;  // relative band re-decided in FP64

// Step phases of a replica (see the step-kernel comment in kernels.cu).
enum Phase : int { PH_SKIP = 0, PH_FIRST = 1, PH_NORMAL = 2, PH_FINAL = 3, PH_FORCE = 4 };

// Per-replica descriptor, device resident (one array over replicas).
struct RepDev {
  // layout
  int off, n;              // bead range
  long long nl_base;       // first neighbor-list entry of the replica
  int L;                   // neighbor-list row capacity
  int nat_base, bnd_base, ang_base, exc_base;  // entry bases
  long long cell_base;     // first cell of the replica's binning range
  int cell_cap;            // cells the binning may use
  // configuration
  int mode;                // SOP_LIST_*
  int type_mask;           // bit t set when bead type t occurs in the replica
  int terms;               // SOP_TERM_* mask
  int prec;                // SOP_PREC_*
  int nnlup, nup;
  float rl_fac;            // list cutoff factor for non-natives (3.2, or (2.5 sigma+skin)/sigma computed per type)
  float skin;              // SKIN mode skin, A
  float cell_edge;         // grid edge for the list build (0 = auto)
  float half_skin2;        // (skin/2)^2
  double boxl, lcell, ncell;
  float Lh, Ll, invL;      // boxl as a two-float (Lh + Ll) and 1/boxl, for images in FP32
  int img;                 // minimum images apply (set at each list build, always in
                           // mode NONE): extent + 2 list cutoffs reached boxl/2
  float a1, a2, a3, a4;    // FP32 integrator constants
  double a1d, a2d, a3d, a4d;
  float noise_amp;         // sqrt(2 T zeta / h)
  double noise_amp_d, pull_fd;  // the same and the pulling force in FP64
  float T;
  float kbnd, R0sq, inv_R0sq;  // FENE
  float fang;              // 6 eps sigma_ss^6 (soft-sphere force coefficient)
  double kbnd_d, R0sq_d, fang_d, e_bnd_coeff, e_ang_coeff;
  float pull_f;            // pulling force magnitude, kcal/mol/A
  int dyn;                 // SOP_DYN_*
  float a5;                // overdamped step factor h/zeta
  double a5d, zeta_2h;     // the same in FP64; zeta/(2h) for the overdamped kinT
  int pull_i, pull_j;      // local indices of the pulled beads
  unsigned seed_lo, seed_hi;
  // run state (advanced by the prologue kernel)
  long long t;             // reference iteration index of the next force eval
  long long t_end;         // iteration at which the current run stops
  long long t_cur;         // force-eval index of this step (noise counter)
  int phase;               // Phase of this step
  int first_pending;       // next step restarts from stored velocities
  int moved;               // the last step advanced positions
  int cur;                 // position buffer holding X_t for this step
  int inlup;               // reference cadence counter (sop.cpp:100,156-165)
  int rebuild;             // rebuild requested (SKIN displacement or host)
  int near;                // SKIN displacement past the grouping fraction of the trigger
  float dmax2;             // largest squared displacement of a bead since the last
                           // list build (3e38: unknown, rows are scanned whole)
  float band_w;            // width of the rows' far band (0: rows not banded), set at
                           // each binning
  int out;                 // this step is an output step
  int obs_pending;         // observables of the last output step still due
  int en_after;            // energies due after this step's list build
  int running;             // a run window is open
  int active;
  int status;              // SOP_ST_* bits
  int max_row;             // longest neighbor-list row at the last build
  int builds;              // list builds done
  // results
  double energy[6];        // e_bnd, e_ang_ss, e_vdw, e_att, e_rep, etot
  double obs[5];           // Q, contct_nat, rgsq, kinT, end-to-end
};

// Force-field tables (global.cpp:60-92), filled from the host.
struct FFTables {
  double coeff_att[kMaxTypes][kMaxTypes];
  double coeff_rep[kMaxTypes][kMaxTypes];
  double force_coeff_att[kMaxTypes][kMaxTypes];
  double force_coeff_rep[kMaxTypes][kMaxTypes];
  double sigma_rep[kMaxTypes][kMaxTypes];
  double sigma_rep2[kMaxTypes][kMaxTypes];
  double sigma_rep6[kMaxTypes][kMaxTypes];
  double sigma_rep12[kMaxTypes][kMaxTypes];
  double rcut_nat[kMaxTypes][kMaxTypes];
  float fca[kMaxTypes][kMaxTypes];   // force_coeff_att as float
  float fcr[kMaxTypes][kMaxTypes];   // force_coeff_rep as float
  float s2[kMaxTypes][kMaxTypes];    // sigma^2 as float
  double rc2_pl[kMaxTypes][kMaxTypes];   // (2.5 sigma)^2 in FP64, as sop.cpp:539-541
  float rc2_pl_f[kMaxTypes][kMaxTypes];  // the same rounded to float, for the screen
  double rc2_nl[kMaxTypes][kMaxTypes];   // (3.2 sigma)^2 in FP64, as neighbor_list.cpp:97-100
};

// ---- Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -----------------------
SOP_HD void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
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

// ---- exact double <-> float conversions on the integer pipe --------------------
// GB300 runs FP64 arithmetic and f64<->f32 conversions at ~1.7 ops/clk/SM
// (measured), so the step kernel moves values between the two formats with
// integer bit operations instead.  Finite normal inputs only; magnitudes
// outside float range or below 2^-100 are not produced by the engine (tiny
// values flush to zero, which is below every tolerance used).

SOP_HD uint64_t d2u(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u; __builtin_memcpy(&u, &d, 8); return u;
#endif
}
SOP_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d; __builtin_memcpy(&d, &u, 8); return d;
#endif
}
SOP_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(f);
#else
  uint32_t u; __builtin_memcpy(&u, &f, 4); return u;
#endif
}
SOP_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f; __builtin_memcpy(&f, &u, 4); return f;
#endif
}

// float -> double, exact (normal floats; zero and subnormals -> +-0).
SOP_HD double f2d_exact(float f) {
  uint32_t u = f2u(f);
  uint64_t sign = (uint64_t)(u >> 31) << 63;
  uint32_t e = (u >> 23) & 0xFF;
  if (e == 0) return u2d(sign);
  uint64_t m = (uint64_t)(u & 0x7FFFFF) << 29;
  return u2d(sign | ((uint64_t)(e + 896) << 52) | m);
}

// double -> (hi, lo) floats: hi = nearest float (ties to even), lo = nearest
// float of the remainder.  hi + lo carries 48 of the 53 significand bits.
SOP_HD void split_double(double d, float& hi, float& lo) {
  uint64_t u = d2u(d);
  uint32_t sign = (uint32_t)(u >> 63) << 31;
  int e = (int)((u >> 52) & 0x7FF);
  if (e < 1023 - 100 || e > 1023 + 120) {  // |d| < 2^-100 (or huge): flush
    hi = u2f(sign);
    lo = 0.0f;
    if (e > 1023 + 120) hi = u2f(sign | 0x7F800000u);
    return;
  }
  uint64_t m = u & 0xFFFFFFFFFFFFFull;            // 52 bits
  uint32_t top = (uint32_t)(m >> 29);             // 23 bits kept
  uint32_t rest = (uint32_t)(m & 0x1FFFFFFFu);    // 29 bits dropped
  uint32_t half = 0x10000000u;
  uint32_t hb = sign | ((uint32_t)(e - 896) << 23) | top;
  bool up = rest > half || (rest == half && (top & 1u));
  if (up) hb += 1u;                               // carries into the exponent correctly
  hi = u2f(hb);
  // remainder in units of 2^(e-1075): rest, minus 2^29 if rounded up
  int32_t r = up ? (int32_t)rest - (int32_t)0x20000000 : (int32_t)rest;
  if (r == 0) { lo = 0.0f; return; }
  float fr = (float)r;                            // |r| < 2^29: exact to 24 bits (rounded)
  // scale by 2^(e-1075): build the power of two directly (exponent >= -152)
  int pe = e - 1075 + 127;
  float scale;
  if (pe > 0) {
    scale = u2f((uint32_t)pe << 23);
  } else {
    scale = u2f((uint32_t)1 << 23) * u2f((uint32_t)(pe + 126) << 23);  // 2^-126 * 2^(pe-1)
  }
  lo = fr * scale;
  if (sign) lo = -lo;
}

// double -> float when the double is known to hold a float value exactly.
SOP_HD float d2f_exact(double d) {
  uint64_t u = d2u(d);
  uint32_t sign = (uint32_t)(u >> 63) << 31;
  int e = (int)((u >> 52) & 0x7FF);
  if (e < 1023 - 126) return u2f(sign);
  return u2f(sign | ((uint32_t)(e - 896) << 23) | (uint32_t)((u >> 29) & 0x7FFFFF));
}

// ---- force fixed point -----------------------------------------------------------
// Lane partial sums (FP32) become int64 = round(f * 2^36) (resolution 1.5e-11
// kcal/mol/A, range +-1.3e8 over 16 lanes) through two F2I.S32 conversions,
// so the cross-lane reduction is exact and order-free.  With t = f * 2^36,
// a = rint(t / 2^32) and r = t - a * 2^32 is exact (Sterbenz), |r| <= 2^31.
// |f| must stay below kFixMax; a lane whose sum of |contributions| exceeds it
// is flagged by the caller (so that int64 sums over up to 16 lanes cannot wrap).
constexpr float kFixMax = 4.0e6f;
SOP_HD long long fixed_from_float(float f) {
  const float t = f * 68719476736.0f;  // 2^36
#ifdef __CUDA_ARCH__
  const float a = rintf(t * 2.3283064365386963e-10f);  // 2^-32
  const float r = t - a * 4294967296.0f;
  return (long long)__float2int_rn(a) * 4294967296LL + (long long)__float2int_rn(r);
#else
  const float a = __builtin_rintf(t * 2.3283064365386963e-10f);
  const float r = t - a * 4294967296.0f;
  long long rr = (long long)__builtin_rintf(r);
  if (rr > 2147483647LL) rr = 2147483647LL;
  if (rr < -2147483647LL) rr = -2147483647LL;
  return (long long)a * 4294967296LL + rr;
#endif
}

SOP_HD float float_from_fixed(long long v) { return (float)v * 1.4551915228366852e-11f; }  // 2^-36

}  // namespace sop
