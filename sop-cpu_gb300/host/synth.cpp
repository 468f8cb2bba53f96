// Seeded synthetic SOP chains: the workload generator for tests and benches.
//
// A chain is a self-avoiding walk with 3.8 A bonds grown inside a sphere of
// the radius of a compact globule of that many beads, then compacted by steepest descent on bond
// springs (rest 3.8 A), an attractive confinement pull toward that radius and
// an excluded-volume floor (no attraction between beads).  Only + - * / and
// sqrt are used, and this file is compiled with -ffp-contract=off, so a seed
// gives the same coordinates on x86 and on Arm.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/sop_gpu.h"

namespace {

struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed ^ 0x5DEECE66DULL) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  void unit(double* v) {
    for (;;) {
      double x = 2.0 * uniform() - 1.0, y = 2.0 * uniform() - 1.0, z = 2.0 * uniform() - 1.0;
      double r2 = x * x + y * y + z * z;
      if (r2 > 0.01 && r2 <= 1.0) {
        double r = std::sqrt(r2);
        v[0] = x / r; v[1] = y / r; v[2] = z / r;
        return;
      }
    }
  }
};

// Uniform hash grid over 3-D points, for the self-avoidance and floor tests.
struct Grid {
  double cell;
  std::unordered_map<uint64_t, std::vector<int>> bins;
  explicit Grid(double c) : cell(c) {}
  static uint64_t key(long x, long y, long z) {
    return ((uint64_t)(x + (1L << 20)) << 42) ^ ((uint64_t)(y + (1L << 20)) << 21) ^
           (uint64_t)(z + (1L << 20));
  }
  void idx(const double* p, long* c) const {
    for (int k = 0; k < 3; k++) c[k] = (long)std::floor(p[k] / cell);
  }
  void insert(int i, const double* p) {
    long c[3];
    idx(p, c);
    bins[key(c[0], c[1], c[2])].push_back(i);
  }
  template <class F>
  void near(const double* p, F f) const {
    long c[3];
    idx(p, c);
    for (long dx = -1; dx <= 1; dx++)
      for (long dy = -1; dy <= 1; dy++)
        for (long dz = -1; dz <= 1; dz++) {
          auto it = bins.find(key(c[0] + dx, c[1] + dy, c[2] + dz));
          if (it == bins.end()) continue;
          for (int j : it->second) f(j);
        }
  }
};

// Radius of a compact globule at ~270 A^3 per bead (R = 4.0 N^(1/3)), which
// gives protein-like contact densities; cube root by Newton iteration.
double globule_radius(int n) {
  double x = n > 1 ? (double)n : 1.0;
  double c = x > 1 ? x / 3.0 + 1.0 : 1.0;
  for (int it = 0; it < 100; it++) c = c - (c * c * c - x) / (3.0 * c * c);
  return 4.0 * c;
}

void grow(SplitMix& rng, int n, double radius, const double* center, double* x, int offset,
          Grid& grid, double min_sep) {
  const double b = 3.8;
  double* p = x + 3 * offset;
  if (n <= 0) return;
  // first bead: random point inside half the sphere, clear of earlier beads;
  // where the region is already full, the most separated of many tries
  {
    double best[3] = {center[0], center[1], center[2]}, best_sep = -1.0;
    bool ok = false;
    for (int t = 0; t < 20000 && !ok; t++) {
      double v[3];
      rng.unit(v);
      double r = 0.5 * radius * rng.uniform();
      for (int k = 0; k < 3; k++) p[k] = center[k] + r * v[k];
      double sep2 = 1e30;
      grid.near(p, [&](int j) {
        double d2 = 0;
        for (int k = 0; k < 3; k++) { double u = x[3 * j + k] - p[k]; d2 += u * u; }
        if (d2 < sep2) sep2 = d2;
      });
      ok = sep2 >= min_sep * min_sep;
      if (!ok && sep2 > best_sep) { best_sep = sep2; std::memcpy(best, p, sizeof best); }
    }
    if (!ok) std::memcpy(p, best, sizeof best);
  }
  grid.insert(offset, p);
  for (int i = 1; i < n; i++) {
    const double* q = x + 3 * (offset + i - 1);
    double* c = x + 3 * (offset + i);
    double best[3] = {0, 0, 0}, best_sep = -1.0;
    for (int t = 0; t < 200; t++) {
      double v[3], y[3];
      rng.unit(v);
      for (int k = 0; k < 3; k++) y[k] = q[k] + b * v[k];
      double r2 = 0;
      for (int k = 0; k < 3; k++) { double d = y[k] - center[k]; r2 += d * d; }
      if (r2 > radius * radius) continue;
      double sep2 = 1e30;
      grid.near(y, [&](int j) {
        if (j == offset + i - 1) return;
        double d2 = 0;
        for (int k = 0; k < 3; k++) { double d = x[3 * j + k] - y[k]; d2 += d * d; }
        if (d2 < sep2) sep2 = d2;
      });
      if (sep2 >= min_sep * min_sep) { std::memcpy(best, y, sizeof best); best_sep = 1e30; break; }
      if (sep2 > best_sep) { best_sep = sep2; std::memcpy(best, y, sizeof best); }
    }
    if (best_sep < 0) {  // every trial left the sphere: step toward the center
      double d[3], r2 = 0;
      for (int k = 0; k < 3; k++) { d[k] = center[k] - q[k]; r2 += d[k] * d[k]; }
      double r = std::sqrt(r2 > 1e-12 ? r2 : 1e-12);
      for (int k = 0; k < 3; k++) best[k] = q[k] + b * d[k] / r;
    }
    std::memcpy(c, best, sizeof best);
    grid.insert(offset + i, c);
  }
}

// Steepest descent on bond springs + confinement pull + excluded-volume floor.
void compact(int ntot, const int* chain_start, int nchain, double radius, const double* center,
             int steps, double* x) {
  const double kb = 10.0, kc = 0.5, ke = 10.0, dev_floor = 4.6, b = 3.8;
  const double eta = 0.02, max_step = 0.25;
  std::vector<double> g(3 * (size_t)ntot);
  std::vector<int> chain(ntot), pos_in_chain(ntot);
  for (int c = 0; c < nchain; c++)
    for (int i = chain_start[c]; i < chain_start[c + 1]; i++) { chain[i] = c; pos_in_chain[i] = i - chain_start[c]; }
  std::vector<std::pair<int, int>> pairs;
  for (int step = 0; step < steps; step++) {
    if (step % 10 == 0) {
      pairs.clear();
      Grid grid(dev_floor + 1.5);
      for (int i = 0; i < ntot; i++) grid.insert(i, x + 3 * i);
      for (int i = 0; i < ntot; i++) {
        grid.near(x + 3 * i, [&](int j) {
          if (j <= i) return;
          if (chain[i] == chain[j] && j - i < 2) return;
          double d2 = 0;
          for (int k = 0; k < 3; k++) { double d = x[3 * j + k] - x[3 * i + k]; d2 += d * d; }
          double rc = dev_floor + 1.5;
          if (d2 < rc * rc) pairs.emplace_back(i, j);
        });
      }
    }
    std::fill(g.begin(), g.end(), 0.0);
    for (int i = 0; i + 1 < ntot; i++) {
      if (chain[i] != chain[i + 1]) continue;
      double d[3], r2 = 0;
      for (int k = 0; k < 3; k++) { d[k] = x[3 * (i + 1) + k] - x[3 * i + k]; r2 += d[k] * d[k]; }
      double r = std::sqrt(r2);
      double f = 2.0 * kb * (r - b) / r;
      for (int k = 0; k < 3; k++) { g[3 * i + k] -= f * d[k]; g[3 * (i + 1) + k] += f * d[k]; }
    }
    for (auto& pr : pairs) {
      int i = pr.first, j = pr.second;
      double d[3], r2 = 0;
      for (int k = 0; k < 3; k++) { d[k] = x[3 * j + k] - x[3 * i + k]; r2 += d[k] * d[k]; }
      if (r2 >= dev_floor * dev_floor) continue;
      double r = std::sqrt(r2 > 1e-12 ? r2 : 1e-12);
      double f = -2.0 * ke * (dev_floor - r) / r;
      for (int k = 0; k < 3; k++) { g[3 * i + k] -= f * d[k]; g[3 * j + k] += f * d[k]; }
    }
    for (int i = 0; i < ntot; i++) {
      double d[3], r2 = 0;
      for (int k = 0; k < 3; k++) { d[k] = x[3 * i + k] - center[k]; r2 += d[k] * d[k]; }
      double r = std::sqrt(r2);
      // pull every bead inward a little (attractive), stronger beyond the radius
      double f = 0.002 * kc + (r > radius ? 2.0 * kc * (r - radius) / (r > 1e-12 ? r : 1e-12) : 0.0);
      for (int k = 0; k < 3; k++) g[3 * i + k] += f * d[k];
    }
    for (int i = 0; i < ntot; i++) {
      double s2 = 0;
      for (int k = 0; k < 3; k++) s2 += g[3 * i + k] * g[3 * i + k];
      double s = eta * std::sqrt(s2);
      double scale = s > max_step ? max_step / s : 1.0;
      for (int k = 0; k < 3; k++) x[3 * i + k] -= eta * scale * g[3 * i + k];
    }
    (void)pos_in_chain;
  }
}

}  // namespace

extern "C" int sop_synth_chain(uint64_t seed, int nbead, int compact_steps, double* xyz) {
  if (nbead < 1 || !xyz) return SOP_ERR_ARG;
  SplitMix rng(seed);
  double radius = globule_radius(nbead) + 2.0;
  double center[3] = {0, 0, 0};
  Grid grid(5.0);
  grow(rng, nbead, radius, center, xyz, 0, grid, 4.6);
  int starts[2] = {0, nbead};
  compact(nbead, starts, 1, radius, center, compact_steps, xyz);
  return SOP_OK;
}

extern "C" int sop_synth_globule(uint64_t seed, int nchain, int chain_len, int compact_steps,
                                 double* xyz) {
  if (nchain < 1 || chain_len < 1 || !xyz) return SOP_ERR_ARG;
  SplitMix rng(seed);
  int n = nchain * chain_len;
  double radius = globule_radius(n) + 2.0;
  double center[3] = {0, 0, 0};
  // chains grown one after another into the same sphere, each a compact blob
  double rchain = globule_radius(chain_len) + 2.0;
  Grid grid(5.0);
  for (int c = 0; c < nchain; c++) {
    double cc[3];
    for (;;) {
      double v[3];
      rng.unit(v);
      double r = (radius - rchain > 0 ? radius - rchain : 0.0) * std::sqrt(rng.uniform());
      for (int k = 0; k < 3; k++) cc[k] = center[k] + r * v[k];
      break;
    }
    grow(rng, chain_len, rchain, cc, xyz, c * chain_len, grid, 4.6);
  }
  std::vector<int> starts(nchain + 1);
  for (int c = 0; c <= nchain; c++) starts[c] = c * chain_len;
  compact(n, starts.data(), nchain, radius, center, compact_steps, xyz);
  return SOP_OK;
}
