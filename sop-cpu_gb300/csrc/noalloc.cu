// Neighbor list of one system without any device allocation.
//
// For callers that cannot allocate device memory themselves: hosts whose
// device memory is owned by their own pool (a framework's caching allocator
// that holds the GPU's memory), deployments that forbid allocation after
// start-up, and latency-critical loops that cannot take the device-wide
// synchronization a cudaMalloc or cudaFree may cause.  They pass device
// pointers for every input and output; the binning scratch lives in one
// file-scope __device__ array of fixed size (SOP_NOALLOC_MAX_BEADS beads),
// which every GPU that loads this library holds until the process exits.
//
// The list is the engine's non-native neighbor list: pairs i<j on different
// chains or |i-j| > 2 apart, not native, with d^2 < (3.2 sigma_ij)^2 decided
// in FP64 in the same operation order as the engine's list build (open
// boundaries: no minimum image).  Candidates come from a cell grid over the
// system whose edge, and the FP32 pre-screen's margin, grow with the
// system's extent, since relative FP32 positions carry an error of a few
// units in the last place of the extent.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/sop_gpu.h"
#include "sop_common.cuh"

namespace {

constexpr int kMaxBeads = SOP_NOALLOC_MAX_BEADS;
constexpr int kMaxCellsNA = 32768;
constexpr int kBinThreads = 1024;

struct GridInfo {
  float ox, oy, oz, edge;
  float margin;  // relative margin of the FP32 pre-screen
  int nx, ny, nz, ok;
};

constexpr double kTwoM23 = 1.1920928955078125e-07;  // 2^-23
constexpr double kRcMin = 3.2 * 3.8;                 // smallest list cutoff (type 1-1)

// Scratch layout (bytes): P float4[kMaxBeads] | sorted int[kMaxBeads] |
// cell int[kMaxBeads] | cstart int[kMaxCellsNA + 1] | ccur int[kMaxCellsNA] | GridInfo
constexpr size_t kOffP = 0;
constexpr size_t kOffSorted = kOffP + sizeof(float4) * kMaxBeads;
constexpr size_t kOffCell = kOffSorted + sizeof(int) * kMaxBeads;
constexpr size_t kOffStart = kOffCell + sizeof(int) * kMaxBeads;
constexpr size_t kOffCur = kOffStart + sizeof(int) * (kMaxCellsNA + 1);
constexpr size_t kOffGrid = (kOffCur + sizeof(int) * kMaxCellsNA + 255) / 256 * 256;
constexpr size_t kScratchBytes = kOffGrid + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

__constant__ double c_sigma[3][3] = {{0, 0, 0}, {0, 3.8, 5.4}, {0, 5.4, 7.0}};  // global.cpp:76-78

struct Scratch {
  float4* P;
  int* sorted;
  int* cell;
  int* cstart;
  int* ccur;
  GridInfo* grid;
};

__device__ __forceinline__ Scratch scratch_at(unsigned char* base) {
  Scratch s;
  s.P = reinterpret_cast<float4*>(base + kOffP);
  s.sorted = reinterpret_cast<int*>(base + kOffSorted);
  s.cell = reinterpret_cast<int*>(base + kOffCell);
  s.cstart = reinterpret_cast<int*>(base + kOffStart);
  s.ccur = reinterpret_cast<int*>(base + kOffCur);
  s.grid = reinterpret_cast<GridInfo*>(base + kOffGrid);
  return s;
}

__device__ __forceinline__ int type_of(const int* type, int i) { return type ? type[i] : 1; }
__device__ __forceinline__ int chain_of(const int* chain, int i) { return chain ? chain[i] : 0; }

// One CTA: bounding box, cell grid, stable counting sort of the beads into cells.
// Rejected input (*count < 0, nothing else written): positions not finite or
// beyond 1e6 A in magnitude (-1), a bead type other than 1 or 2 (-2).
__global__ void __launch_bounds__(kBinThreads) k_na_bin(unsigned char* base, const double* xyz,
                                                       int n, const int* type, int* count) {
  Scratch S = scratch_at(base);
  __shared__ float red[6][kBinThreads / 32];
  __shared__ int s_tmask;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  if (tid == 0) s_tmask = 0;
  __syncthreads();
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  int tm = 0;
  for (int i = tid; i < n; i += blockDim.x) {
    for (int c = 0; c < 3; c++) {
      const float v = (float)xyz[3 * (long long)i + c];
      // a NaN never enters fminf/fmaxf: count it as out of range
      mn[c] = v == v ? fminf(mn[c], v) : -3.4e38f;
      mx[c] = v == v ? fmaxf(mx[c], v) : 3.4e38f;
    }
    const int t = type_of(type, i);
    tm |= (t == 1 || t == 2) ? (1 << t) : 1;  // bit 0: a bad type
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int c = 0; c < 3; c++) {
      mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
      mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
    }
    tm |= __shfl_xor_sync(0xffffffffu, tm, o);
  }
  if (lane == 0) {
    for (int c = 0; c < 3; c++) { red[c][warp] = mn[c]; red[3 + c][warp] = mx[c]; }
    atomicOr(&s_tmask, tm);
  }
  __syncthreads();
  if (tid == 0) {
    float m0[3] = {3.4e38f, 3.4e38f, 3.4e38f}, m1[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int w = 0; w < nw; w++)
      for (int c = 0; c < 3; c++) {
        m0[c] = fminf(m0[c], red[c][w]);
        m1[c] = fmaxf(m1[c], red[3 + c][w]);
      }
    double rmax = 0;
    for (int a = 1; a < 3; a++)
      for (int b = 1; b < 3; b++)
        if (((s_tmask >> a) & 1) && ((s_tmask >> b) & 1)) rmax = fmax(rmax, 3.2 * c_sigma[a][b]);
    GridInfo g;
    g.ok = 1;
    int reject = 0;
    double ext = 0.0;
    for (int c = 0; c < 3; c++) {
      if (!(isfinite(m0[c]) && isfinite(m1[c]) && m1[c] >= m0[c] && fabsf(m0[c]) < 1e6f &&
            fabsf(m1[c]) < 1e6f))
        reject = 1;
      else
        ext = fmax(ext, (double)m1[c] - (double)m0[c]);
    }
    if (!reject && (s_tmask & 1)) reject = 2;
    if (reject) g.ok = 0;
    // Relative positions P = float(x - origin) lie in [1, ext + 2) and carry
    // up to half an ulp of that, 2^-24 (ext + 2); a cell index P / edge adds
    // the same again.  perr bounds both with a factor two to spare.  Pairs
    // within the cutoff then land in adjacent cells when the edge exceeds the
    // cutoff by a few perr, and the FP32 pre-screen keeps every pair whose
    // FP32 d^2 is within its own error of the cutoff.
    const double perr = (ext + 2.0) * kTwoM23;
    g.edge = (float)(rmax * 1.0001 + 6.0 * perr + 1e-3);
    g.margin = (float)(1e-5 + 8.0 * perr / kRcMin);
    g.ox = m0[0] - 1.0f; g.oy = m0[1] - 1.0f; g.oz = m0[2] - 1.0f;
    for (;;) {
      g.nx = g.ok ? (int)((m1[0] - g.ox) / g.edge) + 1 : 1;
      g.ny = g.ok ? (int)((m1[1] - g.oy) / g.edge) + 1 : 1;
      g.nz = g.ok ? (int)((m1[2] - g.oz) / g.edge) + 1 : 1;
      if ((long long)g.nx * g.ny * g.nz <= kMaxCellsNA) break;
      g.edge *= 1.25f;
    }
    *S.grid = g;
    *count = -reject;  // every call starts from zero pairs, or reports the rejection
  }
  __syncthreads();
  const GridInfo g = *S.grid;
  if (!g.ok) return;
  const int ncell = g.nx * g.ny * g.nz;
  // every call reuses the scratch: counts start from zero
  for (int c = tid; c < ncell; c += blockDim.x) S.ccur[c] = 0;
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    float4 p;
    p.x = (float)(xyz[3 * (long long)i] - (double)g.ox);
    p.y = (float)(xyz[3 * (long long)i + 1] - (double)g.oy);
    p.z = (float)(xyz[3 * (long long)i + 2] - (double)g.oz);
    p.w = 0.f;
    S.P[i] = p;
    const int cx = min(max((int)(p.x / g.edge), 0), g.nx - 1);
    const int cy = min(max((int)(p.y / g.edge), 0), g.ny - 1);
    const int cz = min(max((int)(p.z / g.edge), 0), g.nz - 1);
    const int c = cx + g.nx * (cy + g.ny * cz);
    S.cell[i] = c;
    atomicAdd(&S.ccur[c], 1);
  }
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the counts
    int carry = 0;
    for (int b = 0; b < ncell; b += 32) {
      const int c = b + lane;
      const int v = c < ncell ? S.ccur[c] : 0;
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (c < ncell) S.cstart[c] = carry + x - v;
      carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) S.cstart[ncell] = carry;
  }
  __syncthreads();
  for (int c = tid; c < ncell; c += blockDim.x) S.ccur[c] = 0;
  __syncthreads();
  if (warp == 0) {  // stable scatter in bead order
    for (int b = 0; b < n; b += 32) {
      const int i = b + lane;
      const bool valid = i < n;
      const unsigned act = __ballot_sync(0xffffffffu, valid);
      const int c = valid ? S.cell[i] : -1;
      const unsigned m = valid ? __match_any_sync(act, c) : 0u;
      const int rank = __popc(m & ((1u << lane) - 1u));
      const int basec = valid ? S.ccur[c] : 0;
      __syncwarp();
      if (valid) S.sorted[S.cstart[c] + basec + rank] = i;
      if (valid && lane == __ffs(m) - 1) S.ccur[c] = basec + __popc(m);
      __syncwarp();
    }
  }
}

// One warp per bead i: candidates j > i from the 27 neighbouring cells.
__global__ void k_na_enum(unsigned char* base, const double* xyz, int n, const int* type,
                          const int* chain, const int* nat_ptr, const int* nat_idx, int* pairs,
                          int cap, int* count) {
  const Scratch S = scratch_at(base);
  const GridInfo g = *S.grid;
  if (!g.ok) return;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const float4 pi = S.P[i];
    const int c = S.cell[i];
    const int cx = c % g.nx, cy = (c / g.nx) % g.ny, cz = c / (g.nx * g.ny);
    const int ti = type_of(type, i), chi = chain_of(chain, i);
    const int n0 = nat_ptr ? nat_ptr[i] : 0, n1 = nat_ptr ? nat_ptr[i + 1] : 0;
    for (int k = 0; k < 27; k++) {
      const int xx = cx + k % 3 - 1, yy = cy + (k / 3) % 3 - 1, zz = cz + k / 9 - 1;
      if (xx < 0 || xx >= g.nx || yy < 0 || yy >= g.ny || zz < 0 || zz >= g.nz) continue;
      const int cc = xx + g.nx * (yy + g.ny * zz);
      const int e = S.cstart[cc + 1];
      for (int s = S.cstart[cc] + lane; s < e; s += 32) {
        const int j = S.sorted[s];
        if (j <= i) continue;
        if (chain_of(chain, j) == chi && j - i <= 2) continue;
        const float4 pj = S.P[j];
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float d2f = dx * dx + dy * dy + dz * dz;
        const int tj = type_of(type, j);
        const double rc = 3.2 * c_sigma[ti][tj];
        const double rc2 = rc * rc;
        if (d2f > (float)rc2 * (1.0f + g.margin)) continue;
        // the decision itself in FP64 with the reference's order, no FMA
        const double ex = __dsub_rn(xyz[3 * (long long)j], xyz[3 * (long long)i]);
        const double ey = __dsub_rn(xyz[3 * (long long)j + 1], xyz[3 * (long long)i + 1]);
        const double ez = __dsub_rn(xyz[3 * (long long)j + 2], xyz[3 * (long long)i + 2]);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
        if (!(d2 < rc2)) continue;
        bool native = false;
        int lo = n0, hi = n1;
        while (lo < hi) {  // natives of i are sorted by partner
          const int mid = (lo + hi) >> 1;
          const int v = nat_idx[mid];
          if (v == j) { native = true; break; }
          if (v < j) lo = mid + 1;
          else hi = mid;
        }
        if (native) continue;
        const int slot = atomicAdd(count, 1);
        if (slot < cap) {
          pairs[2 * slot] = i + 1;
          pairs[2 * slot + 1] = j + 1;
        }
      }
    }
  }
}

std::mutex g_mu;
void* g_scratch_ptr[64];
bool g_scratch_ready[64];

}  // namespace

extern "C" int sop_neighbor_list_noalloc(const double* xyz, int nbead, const int* bead_type,
                                         const int* chain, const int* nat_ptr, const int* nat_idx,
                                         int* pairs, int cap, int* count, void* stream) {
  if (!xyz || !pairs || !count || nbead < 1 || cap < 0 || (nat_ptr && !nat_idx)) return SOP_ERR_ARG;
  if (nbead > SOP_NOALLOC_MAX_BEADS) return SOP_ERR_UNSUPPORTED;  // scratch holds that many beads
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return SOP_ERR_NODEV;
  }
  void* base = nullptr;
  {
    // set-up once per device, with that device current: the array's address
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ready[dev]) {
      if (cudaGetSymbolAddress(&g_scratch_ptr[dev], g_noalloc_scratch) != cudaSuccess) {
        cudaGetLastError();
        return SOP_ERR_CUDA;
      }
      g_scratch_ready[dev] = true;
    }
    base = g_scratch_ptr[dev];
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(base);
  k_na_bin<<<1, kBinThreads, 0, s>>>(b, xyz, nbead, bead_type, count);
  if (cudaGetLastError() != cudaSuccess) return SOP_ERR_CUDA;
  const int warps_needed = nbead;
  const int blocks = (warps_needed * 32 + 255) / 256;
  k_na_enum<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(b, xyz, nbead, bead_type, chain, nat_ptr,
                                                    nat_idx, pairs, cap, count);
  if (cudaGetLastError() != cudaSuccess) return SOP_ERR_CUDA;
  return SOP_OK;
}
