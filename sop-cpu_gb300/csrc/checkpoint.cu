// Exact per-replica checkpoint / restore.
//
// The reference restarts from coordinate and velocity files plus the saved
// generator state (sop.cpp:132-140, restart / rgen_restart).  Here a snapshot
// holds everything the next step reads, so that a restored replica continues
// bit for bit: both position buffers (X_t and X_{t-1}: the pair-list bits of
// step t were filtered at X_{t-1}), the last increments, the velocities, the
// neighbor-list rows with their pair-list bits, the native-entry flags, the
// displacement references of the skin trigger and the run state (step and
// noise counters, nnlup cadence, phase flags).  The counter-based noise needs
// no generator state beyond the step counter.  Layout (little-endian host
// order): header | RepDev | X0 | X1 (3n doubles each, x block, y, z) | incr
// (3n floats) | vel (3n doubles) | xb (n float4) | row counts (n ints) | rows
// (n x L ints) | native flags (one int per native entry).
#include <cstring>
#include <vector>

#include "engine.h"

using namespace sop;

namespace {

constexpr char kMagic[8] = {'S', 'O', 'P', 'C', 'K', 'P', 'T', '1'};

struct Header {
  char magic[8];
  int version;
  int n;
  int L;
  int pad;
  long long nnat_e;
  long long bytes;
};

#define KC(call)                                  \
  do {                                            \
    cudaError_t err_ = (call);                    \
    if (err_ != cudaSuccess) return SOP_ERR_CUDA; \
  } while (0)

long long snapshot_bytes(int n, int L, long long nnat_e) {
  return (long long)sizeof(Header) + (long long)sizeof(RepDev) + 2LL * 3 * n * 8 + 3LL * n * 4 +
         3LL * n * 8 + (long long)n * 16 + (long long)n * 4 + (long long)n * L * 4 + nnat_e * 4;
}

bool live_replica(const sop_engine* e, int r) {
  return e && r >= 0 && r < (int)e->reps.size() && e->reps[r].live;
}

}  // namespace

extern "C" int sop_replica_checkpoint(sop_engine* e, int r, void* buf, int64_t cap, int64_t* size) {
  if (!live_replica(e, r) || !size) return SOP_ERR_ARG;
  const Replica& R = e->reps[r];
  const int n = R.n, L = R.L;
  const long long need = snapshot_bytes(n, L, R.nnat_e);
  *size = need;
  if (!buf) return SOP_OK;
  if (cap < need) return SOP_ERR_OVERFLOW;
  KC(cudaSetDevice(e->cfg.device));
  KC(cudaStreamSynchronize(e->stream));
  char* p = static_cast<char*>(buf);
  Header h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kMagic, 8);
  h.version = 1;
  h.n = n;
  h.L = L;
  h.nnat_e = R.nnat_e;
  h.bytes = need;
  std::memcpy(p, &h, sizeof h);
  p += sizeof h;
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  std::memcpy(p, &d, sizeof d);
  p += sizeof d;
  const long long off = R.off, cc = e->cap;
  auto d2h = [&](const void* src, size_t bytes) -> int {
    KC(cudaMemcpyAsync(p, src, bytes, cudaMemcpyDeviceToHost, e->stream));
    p += bytes;
    return SOP_OK;
  };
  for (int b = 0; b < 2; b++)
    for (int c = 0; c < 3; c++)
      if ((rc = d2h(e->A.X[b] + c * cc + off, n * sizeof(double)))) return rc;
  for (int c = 0; c < 3; c++)
    if ((rc = d2h(e->A.incr + c * cc + off, n * sizeof(float)))) return rc;
  for (int c = 0; c < 3; c++)
    if ((rc = d2h(e->A.vel + c * cc + off, n * sizeof(double)))) return rc;
  if ((rc = d2h(e->A.xb + off, n * sizeof(float4)))) return rc;
  if ((rc = d2h(e->A.nl_cnt + off, n * sizeof(int)))) return rc;
  if ((rc = d2h(e->A.nl + R.nl_base, (size_t)n * L * sizeof(int)))) return rc;
  // native flags: the .x word of each native entry (partner | NL | PL bits)
  std::vector<int4> nat((size_t)R.nnat_e);
  if (R.nnat_e)
    KC(cudaMemcpyAsync(nat.data(), e->A.nat + R.nat_base, nat.size() * sizeof(int4),
                       cudaMemcpyDeviceToHost, e->stream));
  KC(cudaStreamSynchronize(e->stream));
  for (size_t k = 0; k < nat.size(); k++) {
    std::memcpy(p, &nat[k].x, 4);
    p += 4;
  }
  return SOP_OK;
}

extern "C" int sop_replica_restore(sop_engine* e, int r, const void* buf, int64_t size) {
  if (!live_replica(e, r) || !buf || size < (int64_t)sizeof(Header)) return SOP_ERR_ARG;
  Replica& R = e->reps[r];
  const char* p = static_cast<const char*>(buf);
  Header h;
  std::memcpy(&h, p, sizeof h);
  p += sizeof h;
  if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != 1) return SOP_ERR_ARG;
  if (h.n != R.n || h.nnat_e != R.nnat_e) return SOP_ERR_ARG;  // another system
  if (h.bytes != size || size != snapshot_bytes(h.n, h.L, h.nnat_e)) return SOP_ERR_ARG;
  KC(cudaSetDevice(e->cfg.device));
  KC(cudaStreamSynchronize(e->stream));
  const int n = R.n;
  RepDev s;
  std::memcpy(&s, p, sizeof s);
  p += sizeof s;
  const double* X0 = reinterpret_cast<const double*>(p);
  const double* X1 = X0 + 3 * (size_t)n;
  const float* incr = reinterpret_cast<const float*>(X1 + 3 * (size_t)n);
  const double* vel = reinterpret_cast<const double*>(incr + 3 * (size_t)n);
  const float4* xb = reinterpret_cast<const float4*>(vel + 3 * (size_t)n);
  const int* cnt = reinterpret_cast<const int*>(xb + n);
  const int* rows = cnt + n;
  const int* natx = rows + (size_t)n * h.L;
  // positions of both buffers (and their staged float pairs)
  std::vector<double> aos(3 * (size_t)n);
  for (int b = 0; b < 2; b++) {
    const double* X = b ? X1 : X0;
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 3; c++) aos[3 * (size_t)i + c] = X[(size_t)c * n + i];
    int rc = upload_positions(e, r, aos.data(), 1 << b);
    if (rc) return rc;
  }
  const long long off = R.off, cc = e->cap;
  for (int c = 0; c < 3; c++) {
    KC(cudaMemcpyAsync(e->A.incr + c * cc + off, incr + (size_t)c * n, n * sizeof(float),
                       cudaMemcpyHostToDevice, e->stream));
    KC(cudaMemcpyAsync(e->A.vel + c * cc + off, vel + (size_t)c * n, n * sizeof(double),
                       cudaMemcpyHostToDevice, e->stream));
  }
  KC(cudaMemcpyAsync(e->A.xb + off, xb, n * sizeof(float4), cudaMemcpyHostToDevice, e->stream));
  // list rows, re-strided when this replica's row length differs
  std::vector<int> tr;
  const int* src = rows;
  if (h.L != R.L) {
    tr.assign((size_t)n * R.L, 0);
    for (int i = 0; i < n; i++) {
      if (cnt[i] > R.L) return SOP_ERR_OVERFLOW;
      std::memcpy(tr.data() + (size_t)i * R.L, rows + (size_t)i * h.L, cnt[i] * sizeof(int));
    }
    src = tr.data();
  }
  KC(cudaMemcpyAsync(e->A.nl + R.nl_base, src, (size_t)n * R.L * sizeof(int),
                     cudaMemcpyHostToDevice, e->stream));
  KC(cudaMemcpyAsync(e->A.nl_cnt + off, cnt, n * sizeof(int), cudaMemcpyHostToDevice, e->stream));
  if (R.nnat_e) {
    std::vector<int4> nat((size_t)R.nnat_e);
    KC(cudaMemcpyAsync(nat.data(), e->A.nat + R.nat_base, nat.size() * sizeof(int4),
                       cudaMemcpyDeviceToHost, e->stream));
    KC(cudaStreamSynchronize(e->stream));
    for (size_t k = 0; k < nat.size(); k++) {
      if ((natx[k] & (int)kIdx) != (nat[k].x & (int)kIdx)) return SOP_ERR_ARG;  // other natives
      nat[k].x = natx[k];
    }
    KC(cudaMemcpyAsync(e->A.nat + R.nat_base, nat.data(), nat.size() * sizeof(int4),
                       cudaMemcpyHostToDevice, e->stream));
  }
  // run state onto this replica's layout and configuration
  RepDev d;
  int rc = get_rep(e, r, &d);
  if (rc) return rc;
  d.t = s.t; d.t_end = s.t_end; d.t_cur = s.t_cur; d.phase = s.phase;
  d.first_pending = s.first_pending; d.moved = s.moved; d.cur = s.cur; d.inlup = s.inlup;
  d.rebuild = s.rebuild; d.near = s.near; d.out = s.out; d.obs_pending = s.obs_pending;
  // the snapshot's rows carry no near / far split: scan them whole until the
  // next build (same results, the far entries' pair-list bits are 0)
  d.dmax2 = 3.0e38f;
  d.en_after = s.en_after; d.running = s.running; d.status = s.status; d.max_row = s.max_row;
  d.builds = s.builds;
  std::memcpy(d.energy, s.energy, sizeof d.energy);
  std::memcpy(d.obs, s.obs, sizeof d.obs);
  rc = put_rep(e, r, d);
  if (rc) return rc;
  KC(cudaStreamSynchronize(e->stream));
  return SOP_OK;
}
