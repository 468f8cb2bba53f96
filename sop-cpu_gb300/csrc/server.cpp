// Continuous-batching server over the engine's C ABI.
//
// Requests (a system + a step count) queue in arrival order.  Each pump:
//   1. admits queued requests while a slot is free and their device bytes fit
//      the memory budget and the engine's arenas (head of line waits),
//   2. opens a run window per admitted request and advances every running
//      request by one chunk of graph-captured batched steps,
//   3. retires the requests whose window closed: final energies and
//      observables are read, the replica is removed, its memory freed.
// Requests that arrive while others run join at the next pump, so their work
// overlaps on the device with requests already in flight.  State stays
// resident on the GPU from admission to retirement.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "../../include/sop_gpu.h"

namespace {

// A system description that owns copies of its arrays.
struct OwnedDesc {
  std::vector<double> xyz, vel, r0, rn;
  std::vector<int> type, chain, ib, jb, ia, ka, in, jn, ie, je;
  sop_system_desc d{};

  template <class T>
  static void copy(std::vector<T>& v, const T* p, long long n) {
    if (p && n > 0) v.assign(p, p + n);
    else v.clear();
  }
  template <class T>
  static const T* ptr(const std::vector<T>& v) {
    return v.empty() ? nullptr : v.data();
  }

  void assign(const sop_system_desc& s) {
    const long long n = s.nbead;
    copy(xyz, s.xyz, 3 * n);
    copy(vel, s.vel, 3 * n);
    copy(type, s.bead_type, n);
    copy(chain, s.chain, n);
    copy(ib, s.ib, s.nbnd);
    copy(jb, s.jb, s.nbnd);
    copy(r0, s.r0, s.nbnd);
    copy(ia, s.ia, s.nang);
    copy(ka, s.ka, s.nang);
    copy(in, s.in_, s.nnat);
    copy(jn, s.jn, s.nnat);
    copy(rn, s.rn, s.nnat);
    copy(ie, s.ie, s.nexcl);
    copy(je, s.je, s.nexcl);
    d = s;
    d.xyz = ptr(xyz);
    d.vel = ptr(vel);
    d.bead_type = ptr(type);
    d.chain = ptr(chain);
    d.ib = ptr(ib); d.jb = ptr(jb); d.r0 = ptr(r0);
    d.ia = ptr(ia); d.ka = ptr(ka);
    d.in_ = ptr(in); d.jn = ptr(jn); d.rn = ptr(rn);
    d.ie = ptr(ie); d.je = ptr(je);
  }
};

struct Request {
  int64_t id = 0;
  OwnedDesc desc;
  int64_t nsteps = 0;
  int64_t bytes = 0;
  double submit_s = 0, start_s = 0;
  int replica = -1;
};

}  // namespace

struct sop_server {
  sop_server_config cfg{};
  sop_engine* eng = nullptr;
  std::mutex mu;
  std::deque<std::unique_ptr<Request>> queue;
  std::unordered_map<int, std::unique_ptr<Request>> running;
  std::vector<sop_request_result> done;
  std::chrono::steady_clock::time_point t0;
  int64_t next_id = 1;
  int64_t bead_steps = 0;
  int64_t mem_used = 0;
  std::vector<int> finished;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

extern "C" int sop_server_create(const sop_server_config* cfg, sop_server** out) {
  if (!out) return SOP_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<sop_server> s(new sop_server());
  if (cfg) s->cfg = *cfg;
  else sop_engine_config_default(&s->cfg.engine);
  if (s->cfg.max_active <= 0) s->cfg.max_active = 1024;
  if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 200;
  if (s->cfg.engine.max_replicas <= 0 || s->cfg.engine.max_replicas < s->cfg.max_active)
    s->cfg.engine.max_replicas = s->cfg.max_active + 8;
  int rc = sop_engine_create(&s->cfg.engine, &s->eng);
  if (rc) return rc;
  s->finished.resize(s->cfg.engine.max_replicas);
  s->t0 = std::chrono::steady_clock::now();
  *out = s.release();
  return SOP_OK;
}

extern "C" int sop_server_destroy(sop_server* s) {
  if (!s) return SOP_ERR_ARG;
  if (s->eng) sop_engine_destroy(s->eng);
  delete s;
  return SOP_OK;
}

extern "C" int sop_server_submit(sop_server* s, const sop_system_desc* d, int64_t nsteps,
                                 int64_t* request_id) {
  if (!s || !d || nsteps < 1 || d->nbead < 1 || !d->xyz) return SOP_ERR_ARG;
  std::unique_ptr<Request> r(new Request());
  r->desc.assign(*d);
  r->nsteps = nsteps;
  std::lock_guard<std::mutex> lk(s->mu);
  int rc = sop_system_bytes(s->eng, &r->desc.d, &r->bytes);
  if (rc) return rc;
  r->id = s->next_id++;
  r->submit_s = s->now();
  if (request_id) *request_id = r->id;
  s->queue.push_back(std::move(r));
  return SOP_OK;
}

static void fail(sop_server* s, Request& r, int status) {
  sop_request_result res{};
  res.request_id = r.id;
  res.status = status;
  res.nbead = r.desc.d.nbead;
  res.steps = r.nsteps;
  res.submit_s = r.submit_s;
  res.start_s = res.finish_s = s->now();
  s->done.push_back(res);
}

extern "C" int sop_server_pump(sop_server* s, int* pending) {
  if (!s) return SOP_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  // 1. admission, in arrival order
  while (!s->queue.empty() && (int)s->running.size() < s->cfg.max_active) {
    Request& r = *s->queue.front();
    if (s->cfg.memory_budget > 0 && s->mem_used + r.bytes > s->cfg.memory_budget) break;
    int rep = -1;
    int rc = sop_replica_add(s->eng, &r.desc.d, &rep);
    if (rc == SOP_ERR_FULL) break;  // wait for retirements to free the arenas
    if (rc == SOP_OK) rc = sop_replica_start(s->eng, rep, r.nsteps);
    if (rc) {
      if (rep >= 0) sop_replica_remove(s->eng, rep);
      fail(s, r, rc);
      s->queue.pop_front();
      continue;
    }
    r.replica = rep;
    r.start_s = s->now();
    s->mem_used += r.bytes;
    s->running[rep] = std::move(s->queue.front());
    s->queue.pop_front();
  }
  // 2. one chunk for everything in flight
  if (!s->running.empty()) {
    int nf = 0;
    int rc = sop_run_chunk(s->eng, s->cfg.chunk_steps, s->finished.data(), (int)s->finished.size(), &nf);
    if (rc) return rc;
    // 3. retirement
    for (int k = 0; k < nf; k++) {
      const int rep = s->finished[k];
      auto it = s->running.find(rep);
      if (it == s->running.end()) continue;
      Request& r = *it->second;
      sop_request_result res{};
      res.request_id = r.id;
      res.nbead = r.desc.d.nbead;
      res.steps = r.nsteps;
      res.submit_s = r.submit_s;
      res.start_s = r.start_s;
      int64_t t = 0;
      res.status = sop_energy_eval(s->eng, rep, res.energy);
      if (res.status == SOP_OK) res.status = sop_observables(s->eng, rep, res.observables);
      if (res.status == SOP_OK) res.status = sop_replica_status(s->eng, rep, &res.replica_status, &t);
      res.finish_s = s->now();
      s->done.push_back(res);
      s->bead_steps += (int64_t)r.desc.d.nbead * r.nsteps;
      s->mem_used -= r.bytes;
      sop_replica_remove(s->eng, rep);
      s->running.erase(it);
    }
  }
  if (pending) *pending = (int)(s->queue.size() + s->running.size());
  return SOP_OK;
}

extern "C" int sop_server_poll(sop_server* s, sop_request_result* out, int cap, int* n) {
  if (!s || !n || (cap > 0 && !out)) return SOP_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  const int k = std::min(cap, (int)s->done.size());
  for (int i = 0; i < k; i++) out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + k);
  *n = k;
  return SOP_OK;
}

extern "C" int sop_server_clock(sop_server* s, double* now_s) {
  if (!s || !now_s) return SOP_ERR_ARG;
  *now_s = s->now();
  return SOP_OK;
}

extern "C" int sop_server_stats(sop_server* s, int64_t* bead_steps, int* active, int* queued) {
  if (!s) return SOP_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (bead_steps) *bead_steps = s->bead_steps;
  if (active) *active = (int)s->running.size();
  if (queued) *queued = (int)s->queue.size();
  return SOP_OK;
}

