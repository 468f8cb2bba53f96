// Continuous-batching server over the engine's C ABI.
//
// Requests (a system + a step count) queue in arrival order; each is prepared
// on the host at submission (topology, row sizing, device bytes), outside
// the server lock.  A pump is pipelined with the device:
//   1. it waits for the chunk the previous pump launched and retires, in one
//      batch, the requests whose run window closed in it: final energies,
//      observables and status are read, the replicas removed, memory freed;
//   2. it admits, in one batch, queued requests in order while a slot is
//      free and their device bytes fit the memory budget and the engine's
//      arenas (head of line waits): one list build, run windows opened;
//   3. it launches the next chunk of graph-captured batched steps for every
//      running request and returns while the device runs it.
// The caller's submissions between pumps therefore overlap device work, and
// requests that arrive while others run join at the next pump.  State stays
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

struct Request {
  int64_t id = 0;
  sop_prepared* prep = nullptr;  // released once admitted
  int64_t nsteps = 0;
  int64_t bytes = 0;
  int64_t nbead = 0;
  double submit_s = 0, start_s = 0;
  int replica = -1;

  ~Request() { sop_prepared_free(prep); }
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
  bool chunk_open = false;
  std::vector<int> finished, ids;
  std::vector<double> energy, obs;
  std::vector<int> status;
  std::vector<sop_prepared*> batch;
  std::vector<int64_t> batch_steps;
  double t_admit = 0, t_run = 0, t_retire = 0;  // seconds spent in each pump phase

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
  const int R = s->cfg.engine.max_replicas;
  s->finished.resize(R);
  s->ids.resize(R);
  s->energy.resize(6 * (size_t)R);
  s->obs.resize(5 * (size_t)R);
  s->status.resize(R);
  s->t0 = std::chrono::steady_clock::now();
  *out = s.release();
  return SOP_OK;
}

extern "C" int sop_server_destroy(sop_server* s) {
  if (!s) return SOP_ERR_ARG;
  if (s->eng) {
    int nf = 0;
    if (s->chunk_open) sop_run_chunk_end(s->eng, s->finished.data(), (int)s->finished.size(), &nf);
    sop_engine_destroy(s->eng);
  }
  delete s;
  return SOP_OK;
}

extern "C" int sop_server_submit(sop_server* s, const sop_system_desc* d, int64_t nsteps,
                                 int64_t* request_id) {
  if (!s || !d || nsteps < 1 || d->nbead < 1 || !d->xyz) return SOP_ERR_ARG;
  std::unique_ptr<Request> r(new Request());
  int rc = sop_prepare(d, &r->prep);  // host work, no lock held
  if (rc == SOP_OK) rc = sop_prepared_bytes(r->prep, &r->bytes);
  if (rc) return rc;
  r->nsteps = nsteps;
  r->nbead = d->nbead;
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  r->submit_s = s->now();
  if (request_id) *request_id = r->id;
  s->queue.push_back(std::move(r));
  return SOP_OK;
}

static sop_request_result result_of(const Request& r) {
  sop_request_result res{};
  res.request_id = r.id;
  res.nbead = r.nbead;
  res.steps = r.nsteps;
  res.submit_s = r.submit_s;
  res.start_s = r.start_s;
  return res;
}

static void fail(sop_server* s, Request& r, int status) {
  sop_request_result res = result_of(r);
  res.status = status;
  res.start_s = res.finish_s = s->now();
  s->done.push_back(res);
}

// Retire, in one batch, the requests whose replicas are listed.
static int retire(sop_server* s, const int* reps, int nf) {
  int n = 0;
  for (int k = 0; k < nf; k++)
    if (s->running.count(reps[k])) s->ids[n++] = reps[k];
  if (n == 0) return SOP_OK;
  const int rc = sop_replicas_retire(s->eng, s->ids.data(), n, s->energy.data(), s->obs.data(),
                                     s->status.data());
  const double t = s->now();
  for (int k = 0; k < n; k++) {
    auto it = s->running.find(s->ids[k]);
    Request& r = *it->second;
    sop_request_result res = result_of(r);
    res.status = rc;
    if (rc == SOP_OK) {
      res.replica_status = s->status[k];
      std::memcpy(res.energy, &s->energy[6 * k], sizeof res.energy);
      std::memcpy(res.observables, &s->obs[5 * k], sizeof res.observables);
    }
    res.finish_s = t;
    s->done.push_back(res);
    s->bead_steps += r.nbead * r.nsteps;
    s->mem_used -= r.bytes;
    s->running.erase(it);
  }
  return rc;
}

// Admit queued requests in order, in batches, until the head of the queue
// does not fit.  A batch the engine refuses for a reason other than room
// fails its head request, and admission goes on with the next.
static int admit(sop_server* s) {
  while (!s->queue.empty()) {
    s->batch.clear();
    s->batch_steps.clear();
    int64_t mem = s->mem_used;
    const int slots = s->cfg.max_active - (int)s->running.size();
    for (size_t k = 0; k < s->queue.size() && (int)s->batch.size() < slots; k++) {
      const Request& r = *s->queue[k];
      if (s->cfg.memory_budget > 0 && mem + r.bytes > s->cfg.memory_budget) break;
      mem += r.bytes;
      s->batch.push_back(r.prep);
      s->batch_steps.push_back(r.nsteps);
    }
    if (s->batch.empty()) return SOP_OK;
    int got = 0;
    const int rc = sop_replicas_admit(s->eng, s->batch.data(), s->batch_steps.data(),
                                      (int)s->batch.size(), s->ids.data(), &got);
    if (rc == SOP_ERR_FULL) return SOP_OK;  // wait for retirements to free the arenas
    if (rc) {
      fail(s, *s->queue.front(), rc);
      s->queue.pop_front();
      continue;
    }
    const double t = s->now();
    for (int k = 0; k < got; k++) {
      std::unique_ptr<Request> r = std::move(s->queue.front());
      s->queue.pop_front();
      sop_prepared_free(r->prep);
      r->prep = nullptr;
      r->replica = s->ids[k];
      r->start_s = t;
      s->mem_used += r->bytes;
      s->running[r->replica] = std::move(r);
    }
    if (got < (int)s->batch.size()) return SOP_OK;  // the engine is full
  }
  return SOP_OK;
}

extern "C" int sop_server_pump(sop_server* s, int* pending) {
  if (!s) return SOP_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  double tp = s->now();
  // 1. the chunk in flight ends; its finished requests retire
  if (s->chunk_open) {
    int nf = 0;
    s->chunk_open = false;
    int rc = sop_run_chunk_end(s->eng, s->finished.data(), (int)s->finished.size(), &nf);
    if (rc) return rc;
    double tq = s->now();
    s->t_run += tq - tp;
    rc = retire(s, s->finished.data(), nf);
    tp = s->now();
    s->t_retire += tp - tq;
    if (rc) return rc;
  }
  // 2. admission, in arrival order
  int rc = admit(s);
  double tq = s->now();
  s->t_admit += tq - tp;
  if (rc) return rc;
  // 3. the next chunk for everything in flight, left running
  if (!s->running.empty()) {
    rc = sop_run_chunk_begin(s->eng, s->cfg.chunk_steps);
    if (rc) return rc;
    s->chunk_open = true;
    s->t_run += s->now() - tq;
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

extern "C" int sop_server_timing(sop_server* s, double* admit_s, double* run_s, double* retire_s) {
  if (!s) return SOP_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (admit_s) *admit_s = s->t_admit;
  if (run_s) *run_s = s->t_run;
  if (retire_s) *retire_s = s->t_retire;
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

