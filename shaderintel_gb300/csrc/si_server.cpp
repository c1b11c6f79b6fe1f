// si_server.cpp — the served form: a request loop over one world that keeps every scene resident
// in HBM, admits scenes by their memory footprint and runs step(dt, K) requests by continuous
// batching. Each round of the loop takes the head request of every scene that has one and runs
// a few substeps of all of them in one plan (one launch per phase for all scenes); requests that
// arrive meanwhile join at the next round. A request completes when the GPU has finished its last
// substep: a host callback on the stream stamps the time (latency = submit -> that moment).
// The world's lock serialises the rounds with API calls from other threads, so resident scenes
// can be edited (particles, materials, colliders) while the server runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "si_cuda.h"
#include "si_internal.h"
#include "si_runtime.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  si_mpm* h = nullptr;
  double dt = 0;
  int32_t K = 0;
  int32_t remaining = 0;   // substeps not yet enqueued
  int32_t ncol = -1;       // the request's collider table (rows below), or -1: keep the scene's
  std::vector<float> cols;
  Clock::time_point t_submit;
  bool done = false;
  int32_t status = SI_OK;
  double latency_ms = 0;
};

struct Completion {              // handed to the stream callback
  si_server* s;
  std::vector<Request*> reqs;
  int64_t particle_substeps;
  int64_t substeps;
};

}  // namespace

struct si_server {
  si_world* w = nullptr;
  int64_t budget = 0, resident = 0;   // resident: scene footprints + the scratch reserve
  int64_t reserve = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  uint64_t next_ticket = 1;
  std::unordered_map<uint64_t, Request*> reqs;
  std::map<si_mpm*, std::deque<Request*>> queues;   // per resident scene, FIFO
  std::map<si_mpm*, int64_t> footprint;
  int inflight = 0;
  // stats
  std::vector<double> lat;
  int64_t requests_done = 0, substeps_done = 0, particle_substeps = 0, ticks = 0;
  double busy_s = 0;
  Clock::time_point busy_since;
  int max_round = 4;   // substeps per round: arrivals wait at most this many substeps to join
};

static void CUDART_CB on_complete(void* p) {
  Completion* c = static_cast<Completion*>(p);
  si_server* s = c->s;
  const Clock::time_point now = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (Request* r : c->reqs) {
      r->latency_ms = std::chrono::duration<double, std::milli>(now - r->t_submit).count();
      r->done = true;
      s->lat.push_back(r->latency_ms);
      s->requests_done++;
    }
    s->substeps_done += c->substeps;
    s->particle_substeps += c->particle_substeps;
    if (--s->inflight == 0) s->busy_s += std::chrono::duration<double>(now - s->busy_since).count();
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();
  delete c;
}

static void fail_request(si_server* s, Request* r, int status) {
  r->status = status;
  r->done = true;
  (void)s;
}

static void server_loop(si_server* s) {
  si_world* w = s->w;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    std::vector<si_mpm*> act;
    for (auto& q : s->queues)
      if (!q.second.empty()) act.push_back(q.first);
    if (act.empty() || s->inflight >= 2) {
      if (s->stop && act.empty() && s->inflight == 0) break;
      s->cv_work.wait_for(lk, std::chrono::milliseconds(act.empty() ? 50 : 1));
      continue;
    }
    // one round: up to max_round substeps of every scene with a queued request
    int K = s->max_round;
    for (si_mpm* h : act) K = std::min(K, s->queues[h].front()->remaining);
    K = std::max(K, 1);
    std::vector<si_mpm*> run;
    std::vector<double> dts;
    std::vector<Request*> fin;     // the request that this round finishes, per scene (or null)
    std::vector<Request*> start;   // the request that this round starts, per scene (or null)
    auto* comp = new Completion{s, {}, 0, (int64_t)K};
    for (si_mpm* h : act) {
      Request* r = s->queues[h].front();
      start.push_back(r->remaining == r->K ? r : nullptr);
      if (r->remaining == r->K) h->frame_sub = 0;   // a request is one step(dt, K) call
      r->remaining -= K;
      fin.push_back(nullptr);
      if (r->remaining <= 0) {
        comp->reqs.push_back(r);
        fin.back() = r;
        s->queues[h].pop_front();
      }
      run.push_back(h);
      dts.push_back(r->dt);
    }
    lk.unlock();
    int err = SI_OK;
    {
      std::lock_guard<std::recursive_mutex> wg(w->api_mu);
      {
        // drop scenes retired since they were picked (retire destroys them only under api_mu);
        // a request they would have finished ends as destroyed
        std::lock_guard<std::mutex> g(s->mu);
        size_t k = 0;
        for (size_t i = 0; i < run.size(); i++) {
          if (s->footprint.count(run[i])) {
            run[k] = run[i]; dts[k] = dts[i]; start[k] = start[i]; k++;
          } else if (fin[i]) {
            fin[i]->status = SI_EDESTROYED;
          }
        }
        run.resize(k);
        dts.resize(k);
        start.resize(k);
      }
      // a request that starts now brings the collider table that step() would upload (mpm.js:586)
      for (size_t i = 0; i < run.size(); i++) {
        const Request* r = start[i];
        if (!r || r->ncol < 0) continue;
        std::memset(run[i]->cols, 0, sizeof(run[i]->cols));
        if (r->ncol) std::memcpy(run[i]->cols, r->cols.data(), sizeof(float) * 12 * (size_t)r->ncol);
        run[i]->ncol = r->ncol;
        run[i]->prm_dirty = true;
      }
      for (si_mpm* h : run) comp->particle_substeps += h->count * (int64_t)K;
      // requests carry their own dt: retime before the round when it changes (mpm.js:140-145)
      for (size_t i = 0; i < run.size() && !err; i++)
        if (dts[i] > 0 && dts[i] != run[i]->dt) err = si_mpm_set_substep_dt(run[i], dts[i]);
      if (!err && !run.empty()) err = run_substeps(w, run, K);
      if (!err) {
        {
          std::lock_guard<std::mutex> g(s->mu);
          if (s->inflight++ == 0) s->busy_since = Clock::now();
          s->ticks += K;
        }
        if (cudaLaunchHostFunc(w->st, on_complete, comp) != cudaSuccess) {
          std::lock_guard<std::mutex> g(s->mu);
          if (--s->inflight == 0) s->busy_s += std::chrono::duration<double>(Clock::now() - s->busy_since).count();
          err = si_fail(SI_EDEVICE, "cudaLaunchHostFunc failed");
        }
      }
    }
    lk.lock();
    if (err) {
      for (Request* r : comp->reqs) fail_request(s, r, err);
      delete comp;
      s->cv_done.notify_all();
    }
  }
  lk.unlock();
  cudaStreamSynchronize(w->st);
}

static int run_on_world(si_server* s, void (*fn)(void*), void* ctx) {
  std::lock_guard<std::recursive_mutex> wg(s->w->api_mu);   // between two rounds
  fn(ctx);
  return SI_OK;
}

extern "C" {

int si_server_create(si_world* w, int64_t budget_bytes, si_server** out) {
  if (!w || !out) return si_fail(SI_EINVAL, "null argument");
  if (w->destroyed) return si_fail(SI_EDESTROYED, "the world was destroyed");
  if (w->server) return si_fail(SI_EBUSY, "the world already has a server");
  if (budget_bytes <= 0) return si_fail(SI_EINVAL, "budget must be positive");
  auto* s = new si_server();
  s->w = w;
  s->budget = budget_bytes;
  std::lock_guard<std::recursive_mutex> wg(w->api_mu);
  // Scenes admitted from now on keep one particle buffer (compact); their sort substeps use the
  // world's sort and pregather scratch, which grouping keeps below this reserve, taken from the budget.
  s->reserve = std::min<int64_t>(2ll << 30, budget_bytes / 32);
  s->resident = s->reserve;
  w->compact = true;
  w->group_particles = std::max<int64_t>(1, s->reserve / kGroupBytesPerParticle);
  for (si_mpm* h : w->scenes) {   // scenes already in the world become resident
    h->served = true;
    s->footprint[h] = h->device_bytes;
    s->resident += h->device_bytes;
    s->queues[h];
  }
  w->server = s;
  s->th = std::thread(server_loop, s);
  *out = s;
  return SI_OK;
}

int si_server_destroy(si_server* s) {
  if (!s) return si_fail(SI_EINVAL, "null server");
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (auto& q : s->queues) {   // queued requests that have not started are cancelled
      std::deque<Request*> keep;
      for (Request* r : q.second)
        if (r->remaining == r->K) fail_request(s, r, SI_EDESTROYED); else keep.push_back(r);
      q.second.swap(keep);
    }
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  if (s->th.joinable()) s->th.join();
  {
    std::lock_guard<std::recursive_mutex> wg(s->w->api_mu);
    for (si_mpm* h : s->w->scenes) h->served = false;
    s->w->server = nullptr;
    s->w->compact = false;
    s->w->group_particles = 0;
  }
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
  return SI_OK;
}

struct AdmitCtx { si_server* s; const si_mpm_desc* d; si_mpm* out; int rc; int64_t fp; };

int si_server_admit(si_server* s, const si_mpm_desc* desc, si_mpm** out) {
  if (!s || !out) return si_fail(SI_EINVAL, "null argument");
  *out = nullptr;
  const int64_t fp = scene_footprint_of(desc, true);
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->resident + fp > s->budget)
      return si_fail(SI_ENOMEM, "admission refused: scene footprint " + std::to_string(fp) + " B exceeds the free budget " +
                                    std::to_string(s->budget - s->resident) + " B");
    s->resident += fp;   // reserved now, so concurrent admissions cannot overshoot
  }
  AdmitCtx c{s, desc, nullptr, SI_OK, fp};
  run_on_world(s, [](void* p) {
    AdmitCtx* c = static_cast<AdmitCtx*>(p);
    c->rc = scene_create(c->s->w, c->d, &c->out, false);
    if (!c->rc) c->out->served = true;
  }, &c);
  std::lock_guard<std::mutex> g(s->mu);
  if (c.rc) { s->resident -= fp; return c.rc; }
  s->footprint[c.out] = fp;
  s->queues[c.out];
  *out = c.out;
  return SI_OK;
}

int si_server_retire(si_server* s, si_mpm* h) {
  if (!s || !h) return si_fail(SI_EINVAL, "null argument");
  {
    // The scene stops being resident first: a round that picked it before this point re-checks
    // residency under the world's lock, which the destruction below also takes.
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->queues.find(h);
    if (it == s->queues.end()) return si_fail(SI_EINVAL, "not a resident scene of this server");
    for (Request* r : it->second) fail_request(s, r, SI_EDESTROYED);   // none of these finished
    s->queues.erase(it);
    s->resident -= s->footprint[h];
    s->footprint.erase(h);
  }
  s->cv_done.notify_all();
  // substeps already enqueued are ordered before the stream-ordered release of the scene's memory
  run_on_world(s, [](void* p) {
    si_mpm* h = static_cast<si_mpm*>(p);
    h->served = false;
    si_mpm_destroy(h);
  }, h);
  return SI_OK;
}

int si_server_submit(si_server* s, si_mpm* h, double dt, int32_t K, uint64_t* ticket) {
  return si_server_submit_colliders(s, h, dt, K, nullptr, -1, ticket);
}

int si_server_submit_colliders(si_server* s, si_mpm* h, double dt, int32_t K, const float* rows, int32_t ncol,
                               uint64_t* ticket) {
  if (!s || !h || !ticket) return si_fail(SI_EINVAL, "null argument");
  if (K <= 0) return si_fail(SI_EINVAL, "K must be positive");
  if (ncol > 0 && !rows) return si_fail(SI_EINVAL, "MPM: bad collider table");
  std::vector<float> cols;
  if (ncol > 0) {
    ncol = std::min(ncol, (int32_t)SI_MAX_COLLIDERS);   // colliders.slice(0, 16), mpm.js:280
    cols.assign(rows, rows + 12 * (size_t)ncol);
  }
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return si_fail(SI_EDESTROYED, "the server was destroyed");
  auto it = s->queues.find(h);
  if (it == s->queues.end() || h->destroyed) return si_fail(SI_EINVAL, "not a resident scene of this server");
  auto* r = new Request();
  r->ticket = s->next_ticket++;
  r->h = h;
  r->dt = dt;
  r->K = K;
  r->remaining = K;
  r->ncol = ncol < 0 ? -1 : ncol;
  r->cols = std::move(cols);
  r->t_submit = Clock::now();
  s->reqs[r->ticket] = r;
  if (h->count == 0) {   // step() of an empty simulation is a no-op (mpm.js:584)
    r->done = true;
    r->remaining = 0;
  } else {
    it->second.push_back(r);
  }
  *ticket = r->ticket;
  s->cv_work.notify_all();
  return SI_OK;
}

int si_server_poll(si_server* s, uint64_t ticket, int32_t* done, int32_t* status) {
  if (!s || !done) return si_fail(SI_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return si_fail(SI_EINVAL, "unknown ticket");
  *done = it->second->done ? 1 : 0;
  if (status) *status = it->second->status;
  if (it->second->done) { delete it->second; s->reqs.erase(it); }
  return SI_OK;
}

int si_server_wait(si_server* s, uint64_t ticket, int32_t timeout_ms, int32_t* status) {
  if (!s) return si_fail(SI_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return si_fail(SI_EINVAL, "unknown ticket");
  Request* r = it->second;
  auto pred = [&] { return r->done; };
  if (timeout_ms < 0) s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return si_fail(SI_ETIMEOUT, "request not finished within the timeout");
  if (status) *status = r->status;
  delete r;
  s->reqs.erase(ticket);
  return SI_OK;
}

int si_server_stats_get(si_server* s, si_server_stats* o, int32_t reset) {
  if (!s || !o) return si_fail(SI_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  std::memset(o, 0, sizeof(*o));
  o->requests_done = s->requests_done;
  o->substeps_done = s->substeps_done;
  o->particle_substeps = s->particle_substeps;
  o->ticks = s->ticks;
  std::vector<double> v = s->lat;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto q = [&](double p) { return v[std::min(v.size() - 1, (size_t)std::floor(p * (v.size() - 1) + 0.5))]; };
    o->p50_ms = q(0.50);
    o->p99_ms = q(0.99);
    o->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    o->mean_ms = sum / v.size();
  }
  o->busy_s = s->busy_s;
  o->resident_bytes = s->resident;
  o->budget_bytes = s->budget;
  o->resident_scenes = (int32_t)s->footprint.size();
  int32_t q = 0;
  for (auto& kv : s->queues) q += (int32_t)kv.second.size();
  o->queued_requests = q;
  if (reset) {
    s->lat.clear();
    s->requests_done = s->substeps_done = s->particle_substeps = s->ticks = 0;
    s->busy_s = 0;
  }
  return SI_OK;
}

int si_server_call(si_server* s, void (*fn)(void*), void* ctx) {
  if (!s || !fn) return si_fail(SI_EINVAL, "null argument");
  return run_on_world(s, fn, ctx);
}

}  // extern "C"
