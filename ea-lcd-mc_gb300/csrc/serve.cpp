// serve.cpp -- continuous batching of simulation jobs on one GPU (ea_server_*).
//
// A worker thread owns the device side: it admits queued requests whose
// device bytes fit the HBM budget, creates and initialises their contexts,
// and advances every running job one bin per step through the batch of its
// (replica count, cadence) class.  Batches keep up to `depth` bins in flight;
// their job lists change between bins (ea_batch_set_jobs) without draining
// the GPU, so jobs that arrive while others run are admitted as soon as
// memory and a slot are free and their bins share launches with the rest.
// A reaper thread frees released jobs (cudaFree waits for the device) off
// the worker's path.  The reference has no counterpart: it runs one job per
// process (PROGRAM/src/main.cu:10-283).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "eagb.h"

namespace eagb {
void set_last_error(const char *msg);  // api.cu
}

namespace {

int sfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  eagb::set_last_error(buf);
  return code;
}

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t ticket = 0;
  ea_request req{};
  std::vector<double> betas;
  std::vector<uint64_t> cum;
  ea_ctx *ctx = nullptr;
  ea_sp *sp = nullptr;  // sample-packed jobs
  int state = EA_JOB_QUEUED;
  int rc = EA_OK;
  std::string err;
  int bins_done = 0, bins_queued = 0;
  double t_submit = -1, t_admit = -1, t_done = -1, t_ready = -1, t_start = -1;
  double gpu_s = 0;  // device time of its bins (worker only)
  uint64_t bytes = 0;
  int passed = 0;  // times a later request was admitted ahead of this one
  bool freeing = false;  // handed to the reaper
  bool packed() const { return req.layout == EA_LAYOUT_SAMPLE_PACKED; }
  ea_sp_geom spgeom() const {
    const ea_geom &g = req.geom;
    return ea_sp_geom{g.L, g.Lz, g.nbetas, g.nrep, req.nwords, g.bc};
  }
  double su() const {
    const ea_geom &g = req.geom;
    const ea_cadence &c = req.cad;
    const double samples = packed() ? 64.0 * req.nwords : (double)g.nsamples;
    return (double)req.nbins * c.itmax * c.mesfr * c.houfr * c.ptfr * g.L * g.L * g.Lz * g.nrep * g.nbetas * samples;
  }
};

// Jobs of one batch: same replica count and cadence.
using ClassKey = std::tuple<int, int, int, int, int, int, int>;

struct InFlight {
  cudaEvent_t ev0, ev;  // around the bin on the batch stream
  std::vector<Job *> members;    // jobs of the bin
  std::vector<Job *> finishing;  // jobs whose last bin this is
};

// A group is a batch of multispin jobs of one class, or one sample-packed
// job (solo) whose bins run on its own stream.
struct Group {
  ClassKey key;
  ea_cadence cad{};
  int NR = 0;
  bool packed = false;  // a solo group of sample-packed jobs, one at a time
  Job *solo = nullptr;
  ea_batch *batch = nullptr;
  std::vector<Job *> members;
  bool dirty = false;
  std::deque<InFlight> inflight;
};

}  // namespace

struct ea_server {
  ea_server_config cfg{};
  Clock::time_point t0;
  std::mutex m;
  std::condition_variable cv;        // job state changes, submissions, frees
  std::thread worker, reaper;
  std::vector<std::thread> preppers;  // create and initialise admitted jobs
  std::condition_variable cv_prep;
  std::deque<Job *> prep_q;           // admitted, to be created
  std::deque<Job *> ready_q;          // created, to join a batch
  bool stop = false, reaper_stop = false;
  std::deque<Job *> queue;           // submitted, not admitted (arrival order)
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  std::vector<std::unique_ptr<Group>> groups;  // worker only
  std::deque<Job *> to_free;         // released, waiting for the reaper
  std::vector<cudaEvent_t> ev_pool;  // worker only
  int64_t next_ticket = 1;
  int64_t running = 0, admitted = 0, completed = 0, failed = 0, bins = 0, changes = 0, peak_running = 0;
  uint64_t in_use = 0, peak = 0;
  double first_submit = -1, last_done = -1;
  double gpu_busy_s = 0, enqueue_s = 0;  // worker only
  double admit_s = 0;                     // preparation threads, under m
  std::vector<double> lat_ms;
  std::string worker_err;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void finish(ea_server *s, Job *j, int rc, const std::string &err) {
  // caller holds s->m
  j->t_done = s->now();
  if (rc == EA_OK) {
    j->state = EA_JOB_DONE;
    ++s->completed;
    s->lat_ms.push_back(1e3 * (j->t_done - j->t_submit));
    s->last_done = std::max(s->last_done, j->t_done);
  } else {
    j->state = EA_JOB_FAILED;
    j->rc = rc;
    j->err = err;
    ++s->failed;
  }
  s->cv.notify_all();
}

cudaEvent_t get_event(ea_server *s) {
  if (!s->ev_pool.empty()) {
    cudaEvent_t e = s->ev_pool.back();
    s->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Jobs whose last bin has run become DONE.  block: wait for the oldest bin
// in flight when none has ended yet.
void retire(ea_server *s, bool block) {
  if (block) {
    Group *oldest = nullptr;
    for (auto &g : s->groups)
      if (!g->inflight.empty()) { oldest = g.get(); break; }
    if (oldest) cudaEventSynchronize(oldest->inflight.front().ev);
  }
  for (auto &g : s->groups) {
    while (!g->inflight.empty()) {
      InFlight &f = g->inflight.front();
      const cudaError_t q = cudaEventQuery(f.ev);
      if (q == cudaErrorNotReady) break;
      {
        std::lock_guard<std::mutex> lk(s->m);
        for (Job *j : f.finishing) {
          // the job's own stream already waits for the batch; its results
          // (ea_bin_results, ea_get_spins) read after this bin
          --s->running;
          finish(s, j, q == cudaSuccess ? EA_OK : EA_ERR_CUDA,
                 q == cudaSuccess ? "" : std::string("bin failed: ") + cudaGetErrorString(q));
        }
      }
      float ms = 0.f;
      if (q == cudaSuccess && cudaEventElapsedTime(&ms, f.ev0, f.ev) == cudaSuccess) {
        s->gpu_busy_s += 1e-3 * ms;
        for (Job *j : f.members) j->gpu_s += 1e-3 * ms;
      }
      s->ev_pool.push_back(f.ev0);
      s->ev_pool.push_back(f.ev);
      g->inflight.pop_front();
    }
  }
}

Group *group_for(ea_server *s, Job *j) {
  const ea_cadence &c = j->req.cad;
  const ClassKey key{j->req.geom.nrep, c.itmax, c.houfr, c.mesfr, c.ptfr, c.cluster, c.nclust};
  if (!j->packed())
    for (auto &g : s->groups)
      if (!g->packed && g->key == key) return g.get();
  if (j->packed()) {
    // a solo group whose job has finished and whose bins have all ended is reused
    for (auto &g : s->groups)
      if (g->packed && !g->solo && g->members.empty() && g->inflight.empty()) {
        g->solo = j;
        g->key = key;
        g->cad = c;
        g->NR = j->req.geom.nrep;
        return g.get();
      }
  }
  s->groups.emplace_back(new Group());
  Group *g = s->groups.back().get();
  g->packed = j->packed();
  if (j->packed()) g->solo = j;
  g->key = key;
  g->cad = c;
  g->NR = j->req.geom.nrep;
  return g;
}

// Widest sweep tile width for NR replicas whose shared memory (three random
// words per tile site, replica and temperature, the pre-search of every
// temperature, the tile's neighbour records: sweep_smem_for in kernels.cuh)
// holds nb_max temperatures.
int tile_for(int NR, int nb_max) {
  const int c8[3] = {4, 2, 1}, c4[3] = {8, 4, 2}, c2[3] = {16, 8, 4};
  const int *c = NR == 8 ? c8 : NR == 4 ? c4 : c2;
  for (int i = 0; i < 3; ++i)
    if (3 * nb_max * c[i] * NR * 8 + nb_max * 256 * 2 + c[i] * 32 <= 227 * 1024 - 256) return c[i];
  return c[2];
}

// Creates and initialises an admitted job's context (worker thread).
int create_job(ea_server *s, Job *j) {
  if (j->packed()) {
    const ea_sp_geom g = j->spgeom();
    ea_sp *p = nullptr;
    int rc = ea_sp_create(&g, s->cfg.device, &p);
    if (rc) return rc;
    rc = ea_sp_set_temperatures(p, j->betas.data(), j->cum.data());
    if (!rc) rc = ea_sp_init(p, j->req.masters, j->req.jobid);
    if (rc) {
      ea_sp_destroy(p);
      return rc;
    }
    j->sp = p;
    return EA_OK;
  }
  ea_ctx *c = nullptr;
  int rc = ea_create(&j->req.geom, s->cfg.device, &c);
  if (rc) return rc;
  // the batch draws every job's cluster uniforms on the job's own stream;
  // no SM partition per job
  if (!rc) rc = ea_set_rng_sms(c, 0);
  if (!rc) rc = ea_set_temperatures(c, j->betas.data(), j->cum.data());
  if (!rc) rc = ea_init_run(c, j->req.masters, nullptr, j->req.iter0, j->req.jobid);
  if (rc) {
    ea_destroy(c);
    return rc;
  }
  j->ctx = c;
  return EA_OK;
}

// Admits queued requests in arrival order while their bytes fit the budget
// and a slot is free; a later, smaller request may pass one that does not
// fit, at most 32 times, after which the waiting one blocks the queue.
void admit(ea_server *s) {
  std::vector<Job *> take;
  {
    std::lock_guard<std::mutex> lk(s->m);
    int64_t slots = s->cfg.max_jobs - s->running - (int64_t)take.size();
    uint64_t room = s->cfg.hbm_budget > s->in_use ? s->cfg.hbm_budget - s->in_use : 0;
    bool blocked = false;
    std::vector<Job *> skipped;
    for (auto it = s->queue.begin(); it != s->queue.end() && slots > 0 && !blocked;) {
      Job *j = *it;
      if (j->bytes <= room) {
        for (Job *k : skipped) ++k->passed;
        take.push_back(j);
        room -= j->bytes;
        s->in_use += j->bytes;
        --slots;
        it = s->queue.erase(it);
      } else {
        skipped.push_back(j);
        if (j->passed >= 32) blocked = true;
        ++it;
      }
    }
    s->peak = std::max(s->peak, s->in_use);
    for (Job *j : take) {
      j->state = EA_JOB_RUNNING;
      j->t_admit = s->now();
      ++s->running;
      ++s->admitted;
    }
    s->peak_running = std::max(s->peak_running, s->running);
  }
  if (!take.empty()) {
    std::lock_guard<std::mutex> lk(s->m);
    for (Job *j : take) s->prep_q.push_back(j);
    s->cv_prep.notify_all();
  }
}

// Preparation thread: creates and initialises admitted jobs (device
// allocation, host-side seeding of spins and couplings, uploads) off the
// worker's path, so that bins keep flowing while jobs are being set up.
void prep_main(ea_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;) {
    s->cv_prep.wait(lk, [&] { return !s->prep_q.empty() || s->stop; });
    if (s->stop) break;
    Job *j = s->prep_q.front();
    s->prep_q.pop_front();
    lk.unlock();
    const auto ta = Clock::now();
    const int rc = create_job(s, j);
    const std::string e = rc ? std::string(ea_last_error()) : std::string();
    lk.lock();
    s->admit_s += std::chrono::duration<double>(Clock::now() - ta).count();
    if (rc) {
      s->in_use -= j->bytes;
      --s->running;
      finish(s, j, rc, e);
      continue;
    }
    j->t_ready = s->now();
    s->ready_q.push_back(j);
    s->cv.notify_all();
  }
}

// Jobs whose contexts are ready join the batch of their class.
void join_ready(ea_server *s) {
  std::deque<Job *> ready;
  {
    std::lock_guard<std::mutex> lk(s->m);
    ready.swap(s->ready_q);
  }
  for (Job *j : ready) {
    Group *g = group_for(s, j);
    g->members.push_back(j);
    g->dirty = true;
  }
}

// Enqueues one bin of a group's batch; false if the group has nothing to run
// or too many bins in flight.
bool step_group(ea_server *s, Group *g) {
  if (g->members.empty() || (int)g->inflight.size() >= s->cfg.depth) return false;
  const auto te = Clock::now();
  int rc = EA_OK;
  InFlight f;
  f.ev0 = get_event(s);
  std::vector<ea_ctx *> ctxs;
  for (Job *j : g->members) ctxs.push_back(j->ctx);
  void *st = nullptr;
  if (g->solo) {
    ea_sp_stream(g->solo->sp, &st);
    cudaEventRecord(f.ev0, (cudaStream_t)st);
    rc = ea_sp_run(g->solo->sp, &g->cad, nullptr);
  } else if (!g->batch) {
    rc = ea_batch_create(ctxs.data(), (int32_t)ctxs.size(), s->cfg.tile ? s->cfg.tile : tile_for(g->NR, s->cfg.nb_max),
                         &g->batch);
    if (rc == EA_OK) ++s->changes;
  } else if (g->dirty) {
    rc = ea_batch_set_jobs(g->batch, ctxs.data(), (int32_t)ctxs.size());
    if (rc == EA_OK) ++s->changes;
  }
  if (rc == EA_OK && !g->solo) {
    g->dirty = false;
    ea_batch_stream(g->batch, &st);
    cudaEventRecord(f.ev0, (cudaStream_t)st);
    rc = ea_batch_run_bin(g->batch, &g->cad);
  }
  if (rc) {
    // a batch that cannot run fails its jobs; their bins in flight finish first
    const std::string e = ea_last_error();
    s->ev_pool.push_back(f.ev0);
    for (auto &pending : g->inflight) cudaEventSynchronize(pending.ev);
    retire(s, false);
    std::lock_guard<std::mutex> lk(s->m);
    for (Job *j : g->members) {
      --s->running;
      finish(s, j, rc, e);
      j->freeing = true;  // nothing to read: free at once
      s->to_free.push_back(j);
    }
    g->members.clear();
    g->solo = nullptr;
    if (g->batch) { ea_batch_destroy(g->batch); g->batch = nullptr; }
    s->cv.notify_all();
    return false;
  }
  ++s->bins;
  f.ev = get_event(s);
  cudaEventRecord(f.ev, (cudaStream_t)st);
  s->enqueue_s += std::chrono::duration<double>(Clock::now() - te).count();
  std::vector<Job *> stay;
  {
    std::lock_guard<std::mutex> lk(s->m);
    const double t = s->now();
    f.members = g->members;
    for (Job *j : g->members) {
      if (j->t_start < 0) j->t_start = t;
      ++j->bins_done;
      if (j->bins_done >= j->req.nbins) f.finishing.push_back(j);
      else stay.push_back(j);
    }
  }
  if (!f.finishing.empty()) {
    g->members = stay;
    g->dirty = true;
    if (g->solo && stay.empty()) g->solo = nullptr;
  }
  g->inflight.push_back(std::move(f));
  return true;
}

void worker_main(ea_server *s) {
  cudaSetDevice(s->cfg.device);
  for (;;) {
    {
      std::lock_guard<std::mutex> lk(s->m);
      if (s->stop) break;
    }
    retire(s, false);
    admit(s);
    join_ready(s);
    bool any = false;
    for (auto &g : s->groups) any = step_group(s, g.get()) || any;
    if (any) continue;
    bool inflight = false;
    for (auto &g : s->groups) inflight = inflight || !g->inflight.empty();
    if (inflight) {
      retire(s, true);
      continue;
    }
    std::unique_lock<std::mutex> lk(s->m);
    if (s->stop) break;
    // nothing on the GPU: wait for a submission, a prepared job or a freed budget
    if (s->ready_q.empty()) s->cv.wait_for(lk, std::chrono::milliseconds(20));
  }
  // shutting down: the bins in flight end, running jobs are cancelled
  for (auto &g : s->groups)
    for (auto &f : g->inflight) cudaEventSynchronize(f.ev);
  retire(s, false);
  {
    std::lock_guard<std::mutex> lk(s->m);
    for (auto &g : s->groups)
      for (Job *j : g->members) {
        --s->running;
        finish(s, j, EA_ERR_STATE, "cancelled");
      }
    // the preparation threads have ended (joined before the worker)
    for (Job *j : s->ready_q) {
      --s->running;
      finish(s, j, EA_ERR_STATE, "cancelled");
    }
    s->ready_q.clear();
    for (Job *j : s->prep_q) {
      --s->running;
      s->in_use -= j->bytes;
      finish(s, j, EA_ERR_STATE, "cancelled");
    }
    s->prep_q.clear();
  }
  for (auto &g : s->groups) {
    g->members.clear();
    if (g->batch) ea_batch_destroy(g->batch);
    g->batch = nullptr;
  }
  for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
  s->ev_pool.clear();
}

void reaper_main(ea_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;) {
    s->cv.wait(lk, [&] { return !s->to_free.empty() || s->reaper_stop; });
    if (s->to_free.empty()) break;
    Job *j = s->to_free.front();
    s->to_free.pop_front();
    ea_ctx *c = j->ctx;
    ea_sp *p = j->sp;
    j->ctx = nullptr;
    j->sp = nullptr;
    lk.unlock();
    if (c) ea_destroy(c);
    if (p) ea_sp_destroy(p);
    lk.lock();
    j->state = EA_JOB_RELEASED;
    s->in_use -= j->bytes;
    s->cv.notify_all();
  }
}

}  // namespace

extern "C" {

int ea_server_create(const ea_server_config *cfg, ea_server **out) {
  if (!cfg || !out) return sfail(EA_ERR_ARG, "null argument");
  std::unique_ptr<ea_server> s(new ea_server());
  s->cfg = *cfg;
  if (s->cfg.max_jobs <= 0) s->cfg.max_jobs = 1024;
  if (s->cfg.depth <= 0) s->cfg.depth = 2;
  if (s->cfg.nb_max <= 0) s->cfg.nb_max = 64;
  if (s->cfg.nb_max > 255) return sfail(EA_ERR_ARG, "nb_max above 255");
  if (cudaSetDevice(s->cfg.device) != cudaSuccess) return sfail(EA_ERR_CUDA, "cudaSetDevice(%d)", s->cfg.device);
  if (!s->cfg.hbm_budget) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return sfail(EA_ERR_CUDA, "cudaMemGetInfo");
    s->cfg.hbm_budget = (uint64_t)(0.9 * (double)fr);
  }
  s->t0 = Clock::now();
  ea_server *p = s.release();
  p->worker = std::thread(worker_main, p);
  p->reaper = std::thread(reaper_main, p);
  const unsigned hw = std::thread::hardware_concurrency();
  const int nprep = std::max(2, std::min(8, (int)(hw ? hw / 2 : 2)));
  for (int i = 0; i < nprep; ++i) p->preppers.emplace_back(prep_main, p);
  *out = p;
  return EA_OK;
}

int ea_server_submit(ea_server *s, const ea_request *r, int64_t *ticket) {
  if (!s || !r || !r->betas || !r->cum) return sfail(EA_ERR_ARG, "null argument");
  const ea_geom &g = r->geom;
  if (r->nbins < 1 || r->cad.itmax < 1 || r->cad.houfr < 1 || r->cad.mesfr < 1 || r->cad.ptfr < 0)
    return sfail(EA_ERR_ARG, "bad cadence or bin count");
  if (g.nbetas > s->cfg.nb_max) return sfail(EA_ERR_ARG, "NB=%d above the server's nb_max=%d", g.nbetas, s->cfg.nb_max);
  if (r->cad.cluster && g.nrep < (r->layout == EA_LAYOUT_SAMPLE_PACKED ? 2 : 4))
    return sfail(EA_ERR_ARG, "the Houdayer move needs at least 2 replicas per group");
  if (r->layout == EA_LAYOUT_SAMPLE_PACKED && (r->cad.ptfr < 1 || r->cad.nclust > g.nbetas))
    return sfail(EA_ERR_ARG, "sample-packed jobs temper every ptfr >= 1 sweeps");
  std::unique_ptr<Job> j(new Job());
  int rc;
  if (r->layout == EA_LAYOUT_SAMPLE_PACKED) {
    if (r->nwords < 1) return sfail(EA_ERR_ARG, "a sample-packed job needs nwords >= 1");
    const ea_sp_geom sg{g.L, g.Lz, g.nbetas, g.nrep, r->nwords, g.bc};
    rc = ea_sp_job_bytes(&sg, &r->cad, r->betas, &j->bytes);
  } else if (r->layout == EA_LAYOUT_MULTISPIN) {
    rc = ea_job_bytes(&g, &r->cad, r->betas, &j->bytes);
  } else {
    return sfail(EA_ERR_ARG, "unknown layout %d", r->layout);
  }
  if (rc) return sfail(rc, "%s", ea_last_error());
  std::lock_guard<std::mutex> lk(s->m);
  if (s->stop) return sfail(EA_ERR_STATE, "server is shutting down");
  if (j->bytes > s->cfg.hbm_budget)
    return sfail(EA_ERR_ARG, "job needs %llu bytes, budget %llu", (unsigned long long)j->bytes,
                 (unsigned long long)s->cfg.hbm_budget);
  j->req = *r;
  j->betas.assign(r->betas, r->betas + g.nbetas);
  j->cum.assign(r->cum, r->cum + (size_t)g.nbetas * 256);
  j->req.betas = nullptr;
  j->req.cum = nullptr;
  j->ticket = s->next_ticket++;
  j->t_submit = s->now();
  if (s->first_submit < 0) s->first_submit = j->t_submit;
  if (ticket) *ticket = j->ticket;
  s->queue.push_back(j.get());
  s->jobs[j->ticket] = std::move(j);
  s->cv.notify_all();
  return EA_OK;
}

int ea_server_wait(ea_server *s, int64_t ticket, double timeout_s, ea_ctx **job) {
  if (!s) return sfail(EA_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return sfail(EA_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Job *j = it->second.get();
  auto ready = [&] { return j->state == EA_JOB_DONE || j->state == EA_JOB_FAILED || j->state == EA_JOB_RELEASED; };
  if (timeout_s < 0) {
    s->cv.wait(lk, ready);
  } else if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    return sfail(EA_ERR_STATE, "job %lld not finished", (long long)ticket);
  }
  if (j->state == EA_JOB_FAILED) return sfail(j->rc, "job %lld failed: %s", (long long)ticket, j->err.c_str());
  if (j->state == EA_JOB_RELEASED) return sfail(EA_ERR_STATE, "job %lld was released", (long long)ticket);
  if (job) *job = j->ctx;
  return EA_OK;
}

int ea_server_info(ea_server *s, int64_t ticket, ea_job_info *info) {
  if (!s || !info) return sfail(EA_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return sfail(EA_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  const Job *j = it->second.get();
  info->state = j->state;
  info->bins_done = j->bins_done;
  info->t_submit = j->t_submit;
  info->t_admit = j->t_admit;
  info->t_done = j->t_done;
  info->t_ready = j->t_ready;
  info->t_start = j->t_start;
  info->gpu_s = j->gpu_s;
  info->bytes = j->bytes;
  info->spin_updates = j->su();
  return EA_OK;
}

int ea_server_sp_job(ea_server *s, int64_t ticket, ea_sp **job) {
  if (!s || !job) return sfail(EA_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return sfail(EA_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  const Job *j = it->second.get();
  if (j->state != EA_JOB_DONE || !j->sp) return sfail(EA_ERR_STATE, "job %lld is not a finished sample-packed job", (long long)ticket);
  *job = j->sp;
  return EA_OK;
}

int ea_server_release(ea_server *s, int64_t ticket) {
  if (!s) return sfail(EA_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return sfail(EA_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Job *j = it->second.get();
  if (j->state == EA_JOB_FAILED) {
    j->state = EA_JOB_RELEASED;
    return EA_OK;
  }
  if (j->state != EA_JOB_DONE) return sfail(EA_ERR_STATE, "job %lld has not finished", (long long)ticket);
  j->state = EA_JOB_RELEASED;
  j->freeing = true;
  s->to_free.push_back(j);
  s->cv.notify_all();
  return EA_OK;
}

int ea_server_stats(ea_server *s, ea_serve_stats *st) {
  if (!s || !st) return sfail(EA_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->m);
  std::memset(st, 0, sizeof(*st));
  st->submitted = (int64_t)s->jobs.size();
  st->admitted = s->admitted;
  st->completed = s->completed;
  st->failed = s->failed;
  st->queued = (int64_t)s->queue.size();
  st->running = s->running;
  st->bins = s->bins;
  st->batch_changes = s->changes;
  st->peak_running = s->peak_running;
  std::vector<double> l = s->lat_ms;
  std::sort(l.begin(), l.end());
  // nearest-rank percentiles
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    size_t k = (size_t)std::ceil(p * (double)l.size());
    return l[std::min(l.size(), std::max<size_t>(k, 1)) - 1];
  };
  st->p50_ms = pct(0.50);
  st->p99_ms = pct(0.99);
  st->max_ms = l.empty() ? 0.0 : l.back();
  double sum = 0, su = 0;
  for (double x : l) sum += x;
  st->mean_ms = l.empty() ? 0.0 : sum / (double)l.size();
  for (auto &kv : s->jobs)
    if (kv.second->t_done >= 0 && kv.second->rc == EA_OK) su += kv.second->su();
  st->spin_updates = su;
  st->span_s = s->last_done >= 0 ? s->last_done - s->first_submit : 0.0;
  st->budget = s->cfg.hbm_budget;
  st->bytes_in_use = s->in_use;
  st->bytes_peak = s->peak;
  st->gpu_busy_s = s->gpu_busy_s;
  st->enqueue_s = s->enqueue_s;
  st->admit_s = s->admit_s;
  // latency components of the completed jobs
  std::vector<double> cq, cp, cs, cr, cg;
  for (auto &kv : s->jobs) {
    const Job *j = kv.second.get();
    if (j->t_done < 0 || j->rc != EA_OK || j->t_start < 0) continue;
    cq.push_back(1e3 * (j->t_admit - j->t_submit));
    cp.push_back(1e3 * (j->t_ready - j->t_admit));
    cs.push_back(1e3 * (j->t_start - j->t_ready));
    cr.push_back(1e3 * (j->t_done - j->t_start));
    cg.push_back(1e3 * j->gpu_s);
  }
  auto pct_of = [](std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    size_t k = (size_t)std::ceil(p * (double)v.size());
    return v[std::min(v.size(), std::max<size_t>(k, 1)) - 1];
  };
  st->queue_p50_ms = pct_of(cq, 0.5); st->queue_p99_ms = pct_of(cq, 0.99);
  st->prep_p50_ms = pct_of(cp, 0.5); st->prep_p99_ms = pct_of(cp, 0.99);
  st->start_p50_ms = pct_of(cs, 0.5); st->start_p99_ms = pct_of(cs, 0.99);
  st->run_p50_ms = pct_of(cr, 0.5); st->run_p99_ms = pct_of(cr, 0.99);
  st->gpu_p50_ms = pct_of(cg, 0.5); st->gpu_p99_ms = pct_of(cg, 0.99);
  return EA_OK;
}

int ea_server_drain(ea_server *s) {
  if (!s) return sfail(EA_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->m);
  s->cv.wait(lk, [&] { return s->queue.empty() && s->running == 0; });
  return EA_OK;
}

int ea_server_destroy(ea_server *s) {
  if (!s) return EA_OK;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
    for (Job *j : s->queue) {
      j->state = EA_JOB_FAILED;
      j->rc = EA_ERR_STATE;
      j->err = "cancelled";
      ++s->failed;
    }
    s->queue.clear();
    s->cv.notify_all();
    s->cv_prep.notify_all();
  }
  for (auto &t : s->preppers) t.join();
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->m);
    for (auto &kv : s->jobs)
      if ((kv.second->ctx || kv.second->sp) && !kv.second->freeing) {
        kv.second->freeing = true;
        s->to_free.push_back(kv.second.get());
      }
    s->reaper_stop = true;
    s->cv.notify_all();
  }
  if (s->reaper.joinable()) s->reaper.join();
  delete s;
  return EA_OK;
}

}  // extern "C"
