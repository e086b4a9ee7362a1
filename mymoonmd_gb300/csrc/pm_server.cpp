// Request executor behind pm_server_* (no reference counterpart): the batched
// stream of independent solves and the serving loop.
//
// Convection-diffusion requests run in batch lanes: one lane (host thread,
// CUDA stream) per set-up (kind, geometry, mesh size, levels, element). A lane
// keeps up to `gpu_batch_slots` device-resident problems of its set-up and a
// BatchEngine over them (pm_batch.h): requests that arrive while others are on
// the GPU join at the next restart-cycle boundary as slots free up, and every
// kernel of an Arnoldi step and of the V-cycle serves all of the lane's
// in-flight requests in one launch, each Arnoldi step one CUDA graph. Lanes of
// different set-ups run concurrently on their own streams.
//
// Stokes requests (and convection-diffusion requests when gpu_batch_slots is
// 0) go to n_workers worker threads, each with its own stream and a cache of
// device-resident problems per set-up.
//
// Admission by HBM footprint: one ledger for the whole server. Every problem
// (and every lane's batch memory) is reserved before it is allocated, from
// the measured footprint of an earlier problem of the same set-up or, the
// first time, from an estimate; the reservation is corrected to the measured
// bytes after the allocation. A request that does not fit waits until memory
// frees: idle lanes and idle workers give their cached problems back when the
// ledger is under pressure. A set-up whose one problem is larger than the cap
// is served when nothing else holds memory and released right after.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cstdio>
#include <cstdlib>

#include "pm_batch.h"
#include "pm_problem.h"
#include "pmgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct SetupKey {
  int kind, geometry, root_n, n_refine, n_levels, elem;
  bool operator<(const SetupKey& o) const {
    return std::tie(kind, geometry, root_n, n_refine, n_levels, elem) <
           std::tie(o.kind, o.geometry, o.root_n, o.n_refine, o.n_levels, o.elem);
  }
};

struct SharedSetup {
  std::mutex mu;  // serialises the one build
  pm_disc* disc = nullptr;
  int status = -1;  // -1 not built yet
  std::string error;
  std::atomic<int64_t> footprint{0};  // measured device bytes of one problem (0 = not yet)
  ~SharedSetup() {
    if (disc) pm_disc_destroy(disc);
  }
};

struct Cached {
  pm_problem* p = nullptr;
  int64_t bytes = 0;
  uint64_t last_use = 0;
  int n_dofs = 0;
};

struct Job {
  pm_request req;
  Clock::time_point submitted;
};

// device bytes of one problem before any was measured: matrices (FP64 CSR,
// FP32 copy, sliced FP32 and FP64 copies, element storage) per nonzero and
// the vectors per DOF of the finest level
int64_t estimate_bytes(const pm_disc* d) {
  int64_t nnz = 0, dofs = 0;
  for (int l = 0;; ++l) {
    int nc = 0, nl = 0, nd = 0, na = 0;
    int64_t nz = 0;
    if (pm_disc_level_info(d, l, 0, &nc, &nl, &nd, &na, &nz) != PM_OK) break;
    nnz += nz + int64_t(nc) * nl * (nl + 1);
    dofs = nd;
  }
  return nnz * 48 + dofs * 64 * 8 + (int64_t(64) << 20);
}

}  // namespace

struct Lane;

struct pm_server {
  int device = 0;
  std::string params_cd, params_stokes;
  int batch_slots = 8;
  int n_workers = 1;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  std::deque<Job> jobs;  // worker pool queue
  std::map<SetupKey, std::unique_ptr<Lane>> lanes;
  std::deque<pm_result> done;
  uint64_t submitted = 0, completed = 0;
  bool stop = false;
  std::mutex setup_mu;
  std::map<SetupKey, std::shared_ptr<SharedSetup>> setups;
  std::atomic<uint64_t> served{0}, evictions{0};
  std::atomic<int> workers_ready{0}, workers_failed{0};
  bool trace = std::getenv("PMGPU_SERVER_TRACE") != nullptr;  // request start/finish lines on stderr

  // --- the HBM ledger ---
  std::mutex led_mu;
  std::condition_variable led_cv;
  int64_t cap = INT64_MAX;
  int64_t committed = 0;
  std::atomic<bool> pressure{false};
  std::atomic<int64_t> committed_view{0};

  // the set-up of k (built once; convection-diffusion structures on the
  // caller's GPU when a context is given)
  std::shared_ptr<SharedSetup> setup_for(const SetupKey& k, pm_ctx* ctx = nullptr) {
    std::shared_ptr<SharedSetup> s;
    {
      std::lock_guard<std::mutex> g(setup_mu);
      auto& slot = setups[k];
      if (!slot) slot = std::make_shared<SharedSetup>();
      s = slot;
    }
    std::lock_guard<std::mutex> g(s->mu);
    if (s->status < 0) {
      s->status = ctx && k.kind == 0
                      ? pm_disc_create_device(ctx, k.geometry, k.root_n, k.n_refine, k.n_levels, k.kind, k.elem, 0,
                                              &s->disc)
                      : pm_disc_create(k.geometry, k.root_n, k.n_refine, k.n_levels, k.kind, k.elem, &s->disc);
      if (s->status != PM_OK) s->error = pm_last_error(nullptr);
    }
    return s;
  }

  // Reserve `bytes`, waiting while other holders may still free memory.
  // holds: bytes the caller already holds (an exclusive reservation above the
  // cap needs every other holder gone). Returns false only on shutdown.
  bool reserve(int64_t bytes, int64_t holds) {
    std::unique_lock<std::mutex> lk(led_mu);
    for (;;) {
      const bool fits = committed + bytes <= cap;
      const bool alone = committed == holds;  // nobody else holds memory
      if (fits || (alone && bytes + holds > cap)) {
        committed += bytes;
        committed_view = committed;
        return true;
      }
      if (stop_requested()) return false;
      pressure = true;
      notify_all_threads();
      led_cv.wait_for(lk, std::chrono::milliseconds(20));
    }
  }
  void adjust(int64_t delta) {
    {
      std::lock_guard<std::mutex> lk(led_mu);
      committed += delta;
      committed_view = committed;
      if (committed <= cap) pressure = false;
    }
    led_cv.notify_all();
  }
  bool stop_requested() {
    std::lock_guard<std::mutex> g(mu);
    return stop;
  }
  void notify_all_threads();
  void push_result(const pm_result& r) {
    served++;
    {
      std::lock_guard<std::mutex> g(mu);
      done.push_back(r);
      completed++;
    }
    cv_done.notify_all();
  }

  void worker(int index);
};

// ------------------------------------------------------------------ lanes ---
struct Lane {
  pm_server* srv = nullptr;
  SetupKey key{};
  int index = 0;
  std::thread th;
  std::condition_variable cv;   // guarded by srv->mu
  std::deque<Job> pending;      // guarded by srv->mu
  int active = 0;               // guarded by srv->mu (requests in the engine)

  void run();
};

void pm_server::notify_all_threads() {
  cv_job.notify_all();
  std::lock_guard<std::mutex> g(mu);
  for (auto& kv : lanes) kv.second->cv.notify_all();
}

void Lane::run() {
  pm_server& S = *srv;
  pm_ctx* ctx = nullptr;
  if (pm_ctx_create(S.device, &ctx) != PM_OK) ctx = nullptr;
  struct Slot {
    pm_problem* p = nullptr;
    bool busy = false;
    Job job;
    Clock::time_point started;
    bool fresh = false;  // created for this request (no reuse)
  };
  std::vector<Slot> slots;
  pm::BatchEngine* engine = nullptr;
  bool lone = false;  // the parameters are outside what the batch engine runs
  int64_t held = 0;  // ledger bytes of this lane
  std::shared_ptr<SharedSetup> setup;
  const std::string prm = S.params_cd + "\nmultigrid_n_levels: " + std::to_string(key.n_levels) + "\n" +
                          "gpu_gram_schmidt: cgs2\n";
  auto fail_job = [&](const Job& job, int status, const std::string& msg) {
    pm_result r{};
    r.tag = job.req.tag;
    r.status = status;
    r.worker = S.n_workers + index;
    r.latency_ms = ms_since(job.submitted, Clock::now());
    if (S.trace) std::fprintf(stderr, "[pm_server] lane %d tag %llu failed: %s\n", index,
                              (unsigned long long)job.req.tag, msg.c_str());
    S.push_result(r);
  };
  auto release_all = [&]() {
    pm::batch_destroy(engine);
    engine = nullptr;
    for (auto& sl : slots) pm_problem_destroy(sl.p);
    const size_t n = slots.size();
    slots.clear();
    if (held) S.adjust(-held);
    held = 0;
    if (n) S.evictions += n;
  };
  for (;;) {
    std::vector<Job> taken;
    bool idle_release = false;
    {
      std::unique_lock<std::mutex> lk(S.mu);
      cv.wait_for(lk, std::chrono::milliseconds(50), [&] {
        return S.stop || !pending.empty() || active > 0 || (S.pressure && !slots.empty());
      });
      if (S.stop && pending.empty() && active == 0) break;
      if (pending.empty() && active == 0) {
        if (S.pressure && !slots.empty()) idle_release = true;
        else continue;
      }
      // requests for the free slots (and for new slots while memory allows)
      int free_slots = 0;
      for (auto& sl : slots) free_slots += sl.busy ? 0 : 1;
      const int room = std::max(0, S.batch_slots - int(slots.size()));
      while (!pending.empty() && int(taken.size()) < free_slots + room) {
        taken.push_back(pending.front());
        pending.pop_front();
      }
      active += int(taken.size());
    }
    if (idle_release) {
      release_all();
      continue;
    }
    if (!ctx) {
      for (auto& j : taken) fail_job(j, PM_E_CUDA, "no context");
      std::lock_guard<std::mutex> g(S.mu);
      active -= int(taken.size());
      continue;
    }
    // prepare the joining requests' problems
    std::vector<pm_problem*> join;
    std::vector<Job> deferred;
    for (auto& job : taken) {
      const auto t0 = Clock::now();
      if (!setup) setup = S.setup_for(key, ctx);
      if (setup->status != PM_OK) {
        fail_job(job, setup->status, setup->error);
        std::lock_guard<std::mutex> g(S.mu);
        active--;
        continue;
      }
      Slot* sl = nullptr;
      for (auto& s : slots)
        if (!s.busy) {
          sl = &s;
          break;
        }
      bool fresh = false;
      if (!sl) {
        // a new slot problem: reserve its footprint first (without blocking
        // the requests already on the GPU: then the request waits for a slot)
        const int64_t est = setup->footprint > 0 ? setup->footprint.load() : estimate_bytes(setup->disc);
        bool ok;
        int n_busy = 0;
        for (auto& s : slots) n_busy += s.busy ? 1 : 0;
        if (n_busy == 0 && join.empty()) ok = S.reserve(est, held);
        else {
          std::lock_guard<std::mutex> lk(S.led_mu);
          ok = S.committed + est <= S.cap;
          if (ok) {
            S.committed += est;
            S.committed_view = S.committed;
          }
        }
        if (!ok) {
          if (S.stop_requested()) {
            fail_job(job, PM_E_OOM, "the server stopped before memory for the request was free");
            std::lock_guard<std::mutex> g(S.mu);
            active--;
          } else {
            deferred.push_back(job);  // waits for a slot or for memory
          }
          continue;
        }
        const int64_t before = pm::g_thread_dev_bytes;
        pm_problem* p = nullptr;
        int rc = pm_problem_create_cd(ctx, setup->disc, &job.req.coeffs, 0, prm.c_str(), &p);
        const int64_t grown = pm::g_thread_dev_bytes - before;
        S.adjust(grown - est);
        held += grown;
        if (rc != PM_OK) {
          fail_job(job, rc, pm_last_error(ctx));
          std::lock_guard<std::mutex> g(S.mu);
          active--;
          continue;
        }
        if (setup->footprint == 0) setup->footprint = grown;
        slots.push_back(Slot());
        sl = &slots.back();
        sl->p = p;
        fresh = true;
      }
      sl->busy = true;
      sl->job = job;
      sl->started = t0;
      sl->fresh = fresh;
      pm_problem* p = sl->p;
      p->coeffs = job.req.coeffs;
      const int64_t before = pm::g_thread_dev_bytes;
      int rc = pm_problem_reset_solution(p);
      if (rc == PM_OK) rc = pm_problem_assemble(p);
      if (rc == PM_OK) {
        rc = pm_solver_update_matrix(p->solver, p->mats.back());
        if (rc == PM_OK) p->solver_ready = true;
      }
      if (rc == PM_OK && !engine && !lone) {
        try {
          const int64_t b0 = pm::g_thread_dev_bytes;
          engine = pm::batch_create(ctx, S.batch_slots, p);
          const int64_t eb = pm::g_thread_dev_bytes - b0;
          S.adjust(eb);
          held += eb;
        } catch (const pm::Error& e) {
          // a configuration the batch does not cover (another smoother or
          // Gram-Schmidt variant, a longer restart): the lane solves one
          // request at a time
          if (e.code != PM_E_UNSUPPORTED) {
            rc = e.code;
            ctx->last_error = e.what();
          }
          lone = true;
        }
      }
      const int64_t grown = pm::g_thread_dev_bytes - before;
      if (grown) {
        S.adjust(grown);
        held += grown;
      }
      if (rc != PM_OK) {
        sl->busy = false;
        fail_job(job, rc, pm_last_error(ctx));
        std::lock_guard<std::mutex> g(S.mu);
        active--;
        continue;
      }
      join.push_back(p);
    }
    if (!deferred.empty()) {
      std::lock_guard<std::mutex> g(S.mu);
      for (auto it = deferred.rbegin(); it != deferred.rend(); ++it) pending.push_front(*it);
      active -= int(deferred.size());
    }
    if (!engine && !lone) continue;
    std::vector<pm::BatchDone> finished;
    try {
      if (lone) {
        for (pm_problem* p : join) {
          const int rc = pm_problem_solve(p);
          pm::BatchDone d{p, {}};
          d.r.status = rc;
          finished.push_back(d);
        }
      } else {
        finished = pm::batch_cycle(engine, join);
      }
    } catch (const pm::Error& e) {
      // the lane's device state is suspect: fail its requests and start over
      for (auto& sl : slots)
        if (sl.busy) fail_job(sl.job, e.code, e.what());
      int n_busy = 0;
      for (auto& sl : slots) n_busy += sl.busy ? 1 : 0;
      release_all();
      std::lock_guard<std::mutex> g(S.mu);
      active -= n_busy;
      continue;
    }
    for (const auto& d : finished) {
      Slot* sl = nullptr;
      for (auto& s : slots)
        if (s.p == d.p) sl = &s;
      if (!sl) continue;
      int status = d.r.status;
      if (!lone && (status == PM_E_DIVERGED || status == PM_E_BREAKDOWN)) {
        // a failed cycle of the batch: the request is solved alone, with the
        // lone solve's fallbacks (FP64 cycle after an FP32 overflow)
        pm_problem* p = sl->p;
        int rc = pm_problem_reset_solution(p);
        if (rc == PM_OK) rc = pm_problem_assemble(p);
        if (rc == PM_OK) rc = pm_problem_solve(p);
        status = rc;
      }
      pm_result r{};
      r.tag = sl->job.req.tag;
      r.worker = S.n_workers + index;
      r.cache_hit = sl->fresh ? 0 : 1;
      int n = 0, na = 0;
      pm_problem_size(sl->p, &n, &na);
      r.n_dofs = n;
      pm_problem_last_info(sl->p, &r.iterations, &r.residual, &r.initial_residual);
      if (status == PM_OK) {
        pm_solver* sv = sl->p->solver;
        if (!(r.residual <= std::max(sv->tol, sv->reduction * r.initial_residual))) status = PM_E_MAXIT;
      }
      if ((status == PM_OK || status == PM_E_MAXIT) && sl->job.req.solution_out) {
        const int rc = pm_problem_get_solution(sl->p, sl->job.req.solution_out);
        if (rc != PM_OK) status = rc;
      }
      r.status = status;
      const auto t_end = Clock::now();
      r.queue_ms = ms_since(sl->job.submitted, sl->started);
      r.run_ms = ms_since(sl->started, t_end);
      r.latency_ms = ms_since(sl->job.submitted, t_end);
      if (S.trace)
        std::fprintf(stderr, "[pm_server] lane %d done tag %llu status %d its %d latency %.1f ms\n", index,
                     (unsigned long long)r.tag, r.status, r.iterations, r.latency_ms);
      sl->busy = false;
      sl->p->solver_ready = false;  // re-updated by the next request's assembly
      {
        std::lock_guard<std::mutex> g(S.mu);
        active--;
      }
      S.push_result(r);
    }
    // a set-up above the cap: served alone, then released
    if (held > S.cap) {
      bool any_busy = false;
      for (auto& sl : slots) any_busy = any_busy || sl.busy;
      bool more;
      {
        std::lock_guard<std::mutex> g(S.mu);
        more = !pending.empty();
      }
      if (!any_busy && !more) release_all();
    }
  }
  release_all();
  if (ctx) pm_ctx_destroy(ctx);
}

// --------------------------------------------------------- worker pool ---
void pm_server::worker(int index) {
  pm_ctx* ctx = nullptr;
  const int rc0 = pm_ctx_create(device, &ctx);
  {
    // under the mutex: the creator tests these counts and waits on cv_done
    std::lock_guard<std::mutex> g(mu);
    if (rc0 != PM_OK) workers_failed++;
    else workers_ready++;
  }
  cv_done.notify_all();
  if (rc0 != PM_OK) return;
  std::map<SetupKey, Cached> cache;
  uint64_t tick = 0;
  int64_t held = 0;
  auto evict = [&](std::map<SetupKey, Cached>::iterator victim) {
    held -= victim->second.bytes;
    adjust(-victim->second.bytes);
    pm_problem_destroy(victim->second.p);
    cache.erase(victim);
    evictions++;
  };
  for (;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_job.wait_for(lk, std::chrono::milliseconds(50),
                      [&] { return stop || !jobs.empty() || (pressure && !cache.empty()); });
      if (stop && jobs.empty()) break;
      if (jobs.empty()) {
        if (pressure && !cache.empty()) {
          lk.unlock();
          while (!cache.empty()) evict(cache.begin());  // idle under pressure: give the memory back
        }
        continue;
      }
      job = jobs.front();
      jobs.pop_front();
    }
    const pm_request& rq = job.req;
    if (trace)
      std::fprintf(stderr, "[pm_server] worker %d start tag %llu kind %d geo %d root %d refine %d levels %d elem %d\n",
                   index, (unsigned long long)rq.tag, rq.kind, rq.geometry, rq.root_n, rq.n_refine, rq.n_levels,
                   rq.elem);
    pm_result res{};
    res.tag = rq.tag;
    res.worker = index;
    const auto t_start = Clock::now();
    res.queue_ms = ms_since(job.submitted, t_start);
    const SetupKey key{rq.kind, rq.geometry, rq.root_n, rq.n_refine, rq.n_levels, rq.elem};
    int rc = PM_OK;
    Cached* entry = nullptr;
    auto it = cache.find(key);
    if (it != cache.end()) {
      entry = &it->second;
      res.cache_hit = 1;
    } else {
      auto setup = setup_for(key, ctx);
      if (setup->status != PM_OK) {
        rc = setup->status;
      } else {
        // admission: room for the new problem, evicting this worker's least
        // recently used problems first, then waiting for the others
        const int64_t est = setup->footprint > 0 ? setup->footprint.load() : estimate_bytes(setup->disc);
        for (;;) {
          {
            std::lock_guard<std::mutex> lk(led_mu);
            if (committed + est <= cap) break;
          }
          if (cache.empty()) break;
          auto victim = cache.begin();
          for (auto c = cache.begin(); c != cache.end(); ++c)
            if (c->second.last_use < victim->second.last_use) victim = c;
          evict(victim);
        }
        const bool reserved = reserve(est, held);
        if (!reserved) rc = PM_E_OOM;
        const int64_t before = pm::g_thread_dev_bytes;
        pm_problem* p = nullptr;
        if (rc == PM_OK) {
          // the multigrid runs over all levels of the request (a later key wins)
          const std::string prm = (rq.kind == 1 ? params_stokes : params_cd) +
                                  "\nmultigrid_n_levels: " + std::to_string(rq.n_levels) + "\n";
          if (rq.kind == 1) rc = pm_problem_create_stokes(ctx, setup->disc, rq.nu, prm.c_str(), &p);
          else rc = pm_problem_create_cd(ctx, setup->disc, &rq.coeffs, 0, prm.c_str(), &p);
        }
        const int64_t grown = pm::g_thread_dev_bytes - before;
        adjust(grown - (reserved ? est : 0));  // the reservation becomes the measured bytes
        held += grown;
        if (rc == PM_OK) {
          Cached c;
          c.p = p;
          int n = 0, na = 0;
          pm_problem_size(p, &n, &na);
          c.n_dofs = n;
          c.bytes = grown;
          cache[key] = c;
          entry = &cache[key];
        }
      }
    }
    const auto t_setup = Clock::now();
    res.setup_ms = res.cache_hit ? 0.0 : ms_since(t_start, t_setup);
    if (rc == PM_OK && entry) {
      const int64_t before = pm::g_thread_dev_bytes;
      if (rq.kind == 1) {
        // the cached problem serves every viscosity of its set-up: the
        // assembly below takes this request's nu
        entry->p->nu = rq.nu;
        rc = pm_problem_reset_solution(entry->p);
        if (rc == PM_OK) rc = pm_problem_assemble(entry->p);
        if (rc == PM_OK) rc = pm_problem_solve(entry->p);
        if (rc == PM_OK && rq.solution_out) rc = pm_problem_get_solution(entry->p, rq.solution_out);
      } else {
        std::vector<double> scratch;
        double* out = rq.solution_out;
        if (!out) {
          scratch.resize(size_t(entry->n_dofs));
          out = scratch.data();
        }
        rc = pm_problem_run_host(entry->p, &rq.coeffs, nullptr, out);
      }
      // the first solve allocates the solver's work space: it belongs to the problem
      const int64_t grown = pm::g_thread_dev_bytes - before;
      entry->bytes += grown;
      held += grown;
      adjust(grown);
      {
        auto setup = setup_for(key);
        if (setup->footprint < entry->bytes) setup->footprint = entry->bytes;
      }
      entry->last_use = ++tick;
      res.n_dofs = entry->n_dofs;
      if (rc == PM_OK) {
        pm_problem_last_info(entry->p, &res.iterations, &res.residual, &res.initial_residual);
        // IterativeMethod::converged's residual tests (absolute tolerance or
        // reduction of the initial residual); otherwise the iteration cap ended it
        pm_solver* sv = nullptr;
        pm_problem_solver(entry->p, &sv);
        if (sv && !(res.residual <= std::max(sv->tol, sv->reduction * res.initial_residual))) rc = PM_E_MAXIT;
      }
      if (entry->bytes > cap) {
        // this set-up alone does not fit under the cap: it is served, not kept
        evict(cache.find(key));
      }
    }
    res.status = rc;
    const auto t_end = Clock::now();
    if (trace)
      std::fprintf(stderr, "[pm_server] worker %d done tag %llu status %d its %d setup %.1f ms run %.1f ms%s%s\n", index,
                   (unsigned long long)rq.tag, rc, res.iterations, res.setup_ms, ms_since(t_setup, t_end),
                   rc == PM_OK || rc == PM_E_MAXIT ? "" : " error: ", rc == PM_OK || rc == PM_E_MAXIT ? "" : pm_last_error(ctx));
    res.run_ms = ms_since(t_setup, t_end);
    res.latency_ms = ms_since(job.submitted, t_end);
    push_result(res);
  }
  while (!cache.empty()) evict(cache.begin());
  pm_ctx_destroy(ctx);
}

extern "C" {

/* gpu_batch_slots (a key of params_cd, no reference counterpart): requests of
 * one convection-diffusion set-up solved together, up to this many at once (1
 * to 16, default 8; 0 = convection-diffusion requests on the worker pool, one
 * solve at a time per worker). */
int pm_server_create(int device, int n_workers, const char* params_cd, const char* params_stokes,
                     size_t hbm_cap_bytes, pm_server** out) {
  if (!out || n_workers < 1 || n_workers > 64) return PM_E_INVALID;
  auto* s = new pm_server();
  s->device = device;
  s->n_workers = n_workers;
  s->params_cd = params_cd ? params_cd : "";
  s->params_stokes = params_stokes ? params_stokes : "";
  s->cap = hbm_cap_bytes ? int64_t(hbm_cap_bytes) : INT64_MAX;
  try {
    const pm::Params prm = pm::Params::parse(s->params_cd.c_str());
    s->batch_slots = int(prm.integer("gpu_batch_slots", 8));
  } catch (...) {
    delete s;
    return PM_E_INVALID;
  }
  if (s->batch_slots < 0 || s->batch_slots > pm::kMaxBatch) {
    delete s;
    return PM_E_INVALID;
  }
  for (int w = 0; w < n_workers; ++w) s->threads.emplace_back([s, w] { s->worker(w); });
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->workers_ready + s->workers_failed == n_workers; });
  }
  if (s->workers_failed) {
    pm_server_destroy(s);
    return PM_E_CUDA;
  }
  *out = s;
  return PM_OK;
}

void pm_server_destroy(pm_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (auto& kv : s->lanes) kv.second->cv.notify_all();
  }
  s->cv_job.notify_all();
  s->led_cv.notify_all();
  for (auto& t : s->threads) t.join();
  std::vector<std::thread> lane_threads;
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (auto& kv : s->lanes) lane_threads.push_back(std::move(kv.second->th));
  }
  for (auto& t : lane_threads)
    if (t.joinable()) t.join();
  delete s;
}

int pm_server_submit(pm_server* s, const pm_request* req) {
  if (!s || !req) return PM_E_INVALID;
  if (req->kind != 0 && req->kind != 1) return PM_E_INVALID;
  const Job job{*req, Clock::now()};
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->submitted++;
    if (req->kind == 0 && s->batch_slots > 0) {
      const SetupKey key{req->kind, req->geometry, req->root_n, req->n_refine, req->n_levels, req->elem};
      auto& lane = s->lanes[key];
      if (!lane) {
        lane.reset(new Lane());
        lane->srv = s;
        lane->key = key;
        lane->index = int(s->lanes.size()) - 1;
        Lane* l = lane.get();
        lane->th = std::thread([l] { l->run(); });
      }
      lane->pending.push_back(job);
      lane->cv.notify_one();
      return PM_OK;
    }
    s->jobs.push_back(job);
  }
  s->cv_job.notify_one();
  return PM_OK;
}

int pm_server_poll(pm_server* s, pm_result* out, int max_results, int min_results, int* n_out) {
  if (!s || (!out && max_results > 0) || !n_out) return PM_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  if (min_results > 0) {
    const uint64_t pending = s->submitted - (s->completed - s->done.size());
    const size_t want = size_t(std::min<uint64_t>(uint64_t(min_results), pending));
    s->cv_done.wait(lk, [&] { return s->done.size() >= want; });
  }
  int n = 0;
  while (n < max_results && !s->done.empty()) {
    out[n++] = s->done.front();
    s->done.pop_front();
  }
  *n_out = n;
  return PM_OK;
}

int pm_server_drain(pm_server* s) {
  if (!s) return PM_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->completed == s->submitted; });
  return PM_OK;
}

int pm_server_stats(pm_server* s, size_t* cached_bytes, uint64_t* served, uint64_t* evictions) {
  if (!s) return PM_E_INVALID;
  if (cached_bytes) *cached_bytes = size_t(std::max<int64_t>(0, s->committed_view.load()));
  if (served) *served = s->served.load();
  if (evictions) *evictions = s->evictions.load();
  return PM_OK;
}

}  // extern "C"
