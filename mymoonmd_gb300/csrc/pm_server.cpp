// Request executor behind pm_server_* (no reference counterpart): the batched
// stream of independent solves and the serving loop.
//
// n worker threads, each with its own pm_ctx (one CUDA stream), take requests
// first in first out. A worker keeps the device-resident problem of every
// set-up it has served (keyed by kind, geometry, mesh size, levels and
// element) and reuses it: a request with a known set-up costs one device
// assembly of all levels with the new coefficients, the solve, and the copy of
// the solution. The host set-ups (mesh hierarchies, numbering, structures,
// transfer) are built once and shared by all workers. The device footprint of
// the cached problems is measured by the DBuf accounting of the worker thread
// that owns them and kept under the cap by evicting least recently used
// problems of the worker that needs room (other workers' problems are never
// touched from another thread).
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

}  // namespace

struct pm_server {
  int device = 0;
  std::string params_cd, params_stokes;
  int64_t cap = 0;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  std::deque<Job> jobs;
  std::deque<pm_result> done;
  uint64_t submitted = 0, completed = 0;
  bool stop = false;
  std::mutex setup_mu;
  std::map<SetupKey, std::shared_ptr<SharedSetup>> setups;
  std::atomic<int64_t> cached_bytes{0};
  std::atomic<uint64_t> served{0}, evictions{0};
  std::string create_error;
  std::atomic<int> workers_ready{0}, workers_failed{0};
  bool trace = std::getenv("PMGPU_SERVER_TRACE") != nullptr;  // request start/finish lines on stderr

  std::shared_ptr<SharedSetup> setup_for(const SetupKey& k) {
    std::shared_ptr<SharedSetup> s;
    {
      std::lock_guard<std::mutex> g(setup_mu);
      auto& slot = setups[k];
      if (!slot) slot = std::make_shared<SharedSetup>();
      s = slot;
    }
    std::lock_guard<std::mutex> g(s->mu);
    if (s->status < 0) {
      s->status = pm_disc_create(k.geometry, k.root_n, k.n_refine, k.n_levels, k.kind, k.elem, &s->disc);
      if (s->status != PM_OK) s->error = pm_last_error(nullptr);
    }
    return s;
  }

  void worker(int index);
};

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
  for (;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_job.wait(lk, [&] { return stop || !jobs.empty(); });
      if (stop && jobs.empty()) break;
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
      auto setup = setup_for(key);
      if (setup->status != PM_OK) {
        rc = setup->status;
      } else {
        const int64_t before = pm::g_thread_dev_bytes;
        pm_problem* p = nullptr;
        // the multigrid runs over all levels of the request (a later key wins)
        const std::string prm = (rq.kind == 1 ? params_stokes : params_cd) +
                                "\nmultigrid_n_levels: " + std::to_string(rq.n_levels) + "\n";
        if (rq.kind == 1) rc = pm_problem_create_stokes(ctx, setup->disc, rq.nu, prm.c_str(), &p);
        else rc = pm_problem_create_cd(ctx, setup->disc, &rq.coeffs, 0, prm.c_str(), &p);
        if (rc == PM_OK) {
          Cached c;
          c.p = p;
          int n = 0, na = 0;
          pm_problem_size(p, &n, &na);
          c.n_dofs = n;
          c.bytes = pm::g_thread_dev_bytes - before;
          cache[key] = c;
          entry = &cache[key];
          cached_bytes += c.bytes;
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
      cached_bytes += grown;
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
      // admission cap: evict this worker's least recently used problems
      while (cached_bytes.load() > cap && cache.size() > 1) {
        auto victim = cache.end();
        for (auto c = cache.begin(); c != cache.end(); ++c)
          if (&c->second != entry && (victim == cache.end() || c->second.last_use < victim->second.last_use))
            victim = c;
        if (victim == cache.end()) break;
        cached_bytes -= victim->second.bytes;
        pm_problem_destroy(victim->second.p);
        cache.erase(victim);
        evictions++;
      }
      if (entry->bytes > cap) {
        // this set-up alone does not fit under the cap: it is served, not kept
        cached_bytes -= entry->bytes;
        pm_problem_destroy(entry->p);
        cache.erase(key);
        evictions++;
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
    served++;
    {
      std::lock_guard<std::mutex> g(mu);
      done.push_back(res);
      completed++;
    }
    cv_done.notify_all();
  }
  for (auto& kv : cache) {
    cached_bytes -= kv.second.bytes;
    pm_problem_destroy(kv.second.p);
  }
  cache.clear();
  pm_ctx_destroy(ctx);
}

extern "C" {

int pm_server_create(int device, int n_workers, const char* params_cd, const char* params_stokes,
                     size_t hbm_cap_bytes, pm_server** out) {
  if (!out || n_workers < 1 || n_workers > 64) return PM_E_INVALID;
  auto* s = new pm_server();
  s->device = device;
  s->params_cd = params_cd ? params_cd : "";
  s->params_stokes = params_stokes ? params_stokes : "";
  s->cap = hbm_cap_bytes ? int64_t(hbm_cap_bytes) : INT64_MAX;
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
  }
  s->cv_job.notify_all();
  for (auto& t : s->threads) t.join();
  delete s;
}

int pm_server_submit(pm_server* s, const pm_request* req) {
  if (!s || !req) return PM_E_INVALID;
  if (req->kind != 0 && req->kind != 1) return PM_E_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->jobs.push_back(Job{*req, Clock::now()});
    s->submitted++;
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
  if (cached_bytes) *cached_bytes = size_t(std::max<int64_t>(0, s->cached_bytes.load()));
  if (served) *served = s->served.load();
  if (evictions) *evictions = s->evictions.load();
  return PM_OK;
}

}  // extern "C"
