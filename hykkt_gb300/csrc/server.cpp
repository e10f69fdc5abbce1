// Served solves: a thread-safe request queue in front of a set of plans.
//
// The reference is single-threaded (one HykktSolver, default stream, no
// locking; src/HykktSolver.cpp:18-34, 240-286).  A solve service needs many
// clients, each with its own sparsity (its own plan), submitting solves
// concurrently.  Here:
//   * any host thread submits a solve of one of its plans with borrowed host
//     buffers (the plan's four value arrays, the four right-hand sides, an
//     optional y0, and the four solution arrays) and gets a ticket;
//   * W worker threads, each with its own CUDA stream, take requests in
//     arrival order.  A plan's device buffers serve one solve at a time, so
//     a worker skips requests whose plan is being solved by another worker:
//     requests of one plan complete in submission order, requests of
//     different plans run concurrently on the GPU (up to W at a time);
//   * the worker runs the plan's numeric solve on its stream, copies the
//     solution into the client's buffers, keeps the plan's info and
//     completes the ticket; the client's wait returns the solve status, the
//     info and the latency (submission to completion, queueing included).
// The plans' persistent solve kernels should be sized for W concurrent
// solves (hykkt_plan_set_concurrency(plan, W)).
//
// Admission by device memory (hykkt_server_create_managed): clients may
// together hold more plans than fit in device memory.  The server keeps the
// device storage of at most `budget` bytes of plans resident:
//   * a request whose plan is resident is taken as above;
//   * otherwise its plan is admitted when its bytes fit beside the resident
//     plans, after evicting idle resident plans if needed (least recently
//     used first, plans without queued requests before plans with some);
//   * a request that cannot be admitted yet is deferred; the oldest deferred
//     request reserves its bytes, so newer requests are admitted only beside
//     that reservation and the oldest one is admitted as soon as enough
//     solves end (no starvation);
//   * a plan larger than the whole budget fails its requests with HYKKT_OOM.
// Heavy requests (hykkt_server_set_heavy): requests of plans whose device
// storage is at least a given size take at most a given number of workers
// at a time; the other workers stay free for the smaller plans, whose
// requests then do not queue behind solves that take a thousand times
// longer.  Heavy requests keep their arrival order among themselves.  While
// such a limit is set the other requests run on a high-priority stream, so
// that their kernels' blocks are scheduled ahead of the heavy solves'.
// Eviction releases a plan's device storage and keeps its host analysis;
// its next admission allocates it again.  The worker that takes a request
// does the evictions and the allocation outside the queue's lock, with the
// plans involved marked busy.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "hykkt_gb300.h"

namespace hykkt {
void set_last_error(const std::string& msg);  // capi.cpp
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  hykkt_plan_t plan = nullptr;
  const double* in[9] = {};  // h, ds, jc, jd, rx, rs, ry, ryd, y0
  double* out[4] = {};       // x, s, y, yd
  int status = HYKKT_NOT_READY;
  bool done = false;
  bool claimed = false;  // a client is waiting for (or has collected) this ticket
  bool deferred = false; // counted once as deferred by a managed server
  bool heavy = false;    // counted in the server's heavy requests in flight
  std::string error;
  hykkt_info info{};
  Clock::time_point t_submit, t_taken, t_loaded, t_done;  // t_taken: a worker took it; t_loaded: admitted
};

// residency bookkeeping of one plan (managed servers)
struct PlanMem {
  int64_t bytes = -1;   // device storage when resident (-1: not asked yet)
  bool resident = false;
  int pending = 0;      // queued requests
  int64_t last_use = 0; // tick of the last completion (LRU)
};

// what a worker does for one request outside the lock
struct Work {
  Request* r = nullptr;
  std::vector<hykkt_plan_t> evict;  // idle plans to release first
  int64_t evict_bytes = 0;
  bool load = false;                // allocate r's plan before solving
  bool oom = false;                 // r's plan exceeds the budget: fail it
  bool urgent = false;              // a light request under a heavy limit: high-priority stream
};

}  // namespace

struct hykkt_server_s {
  std::mutex mu;
  std::condition_variable cv_work;  // a request arrived, a plan became free, or stopping
  std::condition_variable cv_done;  // a request completed
  std::deque<Request*> queue;       // arrival order
  std::unordered_map<int64_t, Request*> live;  // submitted and not yet waited for
  std::unordered_set<hykkt_plan_t> busy;       // plans being solved
  std::vector<std::thread> workers;
  hykkt_serve_fn fn = nullptr;
  void* user = nullptr;
  int device = 0;
  bool stopping = false;
  int64_t next_ticket = 1;
  int64_t completed = 0;
  int in_flight = 0;
  int waiters = 0;  // clients inside hykkt_server_wait
  // admission by device memory
  bool managed = false;
  hykkt_server_memory mem{};
  int64_t budget = 0, used = 0, tick = 0;
  int64_t evicting = 0;  // bytes chosen for release whose release has not finished (still held)
  int64_t loading = 0;   // bytes admitted whose allocation has not happened yet (not held)
  int64_t admissions = 0, evictions = 0, deferrals = 0, peak_used = 0;
  std::unordered_map<hykkt_plan_t, PlanMem> pm;
  // heavy requests (0: no limit)
  int64_t heavy_bytes = 0;
  int max_heavy = 0, heavy_in_flight = 0;
  std::unordered_map<hykkt_plan_t, int64_t> sizes;  // plan bytes, asked once

  bool is_heavy(hykkt_plan_t p) {  // caller holds mu
    if (heavy_bytes <= 0) return false;
    auto it = sizes.find(p);
    if (it == sizes.end()) it = sizes.emplace(p, plan_bytes(p)).first;
    return it->second >= heavy_bytes;
  }

  int64_t plan_bytes(hykkt_plan_t p) {
    if (mem.bytes_fn) return mem.bytes_fn(mem.user, p);
    int res = 0;
    int64_t b = 0;
    if (hykkt_plan_residency(p, &res, &b) != HYKKT_OK) return -1;
    return b;
  }
  PlanMem& state(hykkt_plan_t p) {  // caller holds mu
    PlanMem& m = pm[p];
    if (m.bytes < 0) {
      m.bytes = plan_bytes(p);
      int res = 0;
      if (mem.resident_fn) res = mem.resident_fn(mem.user, p);
      else if (!fn) hykkt_plan_residency(p, &res, nullptr);
      m.resident = res != 0;
      if (m.resident) used += m.bytes;  // a plan that arrived resident counts from the start
      peak_used = std::max(peak_used, used);
    }
    return m;
  }

  // Idle resident plans to evict so that `need` more bytes fit beside
  // `reserve` (caller holds mu); empty when even all of them are not enough.
  std::vector<hykkt_plan_t> victims(int64_t need, int64_t reserve) {
    std::vector<std::pair<std::pair<int, int64_t>, hykkt_plan_t>> idle;
    for (auto& kv : pm)
      if (kv.second.resident && !busy.count(kv.first))
        idle.push_back({{kv.second.pending > 0 ? 1 : 0, kv.second.last_use}, kv.first});
    std::sort(idle.begin(), idle.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<hykkt_plan_t> out;
    int64_t freed = 0;
    const int64_t held = used + evicting;  // other workers' releases may still be running
    for (auto& e : idle) {
      if (held - freed + need + reserve <= budget) break;
      out.push_back(e.second);
      freed += pm[e.second].bytes;
    }
    if (held - freed + need + reserve > budget) out.clear();
    return out;
  }

  // the first request that can run now (caller holds mu); w is left empty
  // unless a request is returned
  bool take(Work& out) {
    out = Work{};
    int64_t reserve = 0;  // bytes claimed by the oldest deferred request
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      Request* r = *it;
      if (busy.count(r->plan)) continue;
      const bool heavy = is_heavy(r->plan);
      if (heavy && heavy_in_flight >= max_heavy) continue;
      Work w;
      w.r = r;
      if (managed) {
        PlanMem& m = state(r->plan);
        if (m.bytes < 0 || m.bytes > budget) {
          w.oom = true;  // can never fit: fail it now
        } else if (!m.resident) {
          if (used + evicting + m.bytes + reserve > budget) {
            w.evict = victims(m.bytes, reserve);
            if (w.evict.empty()) {
              if (reserve == 0) reserve = m.bytes;
              if (!r->deferred) {
                r->deferred = true;
                ++deferrals;
              }
              continue;
            }
            for (hykkt_plan_t v : w.evict) {
              PlanMem& vm = pm[v];
              vm.resident = false;
              used -= vm.bytes;
              evicting += vm.bytes;  // held until this worker has released it
              w.evict_bytes += vm.bytes;
              busy.insert(v);  // nobody takes a plan while it is being released
              ++evictions;
            }
          }
          m.resident = true;
          used += m.bytes;
          loading += m.bytes;
          w.load = true;
          ++admissions;
        }
      }
      queue.erase(it);
      busy.insert(r->plan);
      ++in_flight;
      r->heavy = heavy;
      r->t_taken = Clock::now();
      if (heavy) ++heavy_in_flight;
      w.urgent = heavy_bytes > 0 && !heavy;
      out = std::move(w);
      return true;
    }
    return false;
  }

  void run(int w) {
    cudaStream_t st = nullptr, st_hi = nullptr;
    if (!fn) {
      cudaSetDevice(device);
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
      int least = 0, greatest = 0;
      cudaDeviceGetStreamPriorityRange(&least, &greatest);
      cudaStreamCreateWithPriority(&st_hi, cudaStreamNonBlocking, greatest);
    }
    for (;;) {
      Request* r = nullptr;
      Work wk;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return take(wk) || (stopping && queue.empty()); });
        if (!wk.r) break;
        r = wk.r;
      }
      int rc = HYKKT_OK;
      std::string err;
      hykkt_info info{};
      if (!wk.evict.empty()) {
        for (hykkt_plan_t v : wk.evict) {
          if (mem.evict_fn) mem.evict_fn(mem.user, v);
          else hykkt_plan_release_device(v);
        }
        {
          std::lock_guard<std::mutex> lk(mu);
          for (hykkt_plan_t v : wk.evict) busy.erase(v);
          evicting -= wk.evict_bytes;
        }
        cv_work.notify_all();
      }
      if (wk.oom) {
        rc = HYKKT_OOM;
        hykkt::set_last_error("the plan's device storage exceeds the server's memory budget");
      } else if (wk.load) {
        rc = mem.load_fn ? mem.load_fn(mem.user, r->plan) : hykkt_plan_reload_device(r->plan);
        std::lock_guard<std::mutex> lk(mu);
        PlanMem& m = pm[r->plan];
        loading -= m.bytes;
        if (rc != HYKKT_OK) {
          m.resident = false;
          used -= m.bytes;
        }
        // device memory held now: resident plans and unfinished releases
        peak_used = std::max(peak_used, used + evicting - loading);
      }
      r->t_loaded = Clock::now();
      if (rc != HYKKT_OK) {
      } else if (fn) {
        rc = fn(user, r->plan, w, r->in, r->out);
      } else {
        // light requests under a heavy limit run on the high-priority stream:
        // the GPU schedules their kernels' blocks ahead of the pending blocks
        // of heavy solves, whose factorization kernels fill every SM
        cudaStream_t use = wk.urgent && st_hi ? st_hi : st;
        rc = hykkt_plan_solve(r->plan, r->in[0], r->in[1], r->in[2], r->in[3], r->in[4], r->in[5], r->in[6],
                              r->in[7], r->in[8], 0, use, 1);
        if (rc == HYKKT_OK || rc == HYKKT_CG_NOT_CONVERGED || rc == HYKKT_NOT_SPD || rc == HYKKT_ACCURACY_NOT_MET) {
          const int rs = hykkt_plan_get_solution(r->plan, r->out[0], r->out[1], r->out[2], r->out[3], 0, use);
          if (rs != HYKKT_OK) rc = rs;
          hykkt_plan_get_info(r->plan, &info);
        }
      }
      if (rc != HYKKT_OK) err = hykkt_last_error();
      {
        std::lock_guard<std::mutex> lk(mu);
        r->status = rc;
        r->error = err;
        r->info = info;
        r->t_done = Clock::now();
        r->done = true;
        busy.erase(r->plan);
        --in_flight;
        if (r->heavy) --heavy_in_flight;
        ++completed;
        if (managed) {
          PlanMem& m = pm[r->plan];
          m.pending -= 1;
          m.last_use = ++tick;
        }
      }
      cv_done.notify_all();
      cv_work.notify_all();  // the plan is free again
    }
    if (st) cudaStreamDestroy(st);
    if (st_hi) cudaStreamDestroy(st_hi);
  }
};

extern "C" int hykkt_server_set_heavy(hykkt_server_t s, int64_t heavy_bytes, int max_heavy) {
  if (!s) return HYKKT_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (heavy_bytes > 0) {
    if (max_heavy < 1 || max_heavy > (int)s->workers.size()) {
      hykkt::set_last_error("max_heavy must be in 1..workers");
      return HYKKT_INVALID;
    }
    if (s->fn && !(s->managed && s->mem.bytes_fn)) {
      hykkt::set_last_error("a stand-in solve function needs the bytes hook of a managed server for heavy requests");
      return HYKKT_INVALID;
    }
  }
  s->heavy_bytes = heavy_bytes > 0 ? heavy_bytes : 0;
  s->max_heavy = heavy_bytes > 0 ? max_heavy : 0;
  s->cv_work.notify_all();  // a raised limit may let a waiting request run
  return HYKKT_OK;
}

extern "C" int hykkt_server_create_managed(int workers, hykkt_serve_fn fn, void* user,
                                           const hykkt_server_memory* mem, hykkt_server_t* out) {
  if (!out) return HYKKT_INVALID;
  *out = nullptr;
  if (workers < 1 || workers > 256) {
    hykkt::set_last_error("server workers must be in 1..256");
    return HYKKT_INVALID;
  }
  if (mem && mem->budget_bytes < 0) {
    hykkt::set_last_error("memory budget must be >= 0");
    return HYKKT_INVALID;
  }
  if (mem && fn && (!mem->bytes_fn || !mem->load_fn || !mem->evict_fn)) {
    hykkt::set_last_error("a stand-in solve function needs the bytes, load and evict hooks");
    return HYKKT_INVALID;
  }
  auto* s = new hykkt_server_s();
  s->fn = fn;
  s->user = user;
  if (!fn && cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    hykkt::set_last_error("no CUDA device for the server's streams");
    return HYKKT_CUDA_ERROR;
  }
  if (mem) {
    s->managed = true;
    s->mem = *mem;
    s->budget = mem->budget_bytes;
    if (s->budget == 0) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        delete s;
        hykkt::set_last_error("cudaMemGetInfo failed: pass an explicit memory budget");
        return HYKKT_CUDA_ERROR;
      }
      s->budget = (int64_t)(0.9 * (double)free_b);
    }
  }
  for (int w = 0; w < workers; ++w) s->workers.emplace_back([s, w] { s->run(w); });
  *out = s;
  return HYKKT_OK;
}

extern "C" int hykkt_server_create_ex(int workers, hykkt_serve_fn fn, void* user, hykkt_server_t* out) {
  return hykkt_server_create_managed(workers, fn, user, nullptr, out);
}

extern "C" int hykkt_server_create(int workers, hykkt_server_t* out) {
  return hykkt_server_create_managed(workers, nullptr, nullptr, nullptr, out);
}

extern "C" int hykkt_server_memory_stats(hykkt_server_t s, int64_t* budget, int64_t* resident_bytes,
                                         int64_t* peak_bytes, int64_t* resident_plans, int64_t* admissions,
                                         int64_t* evictions, int64_t* deferrals) {
  if (!s) return HYKKT_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  int64_t n = 0;
  for (auto& kv : s->pm) n += kv.second.resident ? 1 : 0;
  if (budget) *budget = s->budget;
  if (resident_bytes) *resident_bytes = s->used;
  if (peak_bytes) *peak_bytes = s->peak_used;
  if (resident_plans) *resident_plans = n;
  if (admissions) *admissions = s->admissions;
  if (evictions) *evictions = s->evictions;
  if (deferrals) *deferrals = s->deferrals;
  return HYKKT_OK;
}

extern "C" int hykkt_server_submit(hykkt_server_t s, hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                                   const double* jc_vals, const double* jd_vals, const double* rx, const double* rs,
                                   const double* ry, const double* ryd, const double* y0, double* x, double* ds,
                                   double* y, double* yd, int64_t* ticket) {
  if (!s || !plan || !ticket) {
    hykkt::set_last_error("server, plan and ticket must not be NULL");
    return HYKKT_INVALID;
  }
  auto* r = new Request();
  r->plan = plan;
  const double* in[9] = {h_vals, ds_vals, jc_vals, jd_vals, rx, rs, ry, ryd, y0};
  double* outp[4] = {x, ds, y, yd};
  std::memcpy(r->in, in, sizeof(in));
  std::memcpy(r->out, outp, sizeof(outp));
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
      delete r;
      hykkt::set_last_error("server is shutting down");
      return HYKKT_INVALID;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    if (s->managed) s->state(plan).pending += 1;
    s->queue.push_back(r);
    s->live[r->ticket] = r;
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return HYKKT_OK;
}

extern "C" int hykkt_server_cancel(hykkt_server_t s, int64_t ticket, int* cancelled) {
  if (!s || !cancelled) return HYKKT_INVALID;
  *cancelled = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) {
      hykkt::set_last_error("unknown or already collected ticket");
      return HYKKT_INVALID;
    }
    Request* r = it->second;
    auto q = std::find(s->queue.begin(), s->queue.end(), r);
    if (q == s->queue.end()) return HYKKT_OK;  // taken by a worker, or done
    s->queue.erase(q);
    if (s->managed) s->state(r->plan).pending -= 1;
    r->status = HYKKT_CANCELLED;
    r->error = "the request was cancelled before a worker took it";
    r->t_taken = r->t_loaded = r->t_done = Clock::now();
    r->done = true;
    *cancelled = 1;
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // a deferred request's reservation may have gone with it
  return HYKKT_OK;
}

extern "C" int hykkt_server_wait(hykkt_server_t s, int64_t ticket, int* solve_status, double* latency_ms,
                                 hykkt_info* info) {
  return hykkt_server_wait_phases(s, ticket, solve_status, latency_ms, info, nullptr);
}

extern "C" int hykkt_server_wait_phases(hykkt_server_t s, int64_t ticket, int* solve_status, double* latency_ms,
                                        hykkt_info* info, double* phases_ms) {
  if (!s) return HYKKT_INVALID;
  Request* r = nullptr;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) {
      hykkt::set_last_error("unknown or already collected ticket");
      return HYKKT_INVALID;
    }
    r = it->second;
    if (r->claimed) {
      hykkt::set_last_error("another thread is already waiting for this ticket");
      return HYKKT_INVALID;
    }
    // claimed under the lock: a second waiter is turned away above, and the
    // request stays alive until this thread deletes it below
    r->claimed = true;
    ++s->waiters;
    s->cv_done.wait(lk, [&] { return r->done; });
    s->live.erase(ticket);  // by key: submits may have rehashed the map meanwhile
    --s->waiters;
    s->cv_done.notify_all();  // under the lock: destroy may be waiting for the waiters to leave
  }
  if (solve_status) *solve_status = r->status;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (phases_ms) {
    using ms = std::chrono::duration<double, std::milli>;
    phases_ms[0] = ms(r->t_taken - r->t_submit).count();
    phases_ms[1] = ms(r->t_loaded - r->t_taken).count();
    phases_ms[2] = ms(r->t_done - r->t_loaded).count();
  }
  if (info) *info = r->info;
  if (r->status != HYKKT_OK) hykkt::set_last_error(r->error);
  delete r;
  return HYKKT_OK;
}

extern "C" int hykkt_server_poll(hykkt_server_t s, int64_t ticket, int* done) {
  if (!s || !done) return HYKKT_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) {
    hykkt::set_last_error("unknown or already collected ticket");
    return HYKKT_INVALID;
  }
  *done = it->second->done ? 1 : 0;
  return HYKKT_OK;
}

extern "C" int hykkt_server_stats(hykkt_server_t s, int64_t* completed, int64_t* queued, int64_t* in_flight) {
  if (!s) return HYKKT_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (queued) *queued = (int64_t)s->queue.size();
  if (in_flight) *in_flight = s->in_flight;
  return HYKKT_OK;
}

extern "C" int hykkt_server_destroy(hykkt_server_t s) {
  if (!s) return HYKKT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;  // workers finish the queued requests, then exit
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  {
    // every request is complete now; let the clients still inside a wait
    // collect theirs before the server goes away
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->waiters == 0; });
  }
  for (auto& kv : s->live) delete kv.second;  // completed but never waited for
  delete s;
  return HYKKT_OK;
}
