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
#include <cuda_runtime.h>

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
  std::string error;
  hykkt_info info{};
  Clock::time_point t_submit, t_done;
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

  // the first request whose plan is free (caller holds mu)
  Request* take() {
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      if (busy.count((*it)->plan)) continue;
      Request* r = *it;
      queue.erase(it);
      busy.insert(r->plan);
      ++in_flight;
      return r;
    }
    return nullptr;
  }

  void run(int w) {
    cudaStream_t st = nullptr;
    if (!fn) {
      cudaSetDevice(device);
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    }
    for (;;) {
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return (r = take()) != nullptr || (stopping && queue.empty()); });
        if (!r) break;
      }
      int rc;
      std::string err;
      hykkt_info info{};
      if (fn) {
        rc = fn(user, r->plan, w, r->in, r->out);
      } else {
        rc = hykkt_plan_solve(r->plan, r->in[0], r->in[1], r->in[2], r->in[3], r->in[4], r->in[5], r->in[6],
                              r->in[7], r->in[8], 0, st, 1);
        if (rc == HYKKT_OK || rc == HYKKT_CG_NOT_CONVERGED || rc == HYKKT_NOT_SPD || rc == HYKKT_ACCURACY_NOT_MET) {
          const int rs = hykkt_plan_get_solution(r->plan, r->out[0], r->out[1], r->out[2], r->out[3], 0, st);
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
        ++completed;
      }
      cv_done.notify_all();
      cv_work.notify_all();  // the plan is free again
    }
    if (st) cudaStreamDestroy(st);
  }
};

extern "C" int hykkt_server_create_ex(int workers, hykkt_serve_fn fn, void* user, hykkt_server_t* out) {
  if (!out) return HYKKT_INVALID;
  *out = nullptr;
  if (workers < 1 || workers > 256) {
    hykkt::set_last_error("server workers must be in 1..256");
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
  for (int w = 0; w < workers; ++w) s->workers.emplace_back([s, w] { s->run(w); });
  *out = s;
  return HYKKT_OK;
}

extern "C" int hykkt_server_create(int workers, hykkt_server_t* out) {
  return hykkt_server_create_ex(workers, nullptr, nullptr, out);
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
    s->queue.push_back(r);
    s->live[r->ticket] = r;
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return HYKKT_OK;
}

extern "C" int hykkt_server_wait(hykkt_server_t s, int64_t ticket, int* solve_status, double* latency_ms,
                                 hykkt_info* info) {
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
