// extern "C" boundary of hykkt_gb300 (declared in include/hykkt_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include "MMatrix.hpp"
#include "components.hpp"
#include "engine.hpp"
#include "hykkt_gb300.h"
#include "input_functions.hpp"
#include "symbolic.hpp"

using namespace hykkt;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc& e) {
    return fail(HYKKT_OOM, std::string("out of memory: ") + e.what());
  } catch (const std::exception& e) {
    std::string m = e.what();
    if (m.find("out of memory") != std::string::npos) return fail(HYKKT_OOM, m);
    if (m.rfind("CUDA:", 0) == 0) return fail(HYKKT_CUDA_ERROR, m);
    return fail(HYKKT_INVALID, m);
  } catch (...) {
    return fail(HYKKT_INVALID, "unknown error");
  }
}

// A solve's status, with the message hykkt_last_error gives for it.
int solve_status(int st) {
  switch (st) {
    case HYKKT_OK: return st;
    case HYKKT_NOT_SPD: return fail(st, "the factorization met a pivot <= 1e-12 (matrix not positive definite)");
    case HYKKT_CG_NOT_CONVERGED: return fail(st, "the Schur-complement CG used its whole iteration budget");
    case HYKKT_TIMEOUT: return fail(st, "a wait of the triangular solves gave up (results invalid)");
    case HYKKT_ACCURACY_NOT_MET: return fail(st, "refinement ended above the requested residual target");
    default: return fail(st, "solve failed");
  }
}

CsrPattern make_pattern(int n, int m, const int* rp, const int* ci, int nnz) {
  CsrPattern p;
  p.n = n;
  p.m = m;
  if (n < 0 || m < 0 || nnz < 0) throw std::runtime_error("negative size");
  if (n > 0 && !rp) throw std::runtime_error("missing row pointers");
  if (nnz > 0 && !ci) throw std::runtime_error("missing column indices");
  p.rp.assign(rp ? rp : nullptr, rp ? rp + n + 1 : nullptr);
  if (!rp) p.rp.assign(n + 1, 0);
  if (p.rp[n] != nnz) throw std::runtime_error("row pointer end does not match nnz");
  p.ci.assign(ci ? ci : nullptr, ci ? ci + nnz : nullptr);
  return p;
}

void fill_info(const Engine& e, hykkt_info* info) {
  const Symbolic& S = e.sym();
  const DevScalars sc = e.last_scalars();
  std::memset(info, 0, sizeof(*info));
  info->status = e.last_status();
  info->cg_iterations = sc.it;
  info->pivot_col = sc.pivot_col == INT_MAX ? -1 : sc.pivot_col;
  info->ordering = S.ordering_used;
  info->cg_residual = sc.cg_err;
  info->rel_residual = sc.rel_res_ref;
  info->rel_residual_full = sc.rel_res_full;
  info->nnz_L = S.nnz_L;
  info->L_stored = S.L_stored;
  info->factor_flops = S.factor_flops;
  info->device_bytes = e.device_bytes();
  info->n_supernodes = S.nsn;
  info->n_levels = S.nlevels;
  info->n_solve_levels = S.nsq_levels;
  info->kernels_per_solve = e.kernels_per_solve();
  info->kernels_per_cg_iteration = e.kernels_per_iter();
  info->cg_iterations_total = sc.it_total;
  info->refine_steps = sc.refine_it;
  info->rel_residual_first = sc.rel_res_first;
  info->kernels_per_refine_step = e.kernels_per_refine();
}

SymbolicOptions default_options(int ordering) {
  SymbolicOptions o;
  o.ordering = ordering;
  // tuning override: multiply-adds per triangular-solve product task
  if (const char* e = std::getenv("HYKKT_SOLVE_CHUNK_FMA")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v >= 1024 && v <= (1 << 20)) o.chunk_fma = (int)v;
  }
  // tuning override: columns per unit of a wide item's panel product
  if (const char* e = std::getenv("HYKKT_SOLVE_UNIT_COLS")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v >= 64 && v <= kMaxUnitCols) o.unit_cols = (int)v;
  }
  // tuning override: most items of one warp-subtree task (0 or 1: none)
  if (const char* e = std::getenv("HYKKT_SOLVE_WARP_SUBTREE")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v >= 0 && v <= kMaxSubtree) o.warp_subtree = (int)v;
  }
  return o;
}

// The solve_piece option selects the throughput layout of the solve items:
// pieces, and warp items one per warp rather than in subtree tasks (a
// subtree task shortens one solve's critical path but holds a CTA with
// mostly idle warps, which costs throughput when plans share the GPU).
void apply_solve_piece(SymbolicOptions& o, int solve_piece) {
  if (solve_piece <= 0) return;
  o.solve_piece = solve_piece;
  if (!std::getenv("HYKKT_SOLVE_WARP_SUBTREE")) o.warp_subtree = 0;
}
}  // namespace

extern "C" const char* hykkt_last_error(void) { return g_err.c_str(); }

namespace hykkt {
// the message hykkt_last_error returns on the calling thread (server.cpp)
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace hykkt
extern "C" const char* hykkt_version(void) { return "hykkt_gb300 0.1 (sm_103a, FP64)"; }

// ===========================================================================
// Plan API
// ===========================================================================
struct hykkt_plan_s {
  std::unique_ptr<Engine> eng;
  cudaStream_t stream = nullptr;
  ~hykkt_plan_s() {
    eng.reset();
    if (stream) cudaStreamDestroy(stream);
  }
  cudaStream_t pick(void* s) {
    if (s) return (cudaStream_t)s;
    if (!stream) HYKKT_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    return stream;
  }
};

static int plan_create(hykkt_plan_t* plan, int n_x, int m_c, int m_d, const int* h_rowptr, const int* h_colidx,
                       int nnz_h, const int* ds_rowptr, const int* ds_colidx, int nnz_ds, const int* jc_rowptr,
                       const int* jc_colidx, int nnz_jc, const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                       double gamma, int ordering, const int* perm, int solve_piece, bool deferred) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "plan pointer is NULL");
    *plan = nullptr;
    if (solve_piece < 0) return fail(HYKKT_INVALID, "solve_piece must be >= 0");
    CsrPattern H = make_pattern(n_x, n_x, h_rowptr, h_colidx, nnz_h);
    CsrPattern Ds = make_pattern(m_d, m_d, ds_rowptr, ds_colidx, nnz_ds);
    CsrPattern Jc = make_pattern(m_c, n_x, jc_rowptr, jc_colidx, nnz_jc);
    CsrPattern Jd = make_pattern(m_d, n_x, jd_rowptr, jd_colidx, nnz_jd);
    SymbolicOptions opt = default_options(ordering);
    apply_solve_piece(opt, solve_piece);
    Symbolic S = build_symbolic(H, Ds, Jc, Jd, opt, perm);
    auto p = std::make_unique<hykkt_plan_s>();
    p->eng = std::make_unique<Engine>(std::move(S), gamma, opt, deferred);
    *plan = p.release();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_create_ex(hykkt_plan_t* plan, int n_x, int m_c, int m_d, const int* h_rowptr,
                                    const int* h_colidx, int nnz_h, const int* ds_rowptr, const int* ds_colidx,
                                    int nnz_ds, const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                                    const int* jd_rowptr, const int* jd_colidx, int nnz_jd, double gamma,
                                    int ordering, const int* perm, int solve_piece) {
  return plan_create(plan, n_x, m_c, m_d, h_rowptr, h_colidx, nnz_h, ds_rowptr, ds_colidx, nnz_ds, jc_rowptr,
                     jc_colidx, nnz_jc, jd_rowptr, jd_colidx, nnz_jd, gamma, ordering, perm, solve_piece, false);
}

extern "C" int hykkt_plan_create_deferred(hykkt_plan_t* plan, int n_x, int m_c, int m_d, const int* h_rowptr,
                                          const int* h_colidx, int nnz_h, const int* ds_rowptr,
                                          const int* ds_colidx, int nnz_ds, const int* jc_rowptr,
                                          const int* jc_colidx, int nnz_jc, const int* jd_rowptr,
                                          const int* jd_colidx, int nnz_jd, double gamma, int ordering,
                                          const int* perm, int solve_piece) {
  return plan_create(plan, n_x, m_c, m_d, h_rowptr, h_colidx, nnz_h, ds_rowptr, ds_colidx, nnz_ds, jc_rowptr,
                     jc_colidx, nnz_jc, jd_rowptr, jd_colidx, nnz_jd, gamma, ordering, perm, solve_piece, true);
}

extern "C" int hykkt_plan_release_device(hykkt_plan_t plan) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    if (plan->stream) HYKKT_CUDA(cudaStreamSynchronize(plan->stream));
    plan->eng->release_device();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_reload_device(hykkt_plan_t plan) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    plan->eng->reload_device();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_residency(hykkt_plan_t plan, int* resident, int64_t* bytes) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    if (resident) *resident = plan->eng->resident() ? 1 : 0;
    if (bytes) *bytes = plan->eng->size_bytes();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_create(hykkt_plan_t* plan, int n_x, int m_c, int m_d, const int* h_rowptr,
                                 const int* h_colidx, int nnz_h, const int* ds_rowptr, const int* ds_colidx,
                                 int nnz_ds, const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                                 const int* jd_rowptr, const int* jd_colidx, int nnz_jd, double gamma,
                                 int ordering, const int* perm) {
  return hykkt_plan_create_ex(plan, n_x, m_c, m_d, h_rowptr, h_colidx, nnz_h, ds_rowptr, ds_colidx, nnz_ds,
                              jc_rowptr, jc_colidx, nnz_jc, jd_rowptr, jd_colidx, nnz_jd, gamma, ordering, perm, 0);
}

extern "C" void hykkt_plan_destroy(hykkt_plan_t plan) { delete plan; }

extern "C" int hykkt_plan_clone(hykkt_plan_t src, hykkt_plan_t* plan) {
  return guarded([&]() {
    if (!src || !plan) return fail(HYKKT_INVALID, "NULL plan");
    *plan = nullptr;
    const Engine& e = *src->eng;
    auto p = std::make_unique<hykkt_plan_s>();
    p->eng = std::make_unique<Engine>(Symbolic(e.sym()), e.gamma(), e.options());
    int itmax, refine_max;
    double rtol, target;
    e.accuracy(itmax, rtol, refine_max, target);
    p->eng->set_accuracy(itmax, rtol, refine_max, target);
    p->eng->set_refine_rtol(e.refine_rtol());
    p->eng->set_concurrency(e.concurrency());
    p->eng->set_delta(e.delta());
    *plan = p.release();
    return HYKKT_OK;
  });
}

// ===========================================================================
// Autotuner of the triangular-solve layout (no counterpart in the reference,
// which leaves the factor and its solves to cuSOLVER).  The layout of the
// solve items decides the solve's critical path and its FP64 work: whole
// supernodes (shortest dependency chain, most inversion work) or pieces of
// the widest supernodes (less inversion work per factorization, more solve
// stages), with or without warp-subtree tasks, and the multiply-adds of one
// product task.  Which is fastest depends on the pattern and on how many
// plans share the GPU, so the tuner measures: every candidate layout is
// built from the plan's own patterns and ordering (no second ordering),
// `share` engines of it (as many as free device memory allows) solve the
// caller's sample system at once, and the candidate with the highest
// throughput replaces the plan's engine.  The choice is stored per pattern
// and share in a text cache file, so later plans of the pattern take it
// without timing.
// ===========================================================================
namespace {

std::mutex g_tune_mu;  // one tuning at a time per process (it fills the GPU)

uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

uint64_t pattern_key(const Symbolic& S) {
  uint64_t h = 1469598103934665603ull;
  const int dims[4] = {S.n_x, S.m_c, S.m_d, S.ordering_used};
  h = fnv(h, dims, sizeof(dims));
  for (const CsrPattern* P : {&S.H, &S.Ds, &S.Jc, &S.Jd}) {
    h = fnv(h, P->rp.data(), P->rp.size() * sizeof(int));
    h = fnv(h, P->ci.data(), P->ci.size() * sizeof(int));
  }
  return fnv(h, S.perm.data(), S.perm.size() * sizeof(int));
}

struct TuneChoice {
  int solve_piece = 0, warp_subtree = 16, chunk_fma = 4096;
};

bool cache_lookup(const char* path, uint64_t key, int share, TuneChoice& c) {
  if (!path || !*path) return false;
  std::ifstream f(path);
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    std::istringstream in(line);
    unsigned long long k;
    int sh;
    TuneChoice t;
    if (in >> std::hex >> k >> std::dec >> sh >> t.solve_piece >> t.warp_subtree >> t.chunk_fma && k == key &&
        sh == share) {
      c = t;
      found = true;  // the last entry for the key wins
    }
  }
  return found;
}

void cache_store(const char* path, uint64_t key, int share, const TuneChoice& c, double rate) {
  if (!path || !*path) return;
  std::ofstream f(path, std::ios::app);
  f << std::hex << (unsigned long long)key << std::dec << " " << share << " " << c.solve_piece << " "
    << c.warp_subtree << " " << c.chunk_fma << " " << rate << "\n";
}

SymbolicOptions options_for(const SymbolicOptions& base, const TuneChoice& c) {
  SymbolicOptions o = base;
  o.solve_piece = c.solve_piece > 0 ? c.solve_piece : (1 << 30);
  o.warp_subtree = c.warp_subtree;
  o.chunk_fma = c.chunk_fma;
  return o;
}

std::unique_ptr<Engine> engine_like(const Engine& base, const SymbolicOptions& o) {
  const Symbolic& B = base.sym();
  Symbolic S = build_symbolic(B.H, B.Ds, B.Jc, B.Jd, o, B.perm.data());
  S.ordering_used = B.ordering_used;  // the plan's ordering, passed on
  auto e = std::make_unique<Engine>(std::move(S), base.gamma(), o);
  int itmax, refine_max;
  double rtol, target;
  base.accuracy(itmax, rtol, refine_max, target);
  e->set_accuracy(itmax, rtol, refine_max, target);
  e->set_refine_rtol(base.refine_rtol());
  e->set_delta(base.delta());
  return e;
}

// solves/s of `share` engines of one layout solving the sample at once
// (fewer when device memory runs short; *used receives how many); 0 when a
// solve failed
double measure_layout(std::unique_ptr<Engine>& first, const double* const v[8], int share, int* used) {
  std::vector<std::unique_ptr<Engine>> es;
  es.push_back(std::move(first));
  size_t free_b = 0, total_b = 0;
  HYKKT_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const int64_t per = es[0]->device_bytes();
  const int fit = (int)std::max<int64_t>(1, std::min<int64_t>(share, 1 + (int64_t)(0.8 * free_b) / std::max<int64_t>(per, 1)));
  for (int k = 1; k < fit; ++k) {
    auto e = std::make_unique<Engine>(Symbolic(es[0]->sym()), es[0]->gamma(), es[0]->options());
    int itmax, refine_max;
    double rtol, target;
    es[0]->accuracy(itmax, rtol, refine_max, target);
    e->set_accuracy(itmax, rtol, refine_max, target);
    e->set_refine_rtol(es[0]->refine_rtol());
    e->set_delta(es[0]->delta());
    es.push_back(std::move(e));
  }
  *used = (int)es.size();
  std::vector<cudaStream_t> st(es.size(), nullptr);
  for (auto& s : st) HYKKT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  double rate = 0.0;
  try {
    for (auto& e : es) e->set_concurrency(share);
    auto round = [&]() {
      for (size_t k = 0; k < es.size(); ++k)
        es[k]->solve(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], nullptr, false, st[k], false);
      bool ok = true;
      for (size_t k = 0; k < es.size(); ++k) ok = (es[k]->finish(st[k]) == ST_OK) && ok;
      return ok;
    };
    bool ok = round();  // warm-up: captures each engine's graph
    const auto t0 = std::chrono::steady_clock::now();
    const int rounds = 2;
    for (int r = 0; r < rounds && ok; ++r) ok = round();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rate = ok ? rounds * (double)es.size() / sec : 0.0;
  } catch (...) {
    for (auto& s : st) cudaStreamDestroy(s);
    first = std::move(es[0]);
    throw;
  }
  for (auto& s : st) HYKKT_CUDA(cudaStreamDestroy(s));
  first = std::move(es[0]);  // the candidate itself survives; its clones go
  return rate;
}

}  // namespace

extern "C" int hykkt_plan_autotune(hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                                   const double* jc_vals, const double* jd_vals, const double* rx, const double* rs,
                                   const double* ry, const double* ryd, int share, const char* cache_path,
                                   hykkt_tune_info* info) {
  return guarded([&]() {
    if (!plan || !info) return fail(HYKKT_INVALID, "plan and info must not be NULL");
    if (share < 1) return fail(HYKKT_INVALID, "share must be >= 1");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::memset(info, 0, sizeof(*info));
    const Engine& base = *plan->eng;
    const SymbolicOptions base_opt = base.options();
    const uint64_t key = pattern_key(base.sym());
    TuneChoice chosen;
    if (cache_lookup(cache_path, key, share, chosen)) {
      auto e = engine_like(base, options_for(base_opt, chosen));
      e->set_concurrency(share);
      plan->eng = std::move(e);
      info->from_cache = 1;
    } else {
      const double* v[8] = {h_vals, ds_vals, jc_vals, jd_vals, rx, rs, ry, ryd};
      for (const double* p : v)
        if (!p) return fail(HYKKT_INVALID, "autotune needs the values of one system of the pattern");
      // widest supernode: pieces at or above it change nothing
      int widest = 0;
      const Symbolic& S = base.sym();
      for (size_t J = 0; J + 1 < S.sn_first.size(); ++J) widest = std::max(widest, S.sn_first[J + 1] - S.sn_first[J]);
      std::vector<TuneChoice> cands;
      cands.push_back({0, 16, 4096});  // whole supernodes, warp subtrees
      cands.push_back({0, 0, 4096});   // whole supernodes, warp items one per warp
      for (int piece : {2048, 2800, 4096})
        if (piece < widest) cands.push_back({piece, 0, 4096});
      int best = -1;
      double best_rate = 0.0;
      std::unique_ptr<Engine> best_eng;
      auto evaluate = [&](const TuneChoice& c) {
        const int slot = info->candidates;
        auto e = engine_like(base, options_for(base_opt, c));
        int used = 0;
        const double r = measure_layout(e, v, share, &used);
        if (slot < 8) {
          info->cand_piece[slot] = c.solve_piece;
          info->cand_subtree[slot] = c.warp_subtree;
          info->cand_chunk_fma[slot] = c.chunk_fma;
          info->solves_per_s[slot] = r;
        }
        info->candidates += 1;
        info->concurrent = used;
        if (r > best_rate) {
          best_rate = r;
          best = slot;
          chosen = c;
          best_eng = std::move(e);
        }
      };
      for (const TuneChoice& c : cands) evaluate(c);
      if (best < 0) return fail(HYKKT_NOT_SPD, "autotune: no candidate layout solved the sample system");
      // product-task size on the best layout
      const TuneChoice layout = chosen;
      for (int fma : {2048, 8192}) {
        TuneChoice c = layout;
        c.chunk_fma = fma;
        evaluate(c);
      }
      best_eng->set_concurrency(share);
      plan->eng = std::move(best_eng);
      cache_store(cache_path, key, share, chosen, best_rate);
      info->best_solves_per_s = best_rate;
    }
    info->solve_piece = chosen.solve_piece;
    info->warp_subtree = chosen.warp_subtree;
    info->chunk_fma = chosen.chunk_fma;
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_set_concurrency(hykkt_plan_t plan, int share) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    plan->eng->set_concurrency(share);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_solve(hykkt_plan_t plan, const double* h_vals, const double* ds_vals, const double* jc_vals,
                                const double* jd_vals, const double* rx, const double* rs, const double* ry,
                                const double* ryd, const double* y0, int values_on_device, void* stream, int sync) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    cudaStream_t st = plan->pick(stream);
    return solve_status(plan->eng->solve(h_vals, ds_vals, jc_vals, jd_vals, rx, rs, ry, ryd, y0,
                                         values_on_device != 0, st, sync != 0));
  });
}

extern "C" int hykkt_plan_wait(hykkt_plan_t plan, void* stream) {
  return guarded([&]() { return solve_status(plan->eng->finish(plan->pick(stream))); });
}

extern "C" int hykkt_plan_get_solution(hykkt_plan_t plan, double* x, double* ds, double* y, double* yd, int to_device,
                                       void* stream) {
  return guarded([&]() { return plan->eng->get_solution(x, ds, y, yd, to_device != 0, plan->pick(stream)); });
}

extern "C" int hykkt_plan_get_info(hykkt_plan_t plan, hykkt_info* info) {
  return guarded([&]() {
    fill_info(*plan->eng, info);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_set_gamma(hykkt_plan_t plan, double gamma) {
  return guarded([&]() {
    plan->eng->set_gamma(gamma);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_set_accuracy(hykkt_plan_t plan, int cg_itmax, double cg_rtol, int refine_max,
                                       double refine_target) {
  return guarded([&]() {
    if (cg_itmax < 1 || refine_max < 0 || cg_rtol < 0) return fail(HYKKT_INVALID, "bad accuracy settings");
    plan->eng->set_accuracy(cg_itmax, cg_rtol, refine_max, refine_target);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_set_delta(hykkt_plan_t plan, double delta) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    plan->eng->set_delta(delta);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_solve_regularized(hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                                            const double* jc_vals, const double* jd_vals, const double* rx,
                                            const double* rs, const double* ry, const double* ryd, const double* y0,
                                            int values_on_device, void* stream, double delta_first, double delta_max,
                                            double growth, double* delta_used) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    if (!(delta_first > 0.0) || !(delta_max >= delta_first) || !(growth > 1.0))
      return fail(HYKKT_INVALID, "need 0 < delta_first <= delta_max and growth > 1");
    cudaStream_t st = plan->pick(stream);
    double delta = plan->eng->delta();
    int rc;
    for (;;) {
      rc = plan->eng->solve(h_vals, ds_vals, jc_vals, jd_vals, rx, rs, ry, ryd, y0, values_on_device != 0, st, true);
      if (rc != HYKKT_NOT_SPD) break;
      const double next = delta == 0.0 ? delta_first : delta * growth;
      if (next > delta_max) break;
      delta = next;
      plan->eng->set_delta(delta);
    }
    if (delta_used) *delta_used = delta;
    return solve_status(rc);
  });
}

extern "C" int hykkt_plan_set_refine_rtol(hykkt_plan_t plan, double rtol) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    if (!(rtol >= 0)) return fail(HYKKT_INVALID, "refinement tolerance must be >= 0");
    plan->eng->set_refine_rtol(rtol);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_get_perm(hykkt_plan_t plan, int* perm) {
  return guarded([&]() {
    const auto& p = plan->eng->sym().perm;
    std::copy(p.begin(), p.end(), perm);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_get_L_pattern(hykkt_plan_t plan, int* cp, int* ri, int64_t* nnz) {
  return guarded([&]() {
    const Symbolic& S = plan->eng->sym();
    if (nnz) *nnz = S.nnz_L;
    if (!cp) return HYKKT_OK;
    std::vector<int> c, r;
    structural_L(S, c, r);
    std::copy(c.begin(), c.end(), cp);
    std::copy(r.begin(), r.end(), ri);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_get_etree(hykkt_plan_t plan, int* parent) {
  return guarded([&]() {
    const auto& p = plan->eng->sym().parent;
    std::copy(p.begin(), p.end(), parent);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_run_stages(hykkt_plan_t plan, int upto, float* stage_ms) {
  return guarded([&]() {
    cudaStream_t st = plan->pick(nullptr);
    plan->eng->run_direct(st, upto, stage_ms);
    return solve_status(plan->eng->finish(st));
  });
}

extern "C" int hykkt_plan_debug_read(hykkt_plan_t plan, const char* what, double* out, int64_t n) {
  return guarded([&]() {
    int rc = plan->eng->debug_read(what, out, n);
    if (rc) return fail(rc, std::string("unknown array or size: ") + what);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_get_sizes(hykkt_plan_t plan, int64_t* sizes) {
  return guarded([&]() {
    const Symbolic& S = plan->eng->sym();
    sizes[0] = S.Ht.nnz();
    sizes[1] = S.lp_cp[S.n_x];
    sizes[2] = S.Hg.nnz();
    sizes[3] = S.nnz_L;
    sizes[4] = S.front_arena;
    sizes[5] = S.nsn;
    sizes[6] = S.nsq;
    sizes[7] = S.u_arena;
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_get_patterns(hykkt_plan_t plan, int* ht_rp, int* ht_ci, int* lp_cp, int* lp_row) {
  return guarded([&]() {
    const Symbolic& S = plan->eng->sym();
    if (ht_rp) std::copy(S.Ht.rp.begin(), S.Ht.rp.end(), ht_rp);
    if (ht_ci) std::copy(S.Ht.ci.begin(), S.Ht.ci.end(), ht_ci);
    if (lp_cp) std::copy(S.lp_cp.begin(), S.lp_cp.end(), lp_cp);
    if (lp_row) std::copy(S.lp_row.begin(), S.lp_row.end(), lp_row);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_profile(hykkt_plan_t plan, int upto, char* buf, int cap) {
  return guarded([&]() {
    std::vector<KernelTime> kt;
    cudaStream_t st = plan->pick(nullptr);
    plan->eng->profile(st, upto, kt);
    std::string js = "{";
    char tmp[256];
    for (size_t i = 0; i < kt.size(); ++i) {
      std::snprintf(tmp, sizeof tmp, "%s\"%s\": [%d, %.6f, %.6e, %.6e]", i ? ", " : "", kt[i].name.c_str(),
                    kt[i].launches, kt[i].ms, kt[i].flops, kt[i].bytes);
      js += tmp;
    }
    js += "}";
    if ((int)js.size() + 1 > cap) return fail(HYKKT_INVALID, "profile buffer too small");
    std::memcpy(buf, js.c_str(), js.size() + 1);
    return solve_status(plan->eng->finish(st));
  });
}

extern "C" int hykkt_plan_debug_set(hykkt_plan_t plan, const char* what, double value) {
  return guarded([&]() {
    if (!plan || !what) return fail(HYKKT_INVALID, "plan and setting name must not be NULL");
    plan->eng->debug_set(what, value);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_trace_trisolve(hykkt_plan_t plan, unsigned long long* out, int64_t cap, int64_t* n) {
  return guarded([&]() {
    if (!plan) return fail(HYKKT_INVALID, "NULL plan");
    std::vector<unsigned long long> t;
    plan->eng->trace_trisolve(plan->pick(nullptr), t);
    if (n) *n = (int64_t)t.size();
    if (out) {
      if (cap < (int64_t)t.size()) return fail(HYKKT_INVALID, "trace buffer too small");
      std::copy(t.begin(), t.end(), out);
    }
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_time_trisolve(hykkt_plan_t plan, int nrep, float* ms) {
  return guarded([&]() {
    *ms = plan->eng->time_trisolve(plan->pick(nullptr), nrep);
    return solve_status(plan->eng->finish(plan->pick(nullptr)));
  });
}

extern "C" int hykkt_plans_time_trisolve(hykkt_plan_t* plans, int n, int nrep, int mode, float* ms) {
  return guarded([&]() {
    if (!plans || n < 1 || !ms || mode < 0 || mode > 2) return fail(HYKKT_INVALID, "bad arguments");
    std::vector<Engine*> es;
    for (int i = 0; i < n; ++i) {
      if (!plans[i]) return fail(HYKKT_INVALID, "NULL plan");
      es.push_back(plans[i]->eng.get());
    }
    cudaStream_t st = plans[0]->pick(nullptr);
    *ms = Engine::time_trisolve_group(es, nrep, mode, st);
    HYKKT_CUDA(cudaStreamSynchronize(st));
    return HYKKT_OK;
  });
}

extern "C" int hykkt_plan_time_solves(hykkt_plan_t plan, int nsteps, float* ms_per_step, void* stream) {
  return guarded([&]() {
    cudaStream_t st = plan->pick(stream);
    plan->eng->ensure_graph();
    cudaEvent_t a, b;
    HYKKT_CUDA(cudaEventCreate(&a));
    HYKKT_CUDA(cudaEventCreate(&b));
    for (int i = 0; i < nsteps; ++i) {
      HYKKT_CUDA(cudaEventRecord(a, st));
      HYKKT_CUDA(cudaGraphLaunch(plan->eng->graph_exec(), st));
      HYKKT_CUDA(cudaEventRecord(b, st));
      HYKKT_CUDA(cudaEventSynchronize(b));
      HYKKT_CUDA(cudaEventElapsedTime(&ms_per_step[i], a, b));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return solve_status(plan->eng->finish(st));
  });
}

// ===========================================================================
// Host-only symbolic
// ===========================================================================
struct hykkt_symbolic_s {
  Symbolic S;
  std::vector<int> L_cp, L_ri;  // built on first request
};

namespace {
const std::vector<int>* sym_array(const Symbolic& S, std::vector<int>& L_cp, std::vector<int>& L_ri,
                                  const char* what) {
  const std::string w(what);
  if (w == "perm") return &S.perm;
  if (w == "etree") return &S.parent;
  if (w == "colcount") return &S.colcount;
  if (w == "ht_rp") return &S.Ht.rp;
  if (w == "ht_ci") return &S.Ht.ci;
  if (w == "hg_rp") return &S.Hg.rp;
  if (w == "hg_ci") return &S.Hg.ci;
  if (w == "lp_cp") return &S.lp_cp;
  if (w == "lp_row") return &S.lp_row;
  if (w == "sn_first") return &S.sn_first;
  if (w == "sn_parent") return &S.sn_parent;
  if (w == "sn_nrows") return &S.sn_nrows;
  if (w == "sn_rows") return &S.sn_rows;
  if (w == "sn_rp") return &S.sn_rp;
  if (w == "sn_child_rp") return &S.sn_child_rp;
  if (w == "sn_children") return &S.sn_children;
  if (w == "sn_relp") return &S.sn_relp;
  if (w == "sn_rel") return &S.sn_rel;
  if (w == "sq_sn") return &S.sq_sn;
  if (w == "sq_c0") return &S.sq_c0;
  if (w == "sq_c1") return &S.sq_c1;
  if (w == "sq_level_rp") return &S.sq_level_rp;
  if (w == "sq_level_items") return &S.sq_level_items;
  if (w == "g_rp") return &S.g_rp;
  if (w == "sn_level") return &S.sn_level;
  if (w == "sq_level") return &S.sq_level;
  if (w == "sq_mode") return &S.sq_mode;
  if (w == "wg_rp") return &S.wg_rp;
  if (w == "wg_item") return &S.wg_item;
  if (w == "sg_rp") return &S.sg_rp;
  if (w == "sg_item") return &S.sg_item;
  if (w == "sg_lvl") return &S.sg_lvl;
  if (w == "sq_pcoff") return &S.sq_pcoff;
  if (w == "sq_parent") return &S.sq_parent;
  if (w == "sq_rpar") return &S.sq_rpar;
  if (w == "nchild") return &S.nchild;
  if (w == "cd_rp") return &S.cd_rp;
  if (w == "cd_item") return &S.cd_item;
  if (w == "cd_lr") return &S.cd_lr;
  if (w == "fch_row0") return &S.fch_row0;
  if (w == "fch_rows") return &S.fch_rows;
  if (w == "fch0") return &S.fch0;
  if (w == "nfch") return &S.nfch;
  if (w == "fct_rp") return &S.fct_rp;
  if (w == "fct_item") return &S.fct_item;
  if (w == "fdiag_need") return &S.fdiag_need;
  if (w == "sq_rows_x") return &S.sq_rows_x;
  if (w == "unit_cols") {
    static thread_local std::vector<int> one;
    one.assign(1, S.unit_cols);
    return &one;
  }
  if (w == "ch_row0") return &S.ch_row0;
  if (w == "ch_rows") return &S.ch_rows;
  if (w == "ch_item") return &S.ch_item;
  if (w == "ch0") return &S.ch0;
  if (w == "nch") return &S.nch;
  if (w == "ct_rp") return &S.ct_rp;
  if (w == "ct_item") return &S.ct_item;
  if (w == "diag_need") return &S.diag_need;
  if (w == "ic_rp") return &S.ic_rp;
  if (w == "ic_chunk") return &S.ic_chunk;
  if (w == "tf_kind") return &S.tf_kind;
  if (w == "tf_item") return &S.tf_item;
  if (w == "tf_arg") return &S.tf_arg;
  if (w == "tb_kind") return &S.tb_kind;
  if (w == "tb_item") return &S.tb_item;
  if (w == "tb_arg") return &S.tb_arg;
  if (w == "bd_need") return &S.bd_need;
  if (w == "g_pos" || w == "sq_uoff" || w == "sq_doff" || w == "ch_poff" || w == "sq_xpoff" ||
      w == "fch_slot" || w == "sq_l21f" || w == "sq_l21b") {  // 64-bit offsets, narrowed for inspection
    static thread_local std::vector<int> narrow;
    const std::vector<int64_t>& v = w == "g_pos"     ? S.g_pos
                                    : w == "sq_uoff" ? S.sq_uoff
                                    : w == "sq_doff" ? S.sq_doff
                                    : w == "ch_poff" ? S.ch_poff
                                    : w == "fch_slot" ? S.fch_slot
                                    : w == "sq_l21f" ? S.sq_l21f
                                    : w == "sq_l21b" ? S.sq_l21b
                                                      : S.sq_xpoff;
    narrow.assign(v.size(), 0);
    for (size_t i = 0; i < v.size(); ++i) {
      if (v[i] > INT_MAX) throw std::runtime_error("offset does not fit 32 bits");
      narrow[i] = (int)v[i];
    }
    return &narrow;
  }
  if (w == "L_cp" || w == "L_ri") {
    if (L_cp.empty()) structural_L(S, L_cp, L_ri);
    return w == "L_cp" ? &L_cp : &L_ri;
  }
  return nullptr;
}
}  // namespace

extern "C" int hykkt_symbolic_create_ex(hykkt_symbolic_t* sym, int n_x, int m_c, int m_d, const int* h_rowptr,
                                        const int* h_colidx, int nnz_h, const int* ds_rowptr, const int* ds_colidx,
                                        int nnz_ds, const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                                        const int* jd_rowptr, const int* jd_colidx, int nnz_jd, int ordering,
                                        const int* perm, int solve_piece) {
  return guarded([&]() {
    *sym = nullptr;
    if (solve_piece < 0) return fail(HYKKT_INVALID, "solve_piece must be >= 0");
    CsrPattern H = make_pattern(n_x, n_x, h_rowptr, h_colidx, nnz_h);
    CsrPattern Ds = make_pattern(m_d, m_d, ds_rowptr, ds_colidx, nnz_ds);
    CsrPattern Jc = make_pattern(m_c, n_x, jc_rowptr, jc_colidx, nnz_jc);
    CsrPattern Jd = make_pattern(m_d, n_x, jd_rowptr, jd_colidx, nnz_jd);
    SymbolicOptions opt = default_options(ordering);
    apply_solve_piece(opt, solve_piece);
    auto h = std::make_unique<hykkt_symbolic_s>();
    h->S = build_symbolic(H, Ds, Jc, Jd, opt, perm);
    *sym = h.release();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_symbolic_create(hykkt_symbolic_t* sym, int n_x, int m_c, int m_d, const int* h_rowptr,
                                     const int* h_colidx, int nnz_h, const int* ds_rowptr, const int* ds_colidx,
                                     int nnz_ds, const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                                     const int* jd_rowptr, const int* jd_colidx, int nnz_jd, int ordering,
                                     const int* perm) {
  return hykkt_symbolic_create_ex(sym, n_x, m_c, m_d, h_rowptr, h_colidx, nnz_h, ds_rowptr, ds_colidx, nnz_ds,
                                  jc_rowptr, jc_colidx, nnz_jc, jd_rowptr, jd_colidx, nnz_jd, ordering, perm, 0);
}

extern "C" void hykkt_symbolic_destroy(hykkt_symbolic_t sym) { delete sym; }

extern "C" int64_t hykkt_symbolic_size(hykkt_symbolic_t sym, const char* what) {
  const std::vector<int>* a = sym_array(sym->S, sym->L_cp, sym->L_ri, what);
  return a ? (int64_t)a->size() : -1;
}

extern "C" int hykkt_symbolic_get(hykkt_symbolic_t sym, const char* what, int* out, int64_t n) {
  return guarded([&]() {
    const std::vector<int>* a = sym_array(sym->S, sym->L_cp, sym->L_ri, what);
    if (!a || n > (int64_t)a->size()) return fail(HYKKT_INVALID, std::string("unknown array or size: ") + what);
    std::copy(a->begin(), a->begin() + n, out);
    return HYKKT_OK;
  });
}

extern "C" int64_t hykkt_plan_symbolic_size(hykkt_plan_t plan, const char* what) {
  static thread_local std::vector<int> cp, ri;
  cp.clear();
  ri.clear();
  const std::vector<int>* a = sym_array(plan->eng->sym(), cp, ri, what);
  return a ? (int64_t)a->size() : -1;
}

extern "C" int hykkt_plan_symbolic_get(hykkt_plan_t plan, const char* what, int* out, int64_t n) {
  return guarded([&]() {
    std::vector<int> cp, ri;
    const std::vector<int>* a = sym_array(plan->eng->sym(), cp, ri, what);
    if (!a || n > (int64_t)a->size()) return fail(HYKKT_INVALID, std::string("unknown array or size: ") + what);
    std::copy(a->begin(), a->begin() + n, out);
    return HYKKT_OK;
  });
}

// ===========================================================================
// HykktSolver mirror
// ===========================================================================
namespace {
struct Block {
  int* rp = nullptr;
  int* ci = nullptr;
  double* v = nullptr;
  int n = 0, m = 0, nnz = 0;
  bool set = false;
  std::vector<int> own_rp, own_ci;
  std::vector<double> own_v;
};
struct Vec {
  double* p = nullptr;
  int n = 0;
  std::vector<double> own;
};
}  // namespace

struct hykkt_solver_s {
  double gamma;
  int ordering = HYKKT_ORDER_AUTO;
  Block H, Ds, Jc, Jd;
  Vec rx, rs, ry, ryd, x0, s0, y0, yd0;
  bool allocated = false, jd_flag = false, status_ok = true;
  int cg_itmax = 100, refine_max = 0;  // reference semantics by default
  double cg_rtol = 0.0, refine_target = 1e-10;
  std::unique_ptr<Engine> eng;
  std::vector<int> snap;  // concatenated patterns at analysis time
  cudaStream_t stream = nullptr;
  ~hykkt_solver_s() {
    eng.reset();
    if (stream) cudaStreamDestroy(stream);
  }
  void snapshot(std::vector<int>& out) const {
    out.clear();
    for (const Block* b : {&H, &Ds, &Jc, &Jd}) {
      out.push_back(b->n);
      out.push_back(b->m);
      out.push_back(b->nnz);
      if (b->rp) out.insert(out.end(), b->rp, b->rp + b->n + 1);
      if (b->ci) out.insert(out.end(), b->ci, b->ci + b->nnz);
    }
  }
};

namespace {
void read_block(Block& b, const char* file, int skip, bool symmetric) {
  MMatrix mat;
  read_mm_file_into_coo(file, mat, skip);
  if (symmetric) sym_coo_to_csr(mat);
  else coo_to_csr(mat);
  b.own_rp.assign(mat.csr_rows, mat.csr_rows + mat.n_ + 1);
  b.own_ci.assign(mat.csr_cols, mat.csr_cols + mat.nnz_);
  b.own_v.assign(mat.csr_vals, mat.csr_vals + mat.nnz_);
  b.rp = b.own_rp.data();
  b.ci = b.own_ci.data();
  b.v = b.own_v.data();
  b.n = mat.n_;
  b.m = mat.m_;
  b.nnz = mat.nnz_;
  b.set = true;
}
void read_vec(Vec& v, const char* file, int n) {
  std::vector<double> tmp(n + 1, 0.0);
  // read_rhs has no size argument in the reference; read into a buffer that
  // is checked against the expected length
  MMatrix dummy;
  (void)dummy;
  FILE* f = std::fopen(file, "r");
  if (!f) throw std::runtime_error(std::string("cannot open ") + file);
  std::fclose(f);
  std::vector<double> all;
  {
    // count lines first to size the buffer
    FILE* g = std::fopen(file, "r");
    int c, lines = 0;
    while ((c = std::fgetc(g)) != EOF)
      if (c == '\n') ++lines;
    std::fclose(g);
    all.assign(lines + 2, 0.0);
  }
  read_rhs(file, all.data());
  v.own.assign(all.begin(), all.begin() + n);
  v.p = v.own.data();
  v.n = n;
}
}  // namespace

extern "C" hykkt_solver_t hykkt_solver_create(double gamma) {
  try {
    auto* s = new hykkt_solver_s();
    s->gamma = gamma;
    return s;
  } catch (...) {
    g_err = "allocation failed";
    return nullptr;
  }
}

extern "C" void hykkt_solver_destroy(hykkt_solver_t s) { delete s; }

extern "C" int hykkt_solver_set_accuracy(hykkt_solver_t s, int cg_itmax, double cg_rtol, int refine_max,
                                         double refine_target) {
  return guarded([&]() {
    if (cg_itmax < 1 || refine_max < 0 || cg_rtol < 0) return fail(HYKKT_INVALID, "bad accuracy settings");
    s->cg_itmax = cg_itmax;
    s->cg_rtol = cg_rtol;
    s->refine_max = refine_max;
    s->refine_target = refine_target;
    if (s->eng) s->eng->set_accuracy(cg_itmax, cg_rtol, refine_max, refine_target);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_solver_set_ordering(hykkt_solver_t s, int ordering) {
  s->ordering = ordering;
  return HYKKT_OK;
}

extern "C" int hykkt_solver_read_matrix_files(hykkt_solver_t s, const char* h_file, const char* ds_file,
                                              const char* jc_file, const char* jd_file, const char* rx_file,
                                              const char* rs_file, const char* ry_file, const char* ryd_file,
                                              int skip_lines) {
  return guarded([&]() {
    read_block(s->H, h_file, skip_lines, true);   // sym_coo_to_csr (HykktSolver.cpp:124-126)
    read_block(s->Ds, ds_file, skip_lines, false);
    read_block(s->Jc, jc_file, skip_lines, false);
    read_block(s->Jd, jd_file, skip_lines, false);
    const bool jd_flag = s->Jd.nnz > 0;
    s->status_ok = (s->jd_flag == jd_flag);  // HykktSolver.cpp:140-144
    s->jd_flag = jd_flag;
    read_vec(s->rx, rx_file, s->H.n);
    read_vec(s->rs, rs_file, s->Ds.n);
    read_vec(s->ry, ry_file, s->Jc.n);
    read_vec(s->ryd, ryd_file, s->Jd.n);
    return HYKKT_OK;
  });
}

static int set_block(hykkt_solver_t s, Block& b, int* rp, int* ci, double* v, int n, int m, int nnz) {
  b.rp = rp;
  b.ci = ci;
  b.v = v;
  b.n = n;
  b.m = m;
  b.nnz = nnz;
  b.set = true;
  b.own_rp.clear();
  b.own_ci.clear();
  b.own_v.clear();
  (void)s;
  return HYKKT_OK;
}

extern "C" int hykkt_solver_set_H(hykkt_solver_t s, int* rp, int* ci, double* v, int n, int m, int nnz) {
  if (n != m) return fail(HYKKT_INVALID, "set_H: H must be square");  // assert(m == n), HykktSolver.cpp:165
  return set_block(s, s->H, rp, ci, v, n, m, nnz);
}
extern "C" int hykkt_solver_set_Ds(hykkt_solver_t s, int* rp, int* ci, double* v, int n, int m, int nnz) {
  if (n != m) return fail(HYKKT_INVALID, "set_Ds: Ds must be square");
  return set_block(s, s->Ds, rp, ci, v, n, m, nnz);
}
extern "C" int hykkt_solver_set_Jc(hykkt_solver_t s, int* rp, int* ci, double* v, int n, int m, int nnz) {
  return set_block(s, s->Jc, rp, ci, v, n, m, nnz);
}
extern "C" int hykkt_solver_set_Jd(hykkt_solver_t s, int* rp, int* ci, double* v, int n, int m, int nnz) {
  int rc = set_block(s, s->Jd, rp, ci, v, n, m, nnz);
  s->jd_flag = nnz > 0;
  s->status_ok = true;  // HykktSolver.cpp:188-191: the pointer API cannot see a changed jd flag
  return rc;
}

static int set_vec(Vec& v, double* p, int n, const char* name) {
  if (v.p != nullptr && v.own.empty()) return fail(HYKKT_INVALID, std::string(name) + ": vector already set");
  v.own.clear();
  v.p = p;
  v.n = n;
  return HYKKT_OK;
}
extern "C" int hykkt_solver_set_rx(hykkt_solver_t s, double* p, int n) { return set_vec(s->rx, p, n, "set_rx"); }
extern "C" int hykkt_solver_set_rs(hykkt_solver_t s, double* p, int n) { return set_vec(s->rs, p, n, "set_rs"); }
extern "C" int hykkt_solver_set_ry(hykkt_solver_t s, double* p, int n) { return set_vec(s->ry, p, n, "set_ry"); }
extern "C" int hykkt_solver_set_ryd(hykkt_solver_t s, double* p, int n) { return set_vec(s->ryd, p, n, "set_ryd"); }
extern "C" int hykkt_solver_set_x_host(hykkt_solver_t s, double* p, int n) { return set_vec(s->x0, p, n, "set_x_host"); }
extern "C" int hykkt_solver_set_s_host(hykkt_solver_t s, double* p, int n) { return set_vec(s->s0, p, n, "set_s_host"); }
extern "C" int hykkt_solver_set_y_host(hykkt_solver_t s, double* p, int n) { return set_vec(s->y0, p, n, "set_y_host"); }
extern "C" int hykkt_solver_set_yd_host(hykkt_solver_t s, double* p, int n) { return set_vec(s->yd0, p, n, "set_yd_host"); }

extern "C" int hykkt_solver_set_gamma(hykkt_solver_t s, double gamma) {
  return guarded([&]() {
    s->gamma = gamma;
    if (s->eng) s->eng->set_gamma(gamma);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_solver_execute(hykkt_solver_t s) {
  int rc = guarded([&]() {
    if (!s->status_ok && s->allocated)
      return fail(HYKKT_PATTERN_CHANGED, "new nonzero structure after the first execute()");
    if (!s->H.set || !s->Jc.set || !s->Ds.set || !s->Jd.set) return fail(HYKKT_INVALID, "matrix blocks not set");
    if (!s->rx.p || !s->rs.p || !s->ry.p || !s->ryd.p) return fail(HYKKT_INVALID, "right-hand sides not set");
    if (!s->stream) HYKKT_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    if (!s->allocated) {
      CsrPattern H = make_pattern(s->H.n, s->H.m, s->H.rp, s->H.ci, s->H.nnz);
      CsrPattern Ds = make_pattern(s->Ds.n, s->Ds.m, s->Ds.rp, s->Ds.ci, s->Ds.nnz);
      CsrPattern Jc = make_pattern(s->Jc.n, s->Jc.m, s->Jc.rp, s->Jc.ci, s->Jc.nnz);
      CsrPattern Jd = make_pattern(s->Jd.n, s->Jd.m, s->Jd.rp, s->Jd.ci, s->Jd.nnz);
      Symbolic S = build_symbolic(H, Ds, Jc, Jd, default_options(s->ordering), nullptr);
      s->eng = std::make_unique<Engine>(std::move(S), s->gamma, default_options(s->ordering));
      s->eng->set_accuracy(s->cg_itmax, s->cg_rtol, s->refine_max, s->refine_target);
      s->snapshot(s->snap);
    } else {
      std::vector<int> now;
      s->snapshot(now);
      if (now != s->snap) return fail(HYKKT_PATTERN_CHANGED, "new nonzero structure after the first execute()");
    }
    int st = s->eng->solve(s->H.v, s->Ds.v, s->Jc.v, s->Jd.v, s->rx.p, s->rs.p, s->ry.p, s->ryd.p, s->y0.p, false,
                           s->stream, true);
    s->allocated = true;
    (void)st;  // CG non-convergence and pivots are reported through get_info
    const double res = s->eng->last_scalars().rel_res_ref;
    if (!(res < 1e-2)) return fail(HYKKT_RESIDUAL_FAILED, "relative residual above 1e-2");  // HykktSolver.cpp:923-929
    return HYKKT_OK;
  });
  return rc == HYKKT_OK ? 0 : 1;
}

extern "C" int hykkt_solver_get_solution(hykkt_solver_t s, double* x, double* ds, double* y, double* yd) {
  return guarded([&]() {
    if (!s->eng) return fail(HYKKT_NOT_READY, "execute() has not run");
    return s->eng->get_solution(x, ds, y, yd, false, s->stream);
  });
}

extern "C" int hykkt_solver_get_info(hykkt_solver_t s, hykkt_info* info) {
  return guarded([&]() {
    if (!s->eng) return fail(HYKKT_NOT_READY, "execute() has not run");
    fill_info(*s->eng, info);
    return HYKKT_OK;
  });
}

// ===========================================================================
// Components
// ===========================================================================
extern "C" int hykkt_perm_maps(int n, const int* perm, const int* a_rows, const int* a_cols, int nnz_a, int n_j,
                               const int* j_rows, const int* j_cols, int nnz_j, int m_j, const int* jt_rows,
                               const int* jt_cols, int* rev_perm, int* rc_rows, int* rc_cols, int* rc_map,
                               int* c_cols, int* c_map, int* r_rows, int* r_cols, int* r_map) {
  return guarded([&]() {
    std::vector<int> rev(n);
    for (int i = 0; i < n; ++i) rev[perm[i]] = i;  // reverse_perm (permcheck.cu:126-132)
    if (rev_perm) std::copy(rev.begin(), rev.end(), rev_perm);
    std::vector<std::pair<int, int>> tmp;
    if (rc_rows && a_rows) {  // make_vec_map_rc: rows by perm, columns by rev_perm, sorted per row
      rc_rows[0] = 0;
      int cnt = 0;
      for (int i = 0; i < n; ++i) {
        const int o = perm[i];
        tmp.clear();
        for (int p = a_rows[o]; p < a_rows[o + 1]; ++p) tmp.push_back({rev[a_cols[p]], p});
        std::stable_sort(tmp.begin(), tmp.end(), [](auto& x, auto& y) { return x.first < y.first; });
        for (auto& t : tmp) { rc_cols[cnt] = t.first; rc_map[cnt] = t.second; ++cnt; }
        rc_rows[i + 1] = cnt;
      }
      (void)nnz_a;
    }
    if (c_cols && j_rows) {  // make_vec_map_c: rows kept, columns by rev_perm, sorted per row
      for (int i = 0; i < n_j; ++i) {
        tmp.clear();
        for (int p = j_rows[i]; p < j_rows[i + 1]; ++p) tmp.push_back({rev[j_cols[p]], p});
        std::stable_sort(tmp.begin(), tmp.end(), [](auto& x, auto& y) { return x.first < y.first; });
        int q = j_rows[i];
        for (auto& t : tmp) { c_cols[q] = t.first; c_map[q] = t.second; ++q; }
      }
      (void)nnz_j;
    }
    if (r_rows && jt_rows) {  // make_vec_map_r: rows by perm, columns unchanged
      r_rows[0] = 0;
      int cnt = 0;
      for (int i = 0; i < m_j; ++i) {
        const int o = perm[i];
        for (int p = jt_rows[o]; p < jt_rows[o + 1]; ++p) { r_cols[cnt] = jt_cols[p]; r_map[cnt] = p; ++cnt; }
        r_rows[i + 1] = cnt;
      }
    }
    return HYKKT_OK;
  });
}

extern "C" int hykkt_fp64_peak(double* tflops) {
  return guarded([&]() {
    *tflops = fp64_peak_tflops();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_fp64_probe(int mode, double* tflops) {
  return guarded([&]() {
    if (!tflops) return fail(HYKKT_INVALID, "NULL output");
    *tflops = fp64_probe_tflops(mode);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_map_index(int n, const int* d_map, const double* d_old, double* d_new, void* stream) {
  return guarded([&]() {
    map_index(n, d_map, d_old, d_new, (cudaStream_t)stream);
    HYKKT_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return HYKKT_OK;
  });
}

extern "C" int hykkt_ruiz_scale(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v,
                                const int* bt_i, const int* bt_j, double* b_v, const int* b_i, const int* b_j,
                                double* rhs1, double* rhs2, double* max_d, void* stream) {
  return guarded([&]() {
    ruiz_scale(its, n, m, a_v, a_i, a_j, bt_v, bt_i, bt_j, b_v, b_i, b_j, rhs1, rhs2, max_d, (cudaStream_t)stream);
    HYKKT_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return HYKKT_OK;
  });
}

// No allocation: for callers that must not touch the device allocator at the
// point where they scale.  Enqueues only; the caller synchronises the stream.
extern "C" int hykkt_ruiz_scale_noalloc(int its, int n, int m, double* a_v, const int* a_i, const int* a_j,
                                        double* bt_v, const int* bt_i, const int* bt_j, double* b_v, const int* b_i,
                                        const int* b_j, double* rhs1, double* rhs2, double* max_d, void* stream) {
  return guarded([&]() {
    ruiz_scale_noalloc(its, n, m, a_v, a_i, a_j, bt_v, bt_i, bt_j, b_v, b_i, b_j, rhs1, rhs2, max_d,
                       (cudaStream_t)stream);
    return HYKKT_OK;
  });
}

extern "C" int hykkt_ruiz_scale_noalloc_max_rows(void) { return ruiz_noalloc_max_rows(); }

struct hykkt_chol_s {
  std::unique_ptr<Engine> eng;
  int n = 0, nnz = 0;
  std::vector<int> entry_to_lp;  // input entry -> permuted lower slot (-1: upper, ignored)
  cudaStream_t stream = nullptr;
  ~hykkt_chol_s() {
    eng.reset();
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" int hykkt_chol_create(hykkt_chol_t* c, int n, int nnz, const int* rowptr, const int* colidx,
                                 int ordering) {
  return guarded([&]() {
    *c = nullptr;
    // symmetric pattern from the lower triangle (col <= row); upper entries are ignored
    std::vector<std::vector<int>> rows(n);
    for (int i = 0; i < n; ++i)
      for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
        const int j = colidx[p];
        if (j < 0 || j >= n) throw std::runtime_error("column index out of range");
        if (j > i) continue;
        rows[i].push_back(j);
        if (j != i) rows[j].push_back(i);
      }
    CsrPattern A;
    A.n = A.m = n;
    A.rp.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      std::sort(rows[i].begin(), rows[i].end());
      rows[i].erase(std::unique(rows[i].begin(), rows[i].end()), rows[i].end());
      A.rp[i + 1] = A.rp[i] + (int)rows[i].size();
      A.ci.insert(A.ci.end(), rows[i].begin(), rows[i].end());
    }
    CsrPattern Ds, Jd, Jc;
    Ds.n = Ds.m = 0;
    Ds.rp.assign(1, 0);
    Jd.n = 0; Jd.m = n; Jd.rp.assign(1, 0);
    Jc.n = 0; Jc.m = n; Jc.rp.assign(1, 0);
    Symbolic S = build_symbolic(A, Ds, Jc, Jd, default_options(ordering), nullptr);
    auto h = std::make_unique<hykkt_chol_s>();
    h->n = n;
    h->nnz = nnz;
    h->entry_to_lp.assign(nnz, -1);
    for (int i = 0; i < n; ++i)
      for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
        const int j = colidx[p];
        if (j > i) continue;
        int a = S.rev_perm[i], b = S.rev_perm[j];
        if (a < b) std::swap(a, b);
        const int* beg = S.lp_row.data() + S.lp_cp[b];
        const int* end = S.lp_row.data() + S.lp_cp[b + 1];
        const int* it = std::lower_bound(beg, end, a);
        if (it == end || *it != a) throw std::runtime_error("chol: entry not in pattern");
        h->entry_to_lp[p] = (int)(it - S.lp_row.data());
      }
    h->eng = std::make_unique<Engine>(std::move(S), 0.0, default_options(ordering));
    HYKKT_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    *c = h.release();
    return HYKKT_OK;
  });
}

extern "C" int hykkt_chol_factor(hykkt_chol_t c, const double* vals) {
  return guarded([&]() {
    const Symbolic& S = c->eng->sym();
    std::vector<double> lp(S.lp_cp[S.n_x], 0.0);
    for (int p = 0; p < c->nnz; ++p)
      if (c->entry_to_lp[p] >= 0) lp[c->entry_to_lp[p]] = vals[p];
    return c->eng->factor_values(lp.data(), c->stream);
  });
}

extern "C" int hykkt_chol_solve(hykkt_chol_t c, double* x, const double* b) {
  return guarded([&]() {
    const Symbolic& S = c->eng->sym();
    const int n = S.n_x;
    std::vector<double> bp(n), xp(n);
    for (int i = 0; i < n; ++i) bp[i] = b[S.perm[i]];
    double* db = c->eng->dp.cg_yv;
    double* dx = c->eng->dp.tmp_n;
    HYKKT_CUDA(cudaMemcpyAsync(db, bp.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    c->eng->trisolve(db, dx, c->stream);
    HYKKT_CUDA(cudaMemcpyAsync(xp.data(), dx, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HYKKT_CUDA(cudaStreamSynchronize(c->stream));
    for (int j = 0; j < n; ++j) x[j] = xp[S.rev_perm[j]];
    return HYKKT_OK;
  });
}

extern "C" void hykkt_chol_destroy(hykkt_chol_t c) { delete c; }

extern "C" int hykkt_schur_cg(hykkt_chol_t c, int m, int n, const int* jc_rowptr, const int* jc_colidx,
                              const double* jc_vals, int nnz_jc, const double* b, double* x, int itmax, double tol,
                              int* iterations, double* final_err) {
  return guarded([&]() {
    if (n != c->eng->sym().n_x) return fail(HYKKT_INVALID, "Jc column count differs from the factor size");
    std::vector<int> rp(jc_rowptr, jc_rowptr + m + 1), ci(jc_colidx, jc_colidx + nnz_jc);
    return c->eng->schur_cg(m, rp, ci, jc_vals, b, x, itmax, tol, iterations, final_err, c->stream);
  });
}
