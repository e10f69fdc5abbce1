/*
 * hykkt_gb300 -- C ABI of the GB300-native HyKKT KKT solve path.
 *
 * Plain pointers and sizes only.  All matrices are 0-based int32 CSR with
 * sorted column indices, values FP64, exactly as the reference's HykktSolver
 * setters take them (src/HykktSolver.hpp:49-108).  Every entry point returns
 * an int status (HYKKT_OK == 0) unless stated otherwise; the message of the
 * last failure on the calling thread is available from hykkt_last_error().
 *
 * Layers:
 *   1. hykkt_solver_*  -- one-to-one mirror of the reference class HykktSolver
 *      (borrowed host buffers, execute() returning 0/1).  include/HykktSolver.hpp
 *      is the C++ drop-in built on it.
 *   2. hykkt_plan_*    -- pattern-level plan: symbolic analysis once per sparsity,
 *      numeric solves from host or device values on a caller stream, clones
 *      and concurrency for batched solving, regularization.
 *   3. hykkt_server_*  -- served solves: a thread-safe request queue over plans.
 *   4. component calls mirroring the reference's component classes and the
 *      tests that drive them (PermClass/permcheck, RuizClass, CholeskyClass,
 *      SchurComplementConjugateGradient).
 */
#ifndef HYKKT_GB300_H
#define HYKKT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define HYKKT_OK 0
#define HYKKT_NOT_SPD 1            /* zero/negative pivot (reference only prints it, CholeskyClass.cpp:87-89) */
#define HYKKT_CG_NOT_CONVERGED 2   /* CG hit itmax (reference returns 1 and ignores it, SchurCG.cpp:189-193) */
#define HYKKT_PATTERN_CHANGED 3    /* new nonzero structure (HykktSolver.cpp:243-250) */
#define HYKKT_OOM 4
#define HYKKT_TIMEOUT 5
#define HYKKT_INVALID 6
#define HYKKT_CUDA_ERROR 7
#define HYKKT_RESIDUAL_FAILED 8    /* relative residual >= 1e-2 (HykktSolver.cpp:923-929) */
#define HYKKT_NOT_READY 9
/* No counterpart in the reference (which has no accuracy target beyond its
 * 1e-2 residual test, HykktSolver.cpp:923-929): refinement was requested
 * (hykkt_plan_set_accuracy with refine_max > 0) and the solve ended with the
 * full 4-block relative residual above refine_target.  The solution is
 * still readable; it is the best iterate the solve reached. */
#define HYKKT_ACCURACY_NOT_MET 10
/* a served request withdrawn before a worker took it (hykkt_server_cancel) */
#define HYKKT_CANCELLED 11

/* orderings */
#define HYKKT_ORDER_AUTO 0        /* reference symamd when available, else builtin AMD */
#define HYKKT_ORDER_REFERENCE 1   /* cusolverSpXcsrsymamdHost, as PermClass::symamd (PermClass.cpp:88-95) */
#define HYKKT_ORDER_BUILTIN 2     /* this project's approximate minimum degree */
#define HYKKT_ORDER_IDENTITY 3    /* factor in the given order */

const char* hykkt_last_error(void);
const char* hykkt_version(void);

/* Result and statistics of the last solve. */
typedef struct hykkt_info {
  int status;              /* HYKKT_* of the numeric solve */
  int cg_iterations;       /* iterations of the last Schur CG run (with refinement: the last correction's) */
  int pivot_col;           /* first bad pivot (permuted column) or -1 */
  int ordering;            /* HYKKT_ORDER_* actually used */
  double cg_residual;      /* final sqrt(r.r) of the CG (SchurCG.cpp:188) */
  double rel_residual;     /* ||[row1;row3]|| / ||b||, the reference's check_error definition */
  double rel_residual_full;/* all four block rows of the 4x4 KKT system */
  int64_t nnz_L;           /* structural nnz of the Cholesky factor */
  int64_t L_stored;        /* stored entries of the supernodal factor */
  double factor_flops;     /* sum of column counts squared */
  int64_t device_bytes;    /* HBM held by the plan */
  int n_supernodes, n_levels, n_solve_levels;
  int kernels_per_solve;   /* kernel launches outside the CG loop */
  int kernels_per_cg_iteration;
  int cg_iterations_total; /* CG iterations including refinement corrections */
  int refine_steps;        /* refinement corrections applied */
  double rel_residual_first; /* full residual before refinement */
  int kernels_per_refine_step; /* launches of one correction outside its CG loop */
  int pad_;
} hykkt_info;

/* ===========================================================================
 * 1. HykktSolver mirror (reference src/HykktSolver.hpp:17-137)
 * ======================================================================== */
typedef struct hykkt_solver_s* hykkt_solver_t;

/* HykktSolver::HykktSolver(double gamma)          (HykktSolver.hpp:21) */
hykkt_solver_t hykkt_solver_create(double gamma);
/* HykktSolver::~HykktSolver()                     (HykktSolver.hpp:24) */
void hykkt_solver_destroy(hykkt_solver_t s);
/* HykktSolver::read_matrix_files(...)             (HykktSolver.hpp:39-48) */
int hykkt_solver_read_matrix_files(hykkt_solver_t s, const char* h_file, const char* ds_file,
                                   const char* jc_file, const char* jd_file, const char* rx_file,
                                   const char* rs_file, const char* ry_file, const char* ryd_file,
                                   int skip_lines);
/* HykktSolver::set_H/set_Ds/set_Jc/set_Jd         (HykktSolver.hpp:61,75,89,103)
 * The arrays are borrowed: the caller keeps them alive and may overwrite the
 * values in place between execute() calls (same-sparsity flow). */
int hykkt_solver_set_H(hykkt_solver_t s, int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
int hykkt_solver_set_Ds(hykkt_solver_t s, int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
int hykkt_solver_set_Jc(hykkt_solver_t s, int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
int hykkt_solver_set_Jd(hykkt_solver_t s, int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
/* HykktSolver::set_rx/rs/ry/ryd                   (HykktSolver.hpp:105-111) */
int hykkt_solver_set_rx(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_rs(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_ry(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_ryd(hykkt_solver_t s, double* vals, int n);
/* HykktSolver::set_x_host/s/y/yd                  (HykktSolver.hpp:113-116) */
int hykkt_solver_set_x_host(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_s_host(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_y_host(hykkt_solver_t s, double* vals, int n);
int hykkt_solver_set_yd_host(hykkt_solver_t s, double* vals, int n);
/* HykktSolver::set_gamma                          (HykktSolver.hpp:125) */
int hykkt_solver_set_gamma(hykkt_solver_t s, double gamma);
/* HykktSolver::execute: 0 when the relative residual is below 1e-2, 1 on any
 * failure or a changed nonzero structure          (HykktSolver.hpp:137, .cpp:240-286) */
int hykkt_solver_execute(hykkt_solver_t s);
/* Addition: the reference keeps the solution on the device with no accessor
 * (HykktSolver.cpp:451-456); this copies dx, ds, dy, dyd to host arrays
 * (any of them may be NULL). */
int hykkt_solver_get_solution(hykkt_solver_t s, double* x, double* ds, double* y, double* yd);
int hykkt_solver_get_info(hykkt_solver_t s, hykkt_info* info);
/* Use a fixed ordering kind for the next symbolic analysis. */
int hykkt_solver_set_ordering(hykkt_solver_t s, int ordering);

/* ===========================================================================
 * 2. Plan API
 * ======================================================================== */
typedef struct hykkt_plan_s* hykkt_plan_t;

/* Symbolic analysis of one KKT sparsity pattern (host arrays).  Covers
 * setup_spgemm_htil, setup_spgemm_hgamma, setup_permutation and
 * setup_hgamma_factorization of the reference (HykktSolver.cpp:685-811).
 * H is the full symmetric pattern.  Ds is diagonal (one entry per Jd row).
 * perm (optional, NULL for `ordering`) forces a permutation perm[new]=old. */
int hykkt_plan_create(hykkt_plan_t* plan, int n_x, int m_c, int m_d,
                      const int* h_rowptr, const int* h_colidx, int nnz_h,
                      const int* ds_rowptr, const int* ds_colidx, int nnz_ds,
                      const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                      const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                      double gamma, int ordering, const int* perm);
/* No counterpart in the reference.  hykkt_plan_create with one tuning
 * option: solve_piece > 0 splits supernodes wider than that many columns
 * into column pieces for the triangular solves.  Only the pieces' diagonal
 * blocks are inverted after each factorization (less FP64 work per system,
 * which raises batched throughput); a split supernode takes more sequential
 * solve stages.  With pieces, small subtrees of warp-sized items are not
 * grouped into one-CTA tasks (that grouping shortens a lone solve and costs
 * throughput when plans share the GPU).  0 = whole supernodes (the default
 * of hykkt_plan_create). */
int hykkt_plan_create_ex(hykkt_plan_t* plan, int n_x, int m_c, int m_d,
                         const int* h_rowptr, const int* h_colidx, int nnz_h,
                         const int* ds_rowptr, const int* ds_colidx, int nnz_ds,
                         const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                         const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                         double gamma, int ordering, const int* perm, int solve_piece);
void hykkt_plan_destroy(hykkt_plan_t plan);
/* No counterpart in the reference (its solver holds its device memory from
 * the first execute() to destruction).  Device residency of a plan, for
 * callers that serve more patterns than fit in device memory at once:
 * hykkt_plan_create_deferred is hykkt_plan_create_ex with the symbolic
 * analysis done and the device storage counted but not allocated;
 * hykkt_plan_release_device frees all of a plan's device storage (waiting
 * for its own stream first; other streams' work on the plan must be
 * complete), keeping the host analysis and every setting;
 * hykkt_plan_reload_device allocates it again (the next solve also does
 * this by itself).  A released plan has no solution to read.
 * hykkt_plan_residency reports whether the storage is allocated and its
 * size in bytes (known before allocation). */
int hykkt_plan_create_deferred(hykkt_plan_t* plan, int n_x, int m_c, int m_d,
                               const int* h_rowptr, const int* h_colidx, int nnz_h,
                               const int* ds_rowptr, const int* ds_colidx, int nnz_ds,
                               const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                               const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                               double gamma, int ordering, const int* perm, int solve_piece);
int hykkt_plan_release_device(hykkt_plan_t plan);
int hykkt_plan_reload_device(hykkt_plan_t plan);
int hykkt_plan_residency(hykkt_plan_t plan, int* resident, int64_t* bytes);
/* No counterpart in the reference (batched solving).  A new plan for the
 * same sparsity, gamma, ordering and accuracy settings as `src`, reusing its
 * symbolic analysis (no second ordering); its own device memory and stream,
 * so that several systems of one sequence can be solved at once. */
int hykkt_plan_clone(hykkt_plan_t src, hykkt_plan_t* plan);
/* No counterpart in the reference.  Autotuner of the triangular-solve
 * layout for the plan's pattern: candidate layouts (whole supernodes with
 * and without warp-subtree tasks, pieces of 2048 / 2800 / 4096 columns of
 * the widest supernodes, then 2048 / 8192 multiply-adds per product task on
 * the best of those) are built from the plan's own patterns and ordering;
 * `share` engines of each (fewer when device memory is short) solve the
 * given system at once, and the layout with the highest measured solves/s
 * replaces the plan's engine, with the plan's accuracy settings and
 * concurrency `share`.  The choice is appended to the text file cache_path
 * (NULL: no cache) under a hash of the pattern and ordering; a later call
 * for the same pattern and share takes it from there without timing (the
 * values may then be NULL).  Synchronous; holds the GPU for seconds to
 * minutes on large patterns. */
typedef struct hykkt_tune_info {
  int from_cache;            /* 1: the layout came from the cache file, nothing was timed */
  int candidates;            /* layouts timed */
  int concurrent;            /* engines solving at once while timing */
  int solve_piece;           /* chosen: most columns of one solve item (0 = whole supernodes) */
  int warp_subtree;          /* chosen: most warp items per subtree task (0 = none) */
  int chunk_fma;             /* chosen: multiply-adds per product task */
  double best_solves_per_s;  /* measured throughput of the chosen layout */
  int cand_piece[8], cand_subtree[8], cand_chunk_fma[8];
  double solves_per_s[8];    /* measured throughput of each candidate (0: a solve failed) */
} hykkt_tune_info;
int hykkt_plan_autotune(hykkt_plan_t plan, const double* h_vals, const double* ds_vals, const double* jc_vals,
                        const double* jd_vals, const double* rx, const double* rs, const double* ry,
                        const double* ryd, int share, const char* cache_path, hykkt_tune_info* info);
/* No counterpart in the reference.  `share` = number of plans that solve
 * concurrently on this GPU: the plan's persistent triangular-solve kernels
 * take 1/share of the GPU's CTA slots (at least one per SM).  Default 1. */
int hykkt_plan_set_concurrency(hykkt_plan_t plan, int share);
/* One numeric solve (the numeric phase of HykktSolver::execute,
 * HykktSolver.cpp:252-285).  values_on_device = 0: the ten arrays are host
 * memory (copied through pinned staging); 1: device memory.  y0 (initial dy
 * of the CG, set_y_host) may be NULL for zeros.  stream: cudaStream_t or NULL.
 * sync = 0 returns after enqueueing (call hykkt_plan_wait before reading). */
int hykkt_plan_solve(hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                     const double* jc_vals, const double* jd_vals, const double* rx,
                     const double* rs, const double* ry, const double* ryd, const double* y0,
                     int values_on_device, void* stream, int sync);
int hykkt_plan_wait(hykkt_plan_t plan, void* stream);
/* Copy the solution (original ordering, unscaled). to_device = 1 for device
 * destination pointers. */
int hykkt_plan_get_solution(hykkt_plan_t plan, double* x, double* ds, double* y, double* yd,
                            int to_device, void* stream);
int hykkt_plan_get_info(hykkt_plan_t plan, hykkt_info* info);
int hykkt_plan_set_gamma(hykkt_plan_t plan, double gamma);
/* Accuracy controls (additions over the reference, whose values are
 * cg_itmax = 100, cg_rtol = 0, refine_max = 0; SchurCG.hpp:125-126):
 * CG stops when sqrt(r.r) < cg_rtol * ||r0|| (cg_rtol > 0; the reference's
 * absolute test sqrt(r.r) < 1e-12 when cg_rtol = 0) or after cg_itmax
 * iterations; then up to refine_max corrections on the full 4x4 KKT system
 * (residual right-hand side, same factorization) run while the relative
 * residual is above refine_target. */
int hykkt_plan_set_accuracy(hykkt_plan_t plan, int cg_itmax, double cg_rtol, int refine_max,
                            double refine_target);
/* No counterpart in the reference.  Relative CG tolerance of the refinement
 * corrections (set_accuracy sets it equal to cg_rtol): a correction only has
 * to reduce the residual by a few orders of magnitude. */
int hykkt_plan_set_refine_rtol(hykkt_plan_t plan, double rtol);
/* Regularization (the reference's add_diag step, HykktSolver.cpp:392, called
 * there with 0): delta >= 0 is added to the diagonal entries of Hgamma that
 * the pattern holds before the factorization, H_delta = Hgamma + delta I.
 * The CG and the recovery then use H_delta; the 4-block residual is always
 * that of the unregularized system, so refinement corrections (set_accuracy)
 * remove the perturbation.  Kept for later solves; clones inherit it. */
int hykkt_plan_set_delta(hykkt_plan_t plan, double delta);
/* An interior-point method's inertia-correction loop: solves; while the
 * factorization reports HYKKT_NOT_SPD, sets delta to delta_first (from 0) or
 * multiplies it by growth, up to delta_max, and solves again (synchronous).
 * Returns the last solve's status; *delta_used receives the delta of that
 * solve, which stays set on the plan. */
int hykkt_plan_solve_regularized(hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                                 const double* jc_vals, const double* jd_vals, const double* rx,
                                 const double* rs, const double* ry, const double* ryd, const double* y0,
                                 int values_on_device, void* stream, double delta_first, double delta_max,
                                 double growth, double* delta_used);
int hykkt_solver_set_accuracy(hykkt_solver_t s, int cg_itmax, double cg_rtol, int refine_max,
                              double refine_target);
/* Permutation used by the plan (perm[new] = old), n_x entries. */
int hykkt_plan_get_perm(hykkt_plan_t plan, int* perm);
/* Structural factor pattern L (lower, by columns, permuted numbering):
 * with cp == NULL returns nnz in *nnz; else fills cp (n_x+1) and ri (nnz). */
int hykkt_plan_get_L_pattern(hykkt_plan_t plan, int* cp, int* ri, int64_t* nnz);
/* Elimination tree parent (permuted numbering, -1 = root), n_x entries. */
int hykkt_plan_get_etree(hykkt_plan_t plan, int* parent);
/* Uncaptured run up to a stage (1: H~/Ruiz/Hgamma, 2: + factorization,
 * 3: full solve) with per-stage times in ms (5 entries: numeric, factor,
 * CG setup, CG loop, recovery+residual).  Inputs from the last upload. */
int hykkt_plan_run_stages(hykkt_plan_t plan, int upto, float* stage_ms);
/* Copy an internal device array (test hook): "ht_v" (H~ values in the H~
 * pattern), "jc_s", "ry_s", "rxt", "max_d", "lp_v" (permuted lower Hgamma,
 * CSC), "rxp", "hrxp", "schur", "x", "s", "y", "yd". */
int hykkt_plan_debug_read(hykkt_plan_t plan, const char* what, double* out, int64_t n);
/* Test hooks for the bounded device waits (no counterpart in the reference):
 * "spin_limit" = polls before a triangular-solve wait gives up (0 restores
 * the default, 2^24 polls of >= 64 ns); "unsatisfiable_waits" = 1 makes every
 * wait ask for one signal more than will come, so the next solve stops after
 * one spin limit with HYKKT_TIMEOUT (a timed-out solve stops its CG and
 * refinement loops; its results are invalid); 0 restores normal solving.
 * Either setting rebuilds the plan's graph on the next solve. */
int hykkt_plan_debug_set(hykkt_plan_t plan, const char* what, double value);
/* Sizes of the plan's internal patterns: H~ nnz, permuted-lower Hgamma nnz. */
int hykkt_plan_get_sizes(hykkt_plan_t plan, int64_t* sizes /* 8 entries */);
/* H~ pattern (full, n_x rows) and the permuted lower Hgamma CSC pattern. */
int hykkt_plan_get_patterns(hykkt_plan_t plan, int* ht_rp, int* ht_ci, int* lp_cp, int* lp_row);
/* Per-kernel device time of one uncaptured solve (CUDA events around every
 * launch on the plan's stream).  Writes a JSON object
 * {"kernel": [launches, total_ms, flops, bytes], ...} into buf (cap bytes);
 * flops/bytes are the algorithmic work of those launches (0 when not modelled). */
int hykkt_plan_profile(hykkt_plan_t plan, int upto, char* buf, int cap);
/* Average device time (ms) of one forward+backward triangular solve pair
 * with the current factor (after a solve). */
int hykkt_plan_time_trisolve(hykkt_plan_t plan, int nrep, float* ms);
/* Device time (ms) of one forward + backward solve pair of each of n plans of
 * one pattern (after a solve of each): mode 0 = one lockstep launch per
 * direction over all plans, 1 = each plan's kernels on its own stream,
 * 2 = one plan after another.  Measurement builds only (built with
 * HYKKT_MEASURE=1); otherwise HYKKT_INVALID. */
int hykkt_plans_time_trisolve(hykkt_plan_t* plans, int n, int nrep, int mode, float* ms);
/* Timeline of one forward + backward triangular solve of the current factor
 * (no counterpart in the reference; tracing aid).  Per task of the persistent
 * solve kernels, forward tasks first: {claimed, dependencies met, done} in ns
 * of the GPU global timer and the SM id.  *n receives 4 x tasks; out may be
 * NULL to query the size.  Measurement builds only (built with
 * HYKKT_MEASURE=1); otherwise HYKKT_INVALID. */
int hykkt_plan_trace_trisolve(hykkt_plan_t plan, unsigned long long* out, int64_t cap, int64_t* n);
/* Time `nsteps` back-to-back graph replays of the numeric solve on device-
 * resident inputs; writes per-step milliseconds. */
int hykkt_plan_time_solves(hykkt_plan_t plan, int nsteps, float* ms_per_step, void* stream);

/* ---- served solves (no counterpart in the reference, which is single-
 * threaded on the default stream, src/HykktSolver.cpp:18-34) -------------
 * A thread-safe request queue over plans: any host thread submits a solve of
 * one of its plans with borrowed host buffers and receives a ticket; worker
 * threads (one CUDA stream each) take requests in arrival order, skipping
 * requests whose plan another worker is solving, so one plan's requests
 * complete in submission order and different plans solve concurrently.  The
 * buffers stay borrowed until hykkt_server_wait returns for the ticket.
 * Size the plans for the worker count: hykkt_plan_set_concurrency(plan, W). */
typedef struct hykkt_server_s* hykkt_server_t;
int hykkt_server_create(int workers, hykkt_server_t* server);
/* Hook for tests and embedding: each request calls fn(user, plan, worker,
 * inputs[9], outputs[4]) on the worker thread instead of the GPU solve (plan
 * handles are then opaque keys); fn returns the request's status. */
typedef int (*hykkt_serve_fn)(void* user, hykkt_plan_t plan, int worker, const double* const* inputs,
                              double* const* outputs);
int hykkt_server_create_ex(int workers, hykkt_serve_fn fn, void* user, hykkt_server_t* server);
/* Admission by device memory: the server keeps at most budget_bytes of plan
 * device storage resident (0: 90% of the free device memory at creation).
 * A request whose plan is not resident is admitted when the plan fits beside
 * the resident ones, after evicting idle plans (least recently used; plans
 * without queued requests first); otherwise it is deferred, and the oldest
 * deferred request reserves its bytes so that newer ones cannot starve it.
 * Requests of a plan larger than the budget complete with HYKKT_OOM.  Plans
 * may be created deferred (hykkt_plan_create_deferred) or resident; eviction
 * is hykkt_plan_release_device, admission hykkt_plan_reload_device.  The
 * hooks (NULL for those calls) let tests and embedders run the policy on
 * stand-in plans; fn as in hykkt_server_create_ex. */
typedef struct hykkt_server_memory {
  int64_t budget_bytes;
  int64_t (*bytes_fn)(void* user, hykkt_plan_t plan);  /* device bytes of a plan when resident */
  int (*resident_fn)(void* user, hykkt_plan_t plan);   /* 1: resident when first seen */
  int (*load_fn)(void* user, hykkt_plan_t plan);       /* allocate; returns a status */
  int (*evict_fn)(void* user, hykkt_plan_t plan);      /* release; returns a status */
  void* user;
} hykkt_server_memory;
int hykkt_server_create_managed(int workers, hykkt_serve_fn fn, void* user, const hykkt_server_memory* mem,
                                hykkt_server_t* server);
/* Heavy requests: requests of plans whose device storage is at least
 * heavy_bytes run on at most max_heavy (1..workers) workers at a time, in
 * arrival order among themselves, so that the other workers stay free for
 * smaller plans, whose solves then run on a high-priority stream (their
 * kernels' blocks are scheduled ahead of the heavy solves'; no counterpart
 * in the single-threaded reference).
 * heavy_bytes <= 0 removes the limit (the default).  A server with a
 * stand-in solve function needs a managed server's bytes hook for it. */
int hykkt_server_set_heavy(hykkt_server_t server, int64_t heavy_bytes, int max_heavy);
/* Memory accounting of a managed server: budget, bytes resident now and at
 * most, plans resident, admissions (allocations), evictions, deferrals. */
int hykkt_server_memory_stats(hykkt_server_t server, int64_t* budget, int64_t* resident_bytes, int64_t* peak_bytes,
                              int64_t* resident_plans, int64_t* admissions, int64_t* evictions,
                              int64_t* deferrals);
/* Inputs as hykkt_plan_solve (host memory; y0 may be NULL); outputs as
 * hykkt_plan_get_solution (host memory). */
int hykkt_server_submit(hykkt_server_t server, hykkt_plan_t plan, const double* h_vals, const double* ds_vals,
                        const double* jc_vals, const double* jd_vals, const double* rx, const double* rs,
                        const double* ry, const double* ryd, const double* y0, double* x, double* ds, double* y,
                        double* yd, int64_t* ticket);
/* Blocks until the ticket's solve completed; solve_status receives the
 * solve's status (its message through hykkt_last_error on this thread),
 * latency_ms the time from submission to completion (queueing included),
 * info the plan's statistics of that solve.  Each ticket is collected once,
 * by one thread: a second thread waiting for the same ticket gets
 * HYKKT_INVALID. */
int hykkt_server_wait(hykkt_server_t server, int64_t ticket, int* solve_status, double* latency_ms,
                      hykkt_info* info);
/* hykkt_server_wait plus where the latency went (phases_ms, 3 entries):
 * queued (submission until a worker took the request), admission (evictions
 * and the allocation of the plan's device storage) and solve (the numeric
 * solve and the copy of the solution). */
int hykkt_server_wait_phases(hykkt_server_t server, int64_t ticket, int* solve_status, double* latency_ms,
                             hykkt_info* info, double* phases_ms);
/* Withdraws a request that no worker has taken yet: *cancelled = 1 and its
 * wait returns HYKKT_CANCELLED.  A request already being solved (or done)
 * completes as usual: *cancelled = 0.  The ticket is still collected by a
 * wait either way. */
int hykkt_server_cancel(hykkt_server_t server, int64_t ticket, int* cancelled);
int hykkt_server_poll(hykkt_server_t server, int64_t ticket, int* done);
int hykkt_server_stats(hykkt_server_t server, int64_t* completed, int64_t* queued, int64_t* in_flight);
/* Completes every submitted request, stops the workers and frees the server.
 * Waits already inside hykkt_server_wait return first; no other call on the
 * server may start once destroy has begun. */
int hykkt_server_destroy(hykkt_server_t server);

/* Host-only symbolic analysis (no GPU needed): the same integer work as
 * hykkt_plan_create -- H~ and Hgamma patterns (SpgemmClass symbolic,
 * src/SpgemmClass.cpp:96-143), ordering (PermClass::symamd,
 * src/PermClass.cpp:71-99), elimination tree, column counts and supernodes
 * (the analysis cusolverSpXcsrcholAnalysis performs, CholeskyClass.cpp:31-58). */
typedef struct hykkt_symbolic_s* hykkt_symbolic_t;
int hykkt_symbolic_create(hykkt_symbolic_t* sym, int n_x, int m_c, int m_d,
                          const int* h_rowptr, const int* h_colidx, int nnz_h,
                          const int* ds_rowptr, const int* ds_colidx, int nnz_ds,
                          const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                          const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                          int ordering, const int* perm);
/* hykkt_symbolic_create with the solve_piece option of hykkt_plan_create_ex
 * (no counterpart in the reference). */
int hykkt_symbolic_create_ex(hykkt_symbolic_t* sym, int n_x, int m_c, int m_d,
                             const int* h_rowptr, const int* h_colidx, int nnz_h,
                             const int* ds_rowptr, const int* ds_colidx, int nnz_ds,
                             const int* jc_rowptr, const int* jc_colidx, int nnz_jc,
                             const int* jd_rowptr, const int* jd_colidx, int nnz_jd,
                             int ordering, const int* perm, int solve_piece);
void hykkt_symbolic_destroy(hykkt_symbolic_t sym);
/* Integer arrays by name: "perm", "etree", "colcount", "ht_rp", "ht_ci",
 * "hg_rp", "hg_ci", "lp_cp", "lp_row", "L_cp", "L_ri", "sn_first",
 * "sn_parent", "sn_nrows", "sn_rows".  Returns the length (or -1). */
int64_t hykkt_symbolic_size(hykkt_symbolic_t sym, const char* what);
int hykkt_symbolic_get(hykkt_symbolic_t sym, const char* what, int* out, int64_t n);
/* Same getters on a plan's symbolic part. */
int64_t hykkt_plan_symbolic_size(hykkt_plan_t plan, const char* what);
int hykkt_plan_symbolic_get(hykkt_plan_t plan, const char* what, int* out, int64_t n);

/* Measured FP64 FMA throughput of this GPU (TFLOP/s): a kernel of
 * independent DFMA chains on every SM, timed with CUDA events. */
int hykkt_fp64_peak(double* tflops);
/* No counterpart in the reference.  FP64 throughput probes (TFLOP/s, CUDA
 * events, best of five): mode 0 = independent DFMA chains (hykkt_fp64_peak),
 * 1 = independent chains of FP64 mma.sync m8n8k4 (the tensor pipe's FP64
 * form on this GPU; tcgen05 has no FP64 kind), 2 = half the warps of each
 * kind in one kernel (shows whether the two compete for one pipe). */
int hykkt_fp64_probe(int mode, double* tflops);

/* ===========================================================================
 * 3. Components
 * ======================================================================== */
/* PermClass::invert_perm + vec_map_rc / vec_map_c / vec_map_r
 * (reference src/permcheck.cu:99-195, PermClass.cpp:101-123).  Host integer
 * work.  Outputs: rc_rows (n+1), rc_cols, rc_map (nnz_a); c_cols, c_map
 * (nnz_j); r_rows (m_j+1), r_cols, r_map (nnz_j).  Any output group may be
 * NULL to skip it. */
int hykkt_perm_maps(int n, const int* perm,
                    const int* a_rows, const int* a_cols, int nnz_a,
                    int n_j, const int* j_rows, const int* j_cols, int nnz_j,
                    int m_j, const int* jt_rows, const int* jt_cols,
                    int* rev_perm, int* rc_rows, int* rc_cols, int* rc_map,
                    int* c_cols, int* c_map, int* r_rows, int* r_cols, int* r_map);
/* Device gather new[i] = old[map[i]] (permcheck.cu:4-19). */
int hykkt_map_index(int n, const int* d_map, const double* d_old, double* d_new, void* stream);

/* RuizClass::ruiz_scale (RuizClass.cpp:54-88): `its` sweeps of Ruiz scaling
 * on the device arrays of [A B^T; B 0] (A n x n rows a_*, B^T n rows bt_*, B
 * m rows b_*), in place on the values and on rhs1 (n), rhs2 (m); max_d
 * (n+m) receives the aggregated scaling.  Device pointers. */
int hykkt_ruiz_scale(int its, int n, int m,
                     double* a_v, const int* a_i, const int* a_j,
                     double* bt_v, const int* bt_i, const int* bt_j,
                     double* b_v, const int* b_i, const int* b_j,
                     double* rhs1, double* rhs2, double* max_d, void* stream);

/* No counterpart in the reference.  hykkt_ruiz_scale without any device
 * allocation, for callers that must not touch the allocator where they scale
 * (a solver loop that reserves all of its device memory up front).  The n+m
 * scale vector lives in a fixed array inside the library: n + m must not
 * exceed hykkt_ruiz_scale_noalloc_max_rows() (1,048,576), else HYKKT_INVALID
 * and nothing is enqueued.  The first call on a device sets up the array's
 * address on it (make it before any stream capture); that address is kept
 * for the life of the process's context, so do not call this entry point
 * after a cudaDeviceReset of the device.  Calls that overlap in
 * time on one device race on the array.  Enqueues only: synchronise `stream`
 * before reading the results. */
int hykkt_ruiz_scale_noalloc(int its, int n, int m,
                             double* a_v, const int* a_i, const int* a_j,
                             double* bt_v, const int* bt_i, const int* bt_j,
                             double* b_v, const int* b_i, const int* b_j,
                             double* rhs1, double* rhs2, double* max_d, void* stream);
int hykkt_ruiz_scale_noalloc_max_rows(void);

/* CholeskyClass (CholeskyClass.cpp): sparse Cholesky of an SPD matrix given
 * by a host CSR pattern whose lower triangle is read (full or lower-only
 * storage both work).  ordering: HYKKT_ORDER_* (the reference factors in the
 * given order: HYKKT_ORDER_IDENTITY). */
typedef struct hykkt_chol_s* hykkt_chol_t;
int hykkt_chol_create(hykkt_chol_t* c, int n, int nnz, const int* rowptr, const int* colidx, int ordering);
/* numerical_factorization on host values (nnz, CSR order) */
int hykkt_chol_factor(hykkt_chol_t c, const double* vals);
/* solve(x, b) on host vectors (n) */
int hykkt_chol_solve(hykkt_chol_t c, double* x, const double* b);
void hykkt_chol_destroy(hykkt_chol_t c);

/* SchurComplementConjugateGradient::setup+solve (SchurCG.cpp:89-194): CG on
 * S = Jc H^{-1} Jc^T with the factor c (same ordering as c), host inputs.
 * x (m rows of Jc) holds x0 on entry and the solution on exit. */
int hykkt_schur_cg(hykkt_chol_t c, int m, int n, const int* jc_rowptr, const int* jc_colidx,
                   const double* jc_vals, int nnz_jc, const double* b, double* x,
                   int itmax, double tol, int* iterations, double* final_err);

#ifdef __cplusplus
}
#endif
#endif /* HYKKT_GB300_H */
