// Device engine of the KKT solve path: one Engine per sparsity pattern holds
// the symbolic plan mirrored in HBM, the per-system numeric buffers and the
// captured CUDA graph of one full solve.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "symbolic.hpp"

namespace hykkt {

// Status codes (mirrored by include/hykkt_gb300.h)
enum Status : int {
  ST_OK = 0,
  ST_NOT_SPD = 1,
  ST_CG_NOT_CONVERGED = 2,
  ST_PATTERN_CHANGED = 3,
  ST_OOM = 4,
  ST_TIMEOUT = 5,
  ST_INVALID = 6,
  ST_CUDA_ERROR = 7,
  ST_RESIDUAL_FAILED = 8,
  ST_NOT_READY = 9,
  ST_ACCURACY_NOT_MET = 10,
  ST_CANCELLED = 11,  // served requests only
};

// Scalars that live on the device during one solve.
struct DevScalars {
  double gam, gam1, delta, alpha, beta;  // CG recurrence (SchurCG.cpp:102-194)
  double cg_err;                         // final sqrt(r.r)
  int it;                                // CG iterations performed
  int stop;                              // CG converged (1), budget exhausted (2), a solve wait gave up (3)
  int pivot_col;                         // first column with a non-positive / tiny pivot, INT_MAX if none
  int cond_calls;                        // while-loop bodies executed (hang guard)
  int it_total;                          // CG iterations over the solve and its refinement steps
  int refine_it;                         // refinement corrections applied
  int refine_calls;                      // refinement loop bodies executed (hang guard)
  int stop_main;                         // CG runs that used their whole iteration budget
  int solve_flags;                       // bit 0: a triangular-solve wait hit its spin limit
  double gam0;                           // r0.r0 of the current CG run
  double rtol_cur;                       // relative tolerance of the current CG run
  // residual pieces (sums of squares): rx, rs, rc, rd, res1, res2, res3, res4
  double nrm[8];
  double rel_res_ref;   // reference definition: rows 1 and 3 (HykktSolver.cpp:846-930)
  double rel_res_full;  // all four block rows
  double rel_res_first; // full residual before refinement
  double rel_res_prev;  // full residual before the latest refinement step
  unsigned int ticket[8];  // last-block reduction tickets
};

// Device pointers of the plan (symbolic arrays) and of the numeric buffers.
struct DevPlan {
  int n_x, m_c, m_d;
  int nnz_h, nnz_jc, nnz_jd, nnz_ds, nnz_ht, nnz_lo;
  int jd_flag;
  double gamma;
  double cg_tol;          // absolute CG tolerance on ||r|| (reference: 1e-12)
  double cg_rtol;         // relative CG tolerance on ||r||/||r0|| (reference: 0)
  double cg_rtol_refine;  // the same for the CG runs of refinement corrections
  int cg_itmax;           // reference: 100
  int refine_max;         // refinement corrections on the full KKT (reference: 0)
  double delta;           // added to the diagonal of Hgamma before the factorization (reference: 0)
  double refine_target;   // stop refining below this relative residual
  double pivot_tol;
  unsigned spin_limit;    // polls before a triangular-solve wait gives up (kSpinLimit)
  int dbg_unsatisfiable;  // test hook: added to every wait's count (0 in use)

  // inputs (device copies)
  const int *h_rp, *h_ci;
  const int *jc_rp, *jc_ci;
  const int *jd_rp, *jd_ci;
  const int *jct_rp, *jct_ci, *jct_src;   // Jc^T rows by original column: Jc row, source index into Jc values
  const int *jdt_rp, *jdt_ci, *jdt_src;
  double *h_v, *ds_v, *jc_v, *jd_v;      // values as given (unscaled)
  double *rx, *rs, *ry, *ryd, *y0;       // rhs and initial y
  // H~
  const int *ht_rp, *ht_ci, *ht_hsrc, *ht_cp, *ht_ca, *ht_cb, *ht_ck;
  double* ht_v;
  // Ruiz
  double *scale, *max_d;
  double *jc_s;                          // scaled Jc values
  double *rxt;                           // r~x, scaled in place
  double *ry_s;                          // scaled copy of ry
  // Hgamma lower (permuted CSC)
  const int *lp_cp, *lp_row, *lp_htsrc, *lp_ccp, *lp_ca, *lp_cb, *lp_lrow;
  double* lp_v;
  const int *perm, *rev_perm;
  // permuted Jc
  const int *jcp_ci;
  const int *jctp_rp, *jctp_ci, *jctp_src;
  // supernodes
  int nsn;
  const int *sn_first, *sn_nrows, *sn_rp, *sn_rows, *sn_child_rp, *sn_children, *sn_relp, *sn_rel;
  const int64_t* sn_off;
  double* front;
  // solve items
  const int *sq_sn, *sq_c0, *sq_c1;
  const int64_t* sq_uoff;
  const int* g_rp;
  const int64_t* g_pos;
  double* u;
  double* part;  // backward partial sums (one vector per chunk)
  double* sv;    // per solve: b' (forward) / y' (backward) of the large items, n_x
  double* sv2;   // per solve: x of the staged items without rows below, written by the
                 // forward pass (their backward y' = x, read while x is overwritten), n_x
  unsigned long long* trace;  // optional per-task timeline of the solve kernels (null: off)
  double* dinv;              // inverses of the items' diagonal blocks (nc x nc, column-major)
  const int64_t* dinv_off;   // nsq+1 offsets into dinv
  double* xpanel;            // row panels of the large items' X (forward and transposed)
  double *l21f, *l21b;       // packed rows-below blocks of panelized items (forward chunks, backward panels)
  double* ppart;             // partial sums of the panel units
  const int64_t* xp_off;     // per item offset into xpanel (-1: small item)
  // vectors
  double *rxp;    // permuted r^x
  double *hrxp;   // Hgamma^-1 rxp
  double *schur;  // CG rhs
  double *cg_x;   // CG iterate (= y in scaled space)
  double *cg_r, *cg_w, *cg_p, *cg_s;  // m_c
  double *cg_yv, *cg_z;               // n_x (permuted)
  double *tmp_n;                      // n_x scratch
  // solution (unscaled, original ordering)
  double *x, *s, *y, *yd;
  // refinement: residual blocks of the current solution and the correction
  double *rr_x, *rr_s, *rr_y, *rr_yd;
  double *dx, *ds, *dy, *dyd;
  double* red;   // reduction partials
  DevScalars* sc;
};

// Task schedule of the persistent triangular-solve kernels (see kernels.cuh
// and SolveTask in symbolic.hpp).
struct SolveSched {
  int nsq, nchunks, ntasks_f, ntasks_b;
  int unit_cols;                          // columns per INV / INVT unit
  const int *tf_kind, *tf_item, *tf_arg;  // forward tasks: kind, item, argument
  const int *tb_kind, *tb_item, *tb_arg;  // backward tasks
  const int *ch_row0, *ch_rows;           // rows below the item covered by each chunk
  const int64_t* ch_poff;                 // backward partial vector of each chunk
  const int *ch0, *nch;                   // chunks of each item (contiguous ids)
  const int* rows_x;                      // rows per INV / INVT / L21 task of each item
  const int* mode;                        // ItemMode of each item
  const int *wg_rp, *wg_item;             // warp-item groups
  const int *sg_rp, *sg_item, *sg_lvl;    // warp subtrees: members by level, root last
  int npanels;                            // row panels of the staged items
  int nfchunks;                           // forward row chunks (one counter each)
  const int64_t* fch_slot;                // per forward chunk: first partial slot entry, -1: one unit
  double* fslot;                          // forward chunks' unit partial sums
  const int64_t *l21f_off, *l21b_off;     // per item: packed rows-below block offsets (-1: not panelized)
  const int* bd_need;                     // per item: backward product tasks
  const int *sq_parent, *sq_rpar, *nchild;  // forward look-ahead (symbolic.hpp)
  const int* cd_rp;                       // per permuted column: child products
  const int64_t* cd_L;                    // per entry: offset of L(row, first child column) in the front arena
  const int *cd_ld, *cd_nc, *cd_x;        // per entry: leading dimension, child columns, child's first column
  const int *fch_row0, *fch_rows, *fch0, *nfch;
  const int *fct_rp, *fct_item, *fdiag_need;
  const int* pcoff;                       // per item: first panel counter
  const int64_t* ppoff;                   // per item: first partial slot in ppart
  const int* diag_need;                   // forward: chunks whose rows include the item's columns
  const int *ct_rp, *ct_item;             // chunk -> distinct items owning its rows
  const int *ic_rp, *ic_chunk;            // item -> chunks with rows in its columns
  int* cnt;  // [head_f, head_b, diag_cnt, g_done, inv_done, bg_cnt (nchunks), bd_cnt, red_done, invt_done, panel_f, panel_b]
};

// Work lists of the blocked inversion of the large items' diagonal blocks,
// per 32-row step.
struct InverseWork {
  std::vector<int> small;                    // items inverted by one CTA each (<= 64 columns)
  std::vector<int> big;                      // items inverted by the blocked steps
  std::vector<int> diag_q, diag_c;           // per CTA: item, first column of a kDiagCols-column tile
  std::vector<int> upd_q, upd_r, upd_c;      // per CTA: item, 64x64 tile origin
  std::vector<int> diag_off, upd_off;        // per step offsets (steps+1)
};

struct PanelWork {
  // flat work lists for the blocked large-front factorization, per (level, panel)
  std::vector<int> potrf_sn;                        // supernode per CTA
  std::vector<int> trsm_sn, trsm_row0;              // supernode, first row of the tile
  std::vector<int> upd_sn, upd_ti, upd_tj;          // supernode, tile row/col start (front-local)
  std::vector<int> potrf_off, trsm_off, upd_off;    // per step offsets (size steps+1)
  std::vector<int> step_level, step_panel;          // per step
};

struct KernelTime {
  std::string name;
  int launches;
  double ms;
  double flops;  // algorithmic work of all launches (0 when not modelled)
  double bytes;
};

class Engine {
 public:
  // defer_device: count the device storage but allocate none yet (the plan
  // starts released; the first solve or reload_device allocates it)
  Engine(Symbolic&& S, double gamma, const SymbolicOptions& opt, bool defer_device = false);
  ~Engine();

  // Copy the numeric inputs into the engine's device buffers (from host
  // memory through pinned staging, or device-to-device).
  int upload(const double* h_v, const double* ds_v, const double* jc_v, const double* jd_v,
             const double* rx, const double* rs, const double* ry, const double* ryd,
             const double* y0, bool on_device, cudaStream_t stream);
  // Upload + one full solve (graph replay); with sync, also reads the status.
  int solve(const double* h_v, const double* ds_v, const double* jc_v, const double* jd_v,
            const double* rx, const double* rs, const double* ry, const double* ryd,
            const double* y0, bool on_device, cudaStream_t stream, bool sync = true);
  int finish(cudaStream_t stream);  // synchronise and translate the status
  int get_solution(double* x, double* s, double* y, double* yd, bool to_device, cudaStream_t stream);
  // Uncaptured run up to a stage (1 numeric, 2 +factor, 3 full) with stage times.
  int run_direct(cudaStream_t stream, int upto, float* stage_ms);
  int trisolve(const double* b, double* x, cudaStream_t stream);
  float time_trisolve(cudaStream_t stream, int nrep);
  // One forward + backward solve with the per-task timeline recorded: per
  // task (forward tasks, then backward) {claimed, dependencies met, done,
  // SM id} with times in ns of the GPU's global timer.
  void trace_trisolve(cudaStream_t stream, std::vector<unsigned long long>& out);
  // Components: factor from permuted-lower values (host, lp order); CG on
  // S = Jc H^{-1} Jc^T with this factor.
  int factor_values(const double* lower_vals_host, cudaStream_t stream);
  int schur_cg(int m, const std::vector<int>& jc_rp, const std::vector<int>& jc_ci, const double* jc_v_host,
               const double* b_host, double* x_host, int itmax, double tol, int* iters, double* err,
               cudaStream_t stream);
  int ensure_graph();
  // Device time (ms) of one forward + backward solve pair of every engine
  // (plans of one pattern, each with its current factor): mode 0 = one
  // lockstep launch per direction over all plans (k_trsv_*_multi), 1 = each
  // plan's own kernels on its own stream, 2 = one plan after another.
  static float time_trisolve_group(const std::vector<Engine*>& es, int nrep, int mode, cudaStream_t st);
  cudaGraphExec_t graph_exec() const { return exec_dev_; }

  const Symbolic& sym() const { return S_; }
  double gamma() const { return gamma_; }
  void set_gamma(double g);
  int last_status() const { return last_status_; }
  DevScalars last_scalars() const { return last_sc_; }
  int64_t device_bytes() const { return dev_bytes_; }
  // device storage of this plan when resident (known before allocation)
  int64_t size_bytes() const { return size_bytes_; }
  bool resident() const { return resident_; }
  // Free every device array and the graph, keeping the host analysis and
  // the settings; reload_device (or the next solve) rebuilds them.  The
  // caller makes sure no work of this plan is in flight.
  void release_device();
  void reload_device();
  int kernels_per_solve() const { return kernels_per_solve_; }
  int kernels_per_iter() const { return kernels_per_iter_; }
  int kernels_per_refine() const { return kernels_per_refine_; }
  // CG budget and tolerance, refinement steps and target (reference
  // semantics: 100, 0, 0; SchurCG.hpp:125-126).
  void set_accuracy(int cg_itmax, double cg_rtol, int refine_max, double refine_target);
  void set_delta(double delta);
  double delta() const { return dp.delta; }
  // relative CG tolerance of the refinement corrections (default: cg_rtol)
  void set_refine_rtol(double rtol);
  // Number of plans expected to solve concurrently on this GPU (other
  // streams): the persistent solve kernels then take a 1/share part of the
  // CTA slots.  Rebuilds the solve graph on the next solve.
  void set_concurrency(int share);
  int concurrency() const { return share_; }
  const SymbolicOptions& options() const { return opt_; }
  void accuracy(int& cg_itmax, double& cg_rtol, int& refine_max, double& refine_target) const {
    cg_itmax = dp.cg_itmax;
    cg_rtol = dp.cg_rtol;
    refine_max = dp.refine_max;
    refine_target = dp.refine_target;
  }
  double refine_rtol() const { return dp.cg_rtol_refine; }
  // Test hooks: "spin_limit" (polls of a triangular-solve wait; 0 restores
  // the default) and "unsatisfiable_waits" (1: every wait asks for one more
  // signal than will come, so the next solve times out).  Rebuild the graph.
  void debug_set(const std::string& what, double value);
  int debug_read(const char* what, double* host_out, int64_t n);
  // Uncaptured run with CUDA events around every kernel launch, summed per kernel.
  int profile(cudaStream_t stream, int upto, std::vector<KernelTime>& out);

  DevPlan dp;  // device view

 private:
  void alloc_and_upload();
  cudaStream_t begin_upload();
  void upload_all();
  void wait_last_launch();
  static void copy_settings(const DevPlan& from, DevPlan& to);
  int64_t size_bytes_ = 0;
  bool resident_ = false;
  void record_numeric(cudaStream_t st);
  void record_factor(cudaStream_t st);
  void record_trisolve(cudaStream_t st, const double* b, double* x, int use_stop, bool reset = true);
  void record_cg_pre(cudaStream_t st, int zero_x0);
  void record_cg_body(cudaStream_t st, cudaGraphConditionalHandle h, bool with_cond);
  void record_post(cudaStream_t st, int correction);
  void record_correction_rhs(cudaStream_t st);
  void direct_cg_loop(cudaStream_t st);
  void capture_graph();
  void drop_graph();
  void capture_while(cudaStream_t st, cudaStream_t bs, int default_value,
                     const std::function<void(cudaStream_t, cudaGraphConditionalHandle)>& pre,
                     const std::function<void(cudaStream_t, cudaGraphConditionalHandle)>& body);

  Symbolic S_;
  SymbolicOptions opt_;
  double gamma_;
  std::vector<void*> allocs_;
  int64_t dev_bytes_ = 0;
  PanelWork pw_;
  const int *d_potrf_sn_ = nullptr, *d_trsm_sn_ = nullptr, *d_trsm_row0_ = nullptr;
  const int *d_upd_sn_ = nullptr, *d_upd_ti_ = nullptr, *d_upd_tj_ = nullptr;
  InverseWork iw_;
  const int *d_inv_small_ = nullptr, *d_inv_big_ = nullptr;
  const int *d_idiag_q_ = nullptr, *d_idiag_c_ = nullptr;
  const int *d_iupd_q_ = nullptr, *d_iupd_r_ = nullptr, *d_iupd_c_ = nullptr;
  const int *d_pack_q_ = nullptr, *d_pack_b_ = nullptr;
  int n_pack_ = 0;
  std::vector<int> l21_items_;  // panelized items (packed rows-below blocks)
  std::vector<const int*> d_small_, d_large_;
  std::vector<const int*> d_ea_sn_, d_ea_row0_;
  std::vector<int> n_ea_;
  SolveSched sched_{};
  int64_t cnt_ints_ = 0;
  int grid_f_ = 1, grid_b_ = 1;
  int sms_ = 1, occ_f_ = 1, occ_b_ = 1, share_ = 1;
  void size_solve_grids();
  int max_small_smem_ = 0;
  double* pin_in_ = nullptr;
  double* pin_out_ = nullptr;
  DevScalars* pin_sc_ = nullptr;
  cudaEvent_t last_launch_ = nullptr;  // recorded after each asynchronous graph launch
  int64_t pin_in_n_ = 0, pin_out_n_ = 0;
  cudaGraphExec_t exec_dev_ = nullptr;
  cudaGraph_t graph_dev_ = nullptr;
  cudaStream_t cap_stream_ = nullptr, body_stream_ = nullptr, body_stream2_ = nullptr;
  int last_status_ = ST_NOT_READY;
  DevScalars last_sc_{};
  int kernels_per_solve_ = 0;
  int kernels_per_iter_ = 0;
  int kernels_per_refine_ = 0;
  struct ProfEvent {
    const char* name;
    cudaEvent_t a, b;
  };
  bool prof_ = false;
  cudaEvent_t prof_open_ = nullptr;
  std::vector<ProfEvent> prof_events_;
  void prof_begin(cudaStream_t st);
  void prof_end(cudaStream_t st, const char* name);
  void prof_work(const char* name, double flops, double bytes);
  std::map<std::string, std::pair<double, double>> prof_work_;
};

// CUDA check helper
#define HYKKT_CUDA(call)                                                      \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") +   \
                                                    cudaGetErrorString(e_) +  \
                                                    " at " #call);            \
  } while (0)

}  // namespace hykkt
