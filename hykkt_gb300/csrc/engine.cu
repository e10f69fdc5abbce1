// Host orchestration of the device solve: HBM layout, level schedules and
// the CUDA graph of one full KKT solve (H~, Ruiz, Hgamma, multifrontal
// Cholesky, Schur CG as a device-side while loop, recovery, residual).
// The graph replaces the reference's per-call sequence of cuSPARSE/cuSOLVER/
// cuBLAS calls with host-synchronised dots (HykktSolver::execute,
// src/HykktSolver.cpp:240-286).
#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <climits>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "kernels.cuh"

namespace hykkt {

void raise_front_small_smem(int bytes);

std::mutex& cuda_setup_mutex() {
  static std::mutex m;
  return m;
}

namespace {
// counting pass (Engine::reload_device with count_only): sizes are summed,
// nothing is allocated or copied
thread_local bool g_count_only = false;
// the stream of the uploads and zero fills of Engine::alloc_and_upload: the
// solves run on non-blocking streams, which do not wait for work on the
// legacy default stream, so the set-up copies go to a stream of their own
// that is synchronized before the plan is used
thread_local cudaStream_t g_upload_stream = nullptr;

template <class T>
T* dev_upload(std::vector<void*>& allocs, int64_t& bytes, const std::vector<T>& v) {
  T* p = nullptr;
  size_t n = std::max<size_t>(v.size(), 1);
  if (g_count_only) {
    bytes += n * sizeof(T);
    return nullptr;
  }
  HYKKT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), n * sizeof(T), g_upload_stream));
  allocs.push_back(p);
  bytes += n * sizeof(T);
  if (!v.empty())
    HYKKT_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, g_upload_stream));
  return p;
}
template <class T>
T* dev_alloc(std::vector<void*>& allocs, int64_t& bytes, int64_t n) {
  T* p = nullptr;
  size_t m = std::max<int64_t>(n, 1);
  if (g_count_only) {
    bytes += m * sizeof(T);
    return nullptr;
  }
  HYKKT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), m * sizeof(T), g_upload_stream));
  allocs.push_back(p);
  bytes += m * sizeof(T);
  HYKKT_CUDA(cudaMemsetAsync(p, 0, m * sizeof(T), g_upload_stream));
  return p;
}
inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Frees a plan's device storage (stream-ordered allocations) on a stream of
// its own: unlike cudaFree, this waits for no other work on the device, so
// releasing one plan does not stall behind other plans' solves.  The caller
// has made sure that no kernel still uses the storage.
void free_storage(std::vector<void*>& allocs) {
  if (allocs.empty()) return;
  cudaStream_t fs = nullptr;
  if (cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    for (void* p : allocs) cudaFree(p);
  } else {
    for (void* p : allocs) cudaFreeAsync(p, fs);
    cudaStreamSynchronize(fs);
    cudaStreamDestroy(fs);
  }
  allocs.clear();
}
}  // namespace

Engine::Engine(Symbolic&& S, double gamma, const SymbolicOptions& opt, bool defer_device)
    : S_(std::move(S)), opt_(opt), gamma_(gamma) {
  // Front arena in level order: small fronts then large fronts of each level,
  // so the large fronts of one level form one contiguous range (one memset).
  {
    int64_t off = 0;
    std::vector<int64_t> noff(S_.nsn + 1, 0);
    for (int l = 0; l < S_.nlevels; ++l) {
      for (int J : S_.flevels[l].small) { noff[J] = off; off += (int64_t)S_.sn_nrows[J] * S_.sn_nrows[J]; }
      for (int J : S_.flevels[l].large) { noff[J] = off; off += (int64_t)S_.sn_nrows[J] * S_.sn_nrows[J]; }
    }
    noff[S_.nsn] = off;
    S_.sn_off = noff;
    S_.front_arena = off;
  }
  if (defer_device) {
    // the exact size, counted without allocating: admission decisions can be
    // made before the plan takes any device memory
    g_count_only = true;
    try {
      alloc_and_upload();
    } catch (...) {
      g_count_only = false;
      throw;
    }
    g_count_only = false;
    size_bytes_ = dev_bytes_;
    dev_bytes_ = 0;
    const DevPlan counted = dp;
    dp = DevPlan{};
    copy_settings(counted, dp);
    resident_ = false;
    return;
  }
  std::lock_guard<std::mutex> lk(cuda_setup_mutex());
  try {
    alloc_and_upload();
  } catch (...) {
    free_storage(allocs_);
    throw;
  }
  size_bytes_ = dev_bytes_;
  resident_ = true;
}

// the per-plan settings a DevPlan carries besides device pointers
void Engine::copy_settings(const DevPlan& from, DevPlan& to) {
  to.gamma = from.gamma;
  to.cg_tol = from.cg_tol;
  to.cg_rtol = from.cg_rtol;
  to.cg_rtol_refine = from.cg_rtol_refine;
  to.cg_itmax = from.cg_itmax;
  to.refine_max = from.refine_max;
  to.delta = from.delta;
  to.refine_target = from.refine_target;
  to.pivot_tol = from.pivot_tol;
  to.spin_limit = from.spin_limit;
  to.dbg_unsatisfiable = from.dbg_unsatisfiable;
}

// The last asynchronous graph launch (a solve returned without waiting)
// has finished: its kernels no longer touch the plan's storage.
void Engine::wait_last_launch() {
  if (last_launch_) cudaEventSynchronize(last_launch_);
}

// Releases the device storage.  The process-wide set-up lock is held only
// while the plan's bookkeeping changes; the frees run after it, on a stream
// of their own, so other plans' set-up does not wait for them.
void Engine::release_device() {
  if (!resident_) return;
  wait_last_launch();
  drop_graph();
  std::vector<void*> mine;
  {
    std::lock_guard<std::mutex> lk(cuda_setup_mutex());
    mine.swap(allocs_);
    dev_bytes_ = 0;
    const DevPlan keep = dp;
    dp = DevPlan{};
    copy_settings(keep, dp);
    sched_ = SolveSched{};
    resident_ = false;
  }
  free_storage(mine);
}

// Takes the device storage back: allocations and copies are enqueued under
// the set-up lock, and waited for after it is released.
void Engine::reload_device() {
  if (resident_) return;
  const DevPlan keep = dp;
  pw_ = PanelWork{};
  iw_ = InverseWork{};
  l21_items_.clear();
  cudaStream_t us = nullptr;
  {
    std::lock_guard<std::mutex> lk(cuda_setup_mutex());
    try {
      us = begin_upload();
    } catch (...) {
      free_storage(allocs_);
      dev_bytes_ = 0;
      dp = keep;  // still released, with its settings
      throw;
    }
  }
  const cudaError_t e = cudaStreamSynchronize(us);
  cudaStreamDestroy(us);
  if (e != cudaSuccess) {
    cudaGetLastError();
    free_storage(allocs_);
    dev_bytes_ = 0;
    dp = keep;
    HYKKT_CUDA(e);
  }
  copy_settings(keep, dp);
  size_bytes_ = dev_bytes_;
  resident_ = true;
}

Engine::~Engine() {
  wait_last_launch();
  std::lock_guard<std::mutex> lk(cuda_setup_mutex());
  if (exec_dev_) cudaGraphExecDestroy(exec_dev_);
  if (graph_dev_) cudaGraphDestroy(graph_dev_);
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
  if (last_launch_) cudaEventDestroy(last_launch_);
  free_storage(allocs_);
  if (pin_in_) cudaFreeHost(pin_in_);
  if (pin_out_) cudaFreeHost(pin_out_);
  if (pin_sc_) cudaFreeHost(pin_sc_);
  if (body_stream_) cudaStreamDestroy(body_stream_);
  if (body_stream2_) cudaStreamDestroy(body_stream2_);
}

// Drops the captured graph (rebuilt at the next solve).
void Engine::drop_graph() {
  std::lock_guard<std::mutex> lk(cuda_setup_mutex());
  if (exec_dev_) { cudaGraphExecDestroy(exec_dev_); exec_dev_ = nullptr; }
  if (graph_dev_) { cudaGraphDestroy(graph_dev_); graph_dev_ = nullptr; }
}

void Engine::set_gamma(double g) {
  gamma_ = g;
  dp.gamma = g;
  // kernels take the DevPlan by value: the captured graph must be rebuilt
  drop_graph();
}

// Allocates and fills the plan's device storage (or, counting, only sizes
// it); every allocation, copy and zero fill has completed when this returns.
void Engine::alloc_and_upload() {
  if (g_count_only) {
    upload_all();
    return;
  }
  cudaStream_t us = begin_upload();
  const cudaError_t e = cudaStreamSynchronize(us);
  cudaStreamDestroy(us);
  HYKKT_CUDA(e);
}

// Enqueues the allocations, copies and zero fills on a new stream and
// returns it; the caller synchronizes and destroys it before the plan is
// used.
cudaStream_t Engine::begin_upload() {
  cudaStream_t us = nullptr;
  HYKKT_CUDA(cudaStreamCreateWithFlags(&us, cudaStreamNonBlocking));
  g_upload_stream = us;
  try {
    upload_all();
  } catch (...) {
    g_upload_stream = nullptr;
    cudaStreamSynchronize(us);
    cudaStreamDestroy(us);
    throw;
  }
  g_upload_stream = nullptr;
  return us;
}

void Engine::upload_all() {
  const Symbolic& S = S_;
  auto& A = allocs_;
  int64_t& B = dev_bytes_;
  DevPlan d{};
  d.n_x = S.n_x; d.m_c = S.m_c; d.m_d = S.m_d;
  d.nnz_h = S.nnz_h; d.nnz_jc = S.nnz_jc; d.nnz_jd = S.nnz_jd; d.nnz_ds = S.nnz_ds;
  d.nnz_ht = S.Ht.nnz(); d.nnz_lo = S.lp_cp[S.n_x];
  d.jd_flag = S.jd_flag ? 1 : 0;
  d.gamma = gamma_;
  d.cg_tol = 1e-12;   // SchurCG.hpp:126
  d.cg_rtol = 0.0;
  d.cg_rtol_refine = 0.0;
  d.cg_itmax = 100;   // SchurCG.hpp:125
  d.refine_max = 0;   // the reference does not refine
  d.refine_target = 1e-10;
  d.pivot_tol = 1e-12;  // CholeskyClass.hpp:92 / HykktSolver.hpp:369
  d.spin_limit = kSpinLimit;
  d.dbg_unsatisfiable = 0;

  d.h_rp = dev_upload(A, B, S.H.rp); d.h_ci = dev_upload(A, B, S.H.ci);
  d.jc_rp = dev_upload(A, B, S.Jc.rp); d.jc_ci = dev_upload(A, B, S.Jc.ci);
  std::vector<int> jd_rp = S.Jd.rp.empty() ? std::vector<int>(S.m_d + 1, 0) : S.Jd.rp;
  d.jd_rp = dev_upload(A, B, jd_rp); d.jd_ci = dev_upload(A, B, S.Jd.ci);
  d.jct_rp = dev_upload(A, B, S.JcT.pat.rp); d.jct_ci = dev_upload(A, B, S.JcT.pat.ci); d.jct_src = dev_upload(A, B, S.JcT.src);
  std::vector<int> jdt_rp = S.jd_flag ? S.JdT.pat.rp : std::vector<int>(S.n_x + 1, 0);
  d.jdt_rp = dev_upload(A, B, jdt_rp); d.jdt_ci = dev_upload(A, B, S.JdT.pat.ci); d.jdt_src = dev_upload(A, B, S.JdT.src);
  d.h_v = dev_alloc<double>(A, B, S.nnz_h);
  d.ds_v = dev_alloc<double>(A, B, std::max(S.nnz_ds, S.m_d));
  d.jc_v = dev_alloc<double>(A, B, S.nnz_jc);
  d.jd_v = dev_alloc<double>(A, B, S.nnz_jd);
  d.rx = dev_alloc<double>(A, B, S.n_x);
  d.rs = dev_alloc<double>(A, B, S.m_d);
  d.ry = dev_alloc<double>(A, B, S.m_c);
  d.ryd = dev_alloc<double>(A, B, S.m_d);
  d.y0 = dev_alloc<double>(A, B, S.m_c);
  d.ht_rp = dev_upload(A, B, S.Ht.rp); d.ht_ci = dev_upload(A, B, S.Ht.ci);
  d.ht_hsrc = dev_upload(A, B, S.ht_hsrc); d.ht_cp = dev_upload(A, B, S.ht_cp);
  d.ht_ca = dev_upload(A, B, S.ht_ca); d.ht_cb = dev_upload(A, B, S.ht_cb); d.ht_ck = dev_upload(A, B, S.ht_ck);
  d.ht_v = dev_alloc<double>(A, B, S.Ht.nnz());
  d.scale = dev_alloc<double>(A, B, S.n_x + S.m_c);
  d.max_d = dev_alloc<double>(A, B, S.n_x + S.m_c);
  d.jc_s = dev_alloc<double>(A, B, S.nnz_jc);
  d.rxt = dev_alloc<double>(A, B, S.n_x);
  d.ry_s = dev_alloc<double>(A, B, S.m_c);
  d.lp_cp = dev_upload(A, B, S.lp_cp); d.lp_row = dev_upload(A, B, S.lp_row);
  d.lp_htsrc = dev_upload(A, B, S.lp_htsrc); d.lp_ccp = dev_upload(A, B, S.lp_ccp);
  d.lp_ca = dev_upload(A, B, S.lp_ca); d.lp_cb = dev_upload(A, B, S.lp_cb); d.lp_lrow = dev_upload(A, B, S.lp_lrow);
  d.lp_v = dev_alloc<double>(A, B, S.lp_cp[S.n_x]);
  d.perm = dev_upload(A, B, S.perm); d.rev_perm = dev_upload(A, B, S.rev_perm);
  d.jcp_ci = dev_upload(A, B, S.jcp_ci);
  d.jctp_rp = dev_upload(A, B, S.jctp_rp); d.jctp_ci = dev_upload(A, B, S.jctp_ci); d.jctp_src = dev_upload(A, B, S.jctp_src);
  d.nsn = S.nsn;
  d.sn_first = dev_upload(A, B, S.sn_first); d.sn_nrows = dev_upload(A, B, S.sn_nrows);
  d.sn_rp = dev_upload(A, B, S.sn_rp); d.sn_rows = dev_upload(A, B, S.sn_rows);
  d.sn_child_rp = dev_upload(A, B, S.sn_child_rp); d.sn_children = dev_upload(A, B, S.sn_children);
  d.sn_relp = dev_upload(A, B, S.sn_relp); d.sn_rel = dev_upload(A, B, S.sn_rel);
  d.sn_off = dev_upload(A, B, S.sn_off);
  d.front = dev_alloc<double>(A, B, S.front_arena);
  d.sq_sn = dev_upload(A, B, S.sq_sn); d.sq_c0 = dev_upload(A, B, S.sq_c0); d.sq_c1 = dev_upload(A, B, S.sq_c1);
  d.sq_uoff = dev_upload(A, B, S.sq_uoff);
  d.g_rp = dev_upload(A, B, S.g_rp); d.g_pos = dev_upload(A, B, S.g_pos);
  d.u = dev_alloc<double>(A, B, S.u_arena);

  // ---- factorization schedules -------------------------------------------
  d_small_.assign(S.nlevels, nullptr);
  d_large_.assign(S.nlevels, nullptr);
  d_ea_sn_.assign(S.nlevels, nullptr);
  d_ea_row0_.assign(S.nlevels, nullptr);
  n_ea_.assign(S.nlevels, 0);
  max_small_smem_ = 0;
  pw_ = PanelWork();
  pw_.potrf_off.push_back(0); pw_.trsm_off.push_back(0); pw_.upd_off.push_back(0);
  for (int l = 0; l < S.nlevels; ++l) {
    const FactorLevel& L = S.flevels[l];
    if (!L.small.empty()) d_small_[l] = dev_upload(A, B, L.small);
    for (int J : L.small) max_small_smem_ = std::max(max_small_smem_, S.sn_nrows[J] * S.sn_nrows[J] * 8);
    if (L.large.empty()) continue;
    d_large_[l] = dev_upload(A, B, L.large);
    std::vector<int> ea_sn, ea_row0;
    for (int J : L.large)
      for (int r = 0; r < S.sn_nrows[J]; r += kEaRows) { ea_sn.push_back(J); ea_row0.push_back(r); }
    n_ea_[l] = (int)ea_sn.size();
    d_ea_sn_[l] = dev_upload(A, B, ea_sn);
    d_ea_row0_[l] = dev_upload(A, B, ea_row0);
    for (int p = 0; p < L.max_panels; ++p) {
      for (int J : L.large) {
        const int ncols = S.sn_first[J + 1] - S.sn_first[J];
        const int nJ = S.sn_nrows[J];
        const int c0 = p * kPanel;
        if (c0 >= ncols) continue;
        const int w = std::min(kPanel, ncols - c0);
        pw_.potrf_sn.push_back(J);
        for (int r = c0 + w; r < nJ; r += kTrsmRows) { pw_.trsm_sn.push_back(J); pw_.trsm_row0.push_back(r); }
        for (int ti = c0 + w; ti < nJ; ti += kTile)
          for (int tj = c0 + w; tj <= ti; tj += kTile) {
            pw_.upd_sn.push_back(J); pw_.upd_ti.push_back(ti); pw_.upd_tj.push_back(tj);
          }
      }
      pw_.potrf_off.push_back((int)pw_.potrf_sn.size());
      pw_.trsm_off.push_back((int)pw_.trsm_sn.size());
      pw_.upd_off.push_back((int)pw_.upd_sn.size());
      pw_.step_level.push_back(l);
      pw_.step_panel.push_back(p);
    }
  }
  d_potrf_sn_ = dev_upload(A, B, pw_.potrf_sn);
  d_trsm_sn_ = dev_upload(A, B, pw_.trsm_sn); d_trsm_row0_ = dev_upload(A, B, pw_.trsm_row0);
  d_upd_sn_ = dev_upload(A, B, pw_.upd_sn); d_upd_ti_ = dev_upload(A, B, pw_.upd_ti); d_upd_tj_ = dev_upload(A, B, pw_.upd_tj);

  // ---- triangular-solve task schedule (persistent kernels) -------------------
  {
    const int nsq = S.nsq;
    const int nch = (int)S.ch_row0.size();
    SolveSched& ss = sched_;
    ss.nsq = nsq;
    ss.nchunks = nch;
    ss.ntasks_f = (int)S.tf_item.size();
    ss.unit_cols = S.unit_cols;
    ss.ntasks_b = (int)S.tb_item.size();
    ss.tf_kind = dev_upload(A, B, S.tf_kind); ss.tf_item = dev_upload(A, B, S.tf_item); ss.tf_arg = dev_upload(A, B, S.tf_arg);
    ss.tb_kind = dev_upload(A, B, S.tb_kind); ss.tb_item = dev_upload(A, B, S.tb_item); ss.tb_arg = dev_upload(A, B, S.tb_arg);
    ss.ch_row0 = dev_upload(A, B, S.ch_row0); ss.ch_rows = dev_upload(A, B, S.ch_rows);
    ss.ch_poff = dev_upload(A, B, S.ch_poff);
    ss.ch0 = dev_upload(A, B, S.ch0); ss.nch = dev_upload(A, B, S.nch);
    ss.rows_x = dev_upload(A, B, S.sq_rows_x);
    ss.mode = dev_upload(A, B, S.sq_mode);
    ss.wg_rp = dev_upload(A, B, S.wg_rp); ss.wg_item = dev_upload(A, B, S.wg_item);
    ss.sg_rp = dev_upload(A, B, S.sg_rp); ss.sg_item = dev_upload(A, B, S.sg_item); ss.sg_lvl = dev_upload(A, B, S.sg_lvl);
    ss.diag_need = dev_upload(A, B, S.diag_need);
    ss.ct_rp = dev_upload(A, B, S.ct_rp); ss.ct_item = dev_upload(A, B, S.ct_item);
    ss.ic_rp = dev_upload(A, B, S.ic_rp); ss.ic_chunk = dev_upload(A, B, S.ic_chunk);
    ss.npanels = S.npanels;
    ss.pcoff = dev_upload(A, B, S.sq_pcoff);
    ss.ppoff = dev_upload(A, B, S.sq_ppoff);
    d.ppart = dev_alloc<double>(A, B, std::max<int64_t>(S.ppart_arena, 1));
    ss.sq_parent = dev_upload(A, B, S.sq_parent); ss.sq_rpar = dev_upload(A, B, S.sq_rpar);
    ss.nchild = dev_upload(A, B, S.nchild);
    ss.cd_rp = dev_upload(A, B, S.cd_rp);
    {
      std::vector<int64_t> cdL(S.cd_loff.size());
      for (size_t e = 0; e < cdL.size(); ++e) cdL[e] = S.sn_off[S.sq_sn[S.cd_item[e]]] + S.cd_loff[e];
      ss.cd_L = dev_upload(A, B, cdL);
    }
    ss.cd_ld = dev_upload(A, B, S.cd_ld); ss.cd_nc = dev_upload(A, B, S.cd_nc); ss.cd_x = dev_upload(A, B, S.cd_x);
    ss.fch_row0 = dev_upload(A, B, S.fch_row0); ss.fch_rows = dev_upload(A, B, S.fch_rows);
    ss.fch0 = dev_upload(A, B, S.fch0); ss.nfch = dev_upload(A, B, S.nfch);
    ss.fct_rp = dev_upload(A, B, S.fct_rp); ss.fct_item = dev_upload(A, B, S.fct_item);
    ss.fdiag_need = dev_upload(A, B, S.fdiag_need);
    ss.l21f_off = dev_upload(A, B, S.sq_l21f);
    ss.l21b_off = dev_upload(A, B, S.sq_l21b);
    ss.bd_need = dev_upload(A, B, S.bd_need);
    d.l21f = dev_alloc<double>(A, B, std::max<int64_t>(S.l21f_arena, 1));
    d.l21b = dev_alloc<double>(A, B, std::max<int64_t>(S.l21b_arena, 1));
    for (int q = 0; q < nsq; ++q)
      if (S.sq_l21f[q] >= 0) l21_items_.push_back(q);
    ss.nfchunks = (int)S.fch_row0.size();
    ss.fch_slot = dev_upload(A, B, S.fch_slot);
    ss.fslot = dev_alloc<double>(A, B, std::max<int64_t>(S.fslot_arena, 1));
    cnt_ints_ = 2 + 7LL * nsq + nch + 2LL * S.npanels + ss.nfchunks;
    ss.cnt = dev_alloc<int>(A, B, cnt_ints_);
    d.dinv_off = dev_upload(A, B, S.sq_doff);
    d.dinv = dev_alloc<double>(A, B, S.dinv_arena);
    d.part = dev_alloc<double>(A, B, std::max<int64_t>(S.part_arena, 1));
    d.sv = dev_alloc<double>(A, B, S.n_x);
    d.sv2 = dev_alloc<double>(A, B, S.n_x);
    d.xp_off = dev_upload(A, B, S.sq_xpoff);
    d.xpanel = dev_alloc<double>(A, B, std::max<int64_t>(S.xpanel_arena, 1));
    for (int q = 0; q < nsq; ++q) {
      if (S.sq_rows_x[q] < 16 || S.sq_rows_x[q] > kBlock || (S.sq_rows_x[q] & (S.sq_rows_x[q] - 1)))
        throw std::runtime_error("solve schedule: rows per task must be a power of two in 16..256");
      const int nc = S.sq_c1[q] - S.sq_c0[q], nrow = S.sn_nrows[S.sq_sn[q]] - S.sq_c0[q];
      const int m = S.sq_mode[q];
      if ((m == ITEM_WARP && nrow > kWarpItemRows) || (m == ITEM_FUSED && (nc > kPiece || nrow > kSmallItemRows)) ||
          (m == ITEM_HEAD && nc > kPiece))
        throw std::runtime_error("solve schedule: item too large for its mode");
    }
    int dev = 0, sms = 0, bf = 0, bb = 0;
    HYKKT_CUDA(cudaGetDevice(&dev));
    HYKKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    HYKKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, k_trsv_fwd, kBlock, 0));
    HYKKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bb, k_trsv_bwd, kBlock, 0));
    sms_ = sms;
    occ_f_ = std::max(bf, 1);
    occ_b_ = std::max(bb, 1);
    size_solve_grids();

    // inversion of the diagonal blocks: small items one CTA each, large
    // items by 32-row steps batched over all of them
    iw_ = InverseWork();
    int steps = 0;
    for (int q = 0; q < nsq; ++q) {
      const int nc = S.sq_c1[q] - S.sq_c0[q];
      if (nc <= kPiece) iw_.small.push_back(q);
      else {
        iw_.big.push_back(q);
        steps = std::max(steps, (nc + kPanel - 1) / kPanel);
      }
    }
    iw_.diag_off.push_back(0);
    iw_.upd_off.push_back(0);
    for (int i = 0; i < steps; ++i) {
      for (int q : iw_.big) {
        const int nc = S.sq_c1[q] - S.sq_c0[q];
        const int b0 = i * kPanel;
        if (b0 >= nc) continue;
        const int cmax = std::min(nc, b0 + kPanel);
        for (int c = 0; c < cmax; c += kDiagCols) { iw_.diag_q.push_back(q); iw_.diag_c.push_back(c); }
        for (int r = b0 + kPanel; r < nc; r += kTile)
          for (int c = 0; c < cmax; c += kTile) { iw_.upd_q.push_back(q); iw_.upd_r.push_back(r); iw_.upd_c.push_back(c); }
      }
      iw_.diag_off.push_back((int)iw_.diag_q.size());
      iw_.upd_off.push_back((int)iw_.upd_q.size());
    }
    d_inv_small_ = dev_upload(A, B, iw_.small);
    d_inv_big_ = dev_upload(A, B, iw_.big);
    d_idiag_q_ = dev_upload(A, B, iw_.diag_q); d_idiag_c_ = dev_upload(A, B, iw_.diag_c);
    d_iupd_q_ = dev_upload(A, B, iw_.upd_q); d_iupd_r_ = dev_upload(A, B, iw_.upd_r); d_iupd_c_ = dev_upload(A, B, iw_.upd_c);
    std::vector<int> pack_q, pack_b;
    for (int q = 0; q < nsq; ++q) {
      if (S.sq_mode[q] != ITEM_STAGED) continue;
      const int nc = S.sq_c1[q] - S.sq_c0[q];
      for (int b = 0; b * S.sq_rows_x[q] < nc; ++b) { pack_q.push_back(q); pack_b.push_back(b); }
    }
    n_pack_ = (int)pack_q.size();
    d_pack_q_ = dev_upload(A, B, pack_q);
    d_pack_b_ = dev_upload(A, B, pack_b);
  }

  // ---- vectors ---------------------------------------------------------------
  d.rxp = dev_alloc<double>(A, B, S.n_x);
  d.hrxp = dev_alloc<double>(A, B, S.n_x);
  d.schur = dev_alloc<double>(A, B, S.m_c);
  d.cg_x = dev_alloc<double>(A, B, S.m_c);
  d.cg_r = dev_alloc<double>(A, B, S.m_c);
  d.cg_w = dev_alloc<double>(A, B, S.m_c);
  d.cg_p = dev_alloc<double>(A, B, S.m_c);
  d.cg_s = dev_alloc<double>(A, B, S.m_c);
  d.cg_yv = dev_alloc<double>(A, B, S.n_x);
  d.cg_z = dev_alloc<double>(A, B, S.n_x);
  d.tmp_n = dev_alloc<double>(A, B, S.n_x);
  d.x = dev_alloc<double>(A, B, S.n_x);
  d.s = dev_alloc<double>(A, B, S.m_d);
  d.y = dev_alloc<double>(A, B, S.m_c);
  d.yd = dev_alloc<double>(A, B, S.m_d);
  d.rr_x = dev_alloc<double>(A, B, S.n_x);
  d.rr_s = dev_alloc<double>(A, B, S.m_d);
  d.rr_y = dev_alloc<double>(A, B, S.m_c);
  d.rr_yd = dev_alloc<double>(A, B, S.m_d);
  d.dx = dev_alloc<double>(A, B, S.n_x);
  d.ds = dev_alloc<double>(A, B, S.m_d);
  d.dy = dev_alloc<double>(A, B, S.m_c);
  d.dyd = dev_alloc<double>(A, B, S.m_d);
  d.red = dev_alloc<double>(A, B, kRedBlocks * 8);
  d.sc = dev_alloc<DevScalars>(A, B, 1);
  dp = d;

  HYKKT_CUDA(cudaFuncSetAttribute(k_piece_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, kInvSmem));
  raise_front_small_smem(max_small_smem_);

  // pinned staging for host inputs / outputs (kept while device storage is released)
  if (g_count_only || pin_in_) return;
  pin_in_n_ = (int64_t)S.nnz_h + std::max(S.nnz_ds, S.m_d) + S.nnz_jc + S.nnz_jd + S.n_x + 3LL * S.m_d + 2LL * S.m_c + 16;
  HYKKT_CUDA(cudaMallocHost(&pin_in_, pin_in_n_ * sizeof(double)));
  pin_out_n_ = (int64_t)S.n_x + 2LL * S.m_d + S.m_c + 16;
  HYKKT_CUDA(cudaMallocHost(&pin_out_, pin_out_n_ * sizeof(double)));
  HYKKT_CUDA(cudaMallocHost(&pin_sc_, sizeof(DevScalars)));
}

// A kernel's dynamic shared-memory limit is one value per device for the
// whole process, shared by every plan: it only ever grows, so that a plan
// created later with smaller fronts cannot lower the limit that an earlier
// plan's launches need.
void raise_front_small_smem(int bytes) {
  static std::mutex mu;
  static std::map<int, int> limit;  // device -> current limit
  if (bytes <= 48 * 1024) return;
  int dev = 0;
  HYKKT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  int& cur = limit[dev];
  if (bytes <= cur) return;
  HYKKT_CUDA(cudaFuncSetAttribute(k_front_small, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  cur = bytes;
}

// ---------------------------------------------------------------------------
// Recording of the solve sequence (into a graph capture or directly)
// ---------------------------------------------------------------------------
#define LAUNCH(kern, grid, block, smem, st, ...)                  \
  do {                                                            \
    if (prof_) prof_begin(st);                                    \
    kern<<<(grid), (block), (smem), (st)>>>(__VA_ARGS__);         \
    if (prof_) prof_end(st, #kern);                               \
    ++kernels_per_solve_;                                         \
  } while (0)

// Per-kernel timing in uncaptured runs: an event pair around every launch.
void Engine::prof_begin(cudaStream_t st) {
  cudaEvent_t a;
  HYKKT_CUDA(cudaEventCreate(&a));
  HYKKT_CUDA(cudaEventRecord(a, st));
  prof_open_ = a;
}
void Engine::prof_end(cudaStream_t st, const char* name) {
  cudaEvent_t b;
  HYKKT_CUDA(cudaEventCreate(&b));
  HYKKT_CUDA(cudaEventRecord(b, st));
  prof_events_.push_back({name, prof_open_, b});
}
void Engine::prof_work(const char* name, double flops, double bytes) {
  auto& w = prof_work_[name];
  w.first += flops;
  w.second += bytes;
}
int Engine::profile(cudaStream_t st, int upto, std::vector<KernelTime>& out) {
  reload_device();
  prof_ = true;
  prof_events_.clear();
  prof_work_.clear();
  try {
    run_direct(st, upto, nullptr);
  } catch (...) {
    prof_ = false;
    throw;
  }
  prof_ = false;
  HYKKT_CUDA(cudaStreamSynchronize(st));
  out.clear();
  for (auto& e : prof_events_) {
    float ms = 0;
    HYKKT_CUDA(cudaEventElapsedTime(&ms, e.a, e.b));
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
    auto it = std::find_if(out.begin(), out.end(), [&](const KernelTime& k) { return k.name == e.name; });
    if (it == out.end()) out.push_back({e.name, 1, ms, 0.0, 0.0});
    else { it->launches += 1; it->ms += ms; }
  }
  for (auto& k : out) {
    auto w = prof_work_.find(k.name);
    if (w != prof_work_.end()) { k.flops = w->second.first; k.bytes = w->second.second; }
  }
  prof_events_.clear();
  return 0;
}

void Engine::record_numeric(cudaStream_t st) {
  const DevPlan& d = dp;
  const int nrows = d.n_x + d.m_c;
  const int grid_big = std::max(1, std::min(cdiv(std::max({d.nnz_ht, d.n_x, d.nnz_jc, d.nnz_lo}), kBlock), 148 * 16));
  LAUNCH(k_prepare, grid_big, kBlock, 0, st, d, RhsPtrs{d.rx, d.rs, d.ry, d.ryd}, 1, 0);
  const int warps_grid = std::max(1, cdiv((int64_t)nrows * 32, kBlock));
  for (int sweep = 0; sweep < 2; ++sweep) {  // ruiz_its_ = 2 (HykktSolver.hpp:367)
    LAUNCH(k_ruiz_rowmax, warps_grid, kBlock, 0, st, d);
    LAUNCH(k_ruiz_scale, warps_grid, kBlock, 0, st, d);
  }
  LAUNCH(k_hgamma, grid_big, kBlock, 0, st, d, 1);
  if (d.delta != 0.0) LAUNCH(k_add_diag, std::max(1, cdiv(d.n_x, kBlock)), kBlock, 0, st, d);
  if (prof_) {
    // algorithmic work: every input value and list entry read once, every
    // output written once (the Ruiz model counts indices 4 B, values 8 B)
    const Symbolic& S = S_;
    const double nht = S.Ht.nnz(), nlo = S.lp_cp[S.n_x], njc = S.nnz_jc, njd = S.nnz_jd, nh = S.nnz_h;
    const double cht = (double)S.ht_ca.size(), chg = (double)S.lp_ca.size();
    const double nx = S.n_x, mc = S.m_c, md = S.m_d;
    prof_work("k_prepare", 3.0 * cht + nht,
              8.0 * (nh + njd + md) + 4.0 * (2.0 * nht + 3.0 * cht) + 8.0 * nht + 8.0 * (2.0 * nx + 3.0 * md + mc));
    const double vals = nht + 2.0 * njc, rows = nx + mc;
    prof_work("k_ruiz_rowmax", 2.0 * vals, 2.0 * (12.0 * vals + 8.0 * (rows + 2)));
    prof_work("k_ruiz_scale", 2.0 * 2.0 * vals, 2.0 * (20.0 * vals + 32.0 * rows));
    prof_work("k_hgamma", 2.0 * chg + nlo,
              8.0 * (nht + njc) + 4.0 * (2.0 * nlo + 2.0 * chg) + 8.0 * nlo + 8.0 * (nx + mc));
  }
}

void Engine::record_factor(cudaStream_t st) {
  const Symbolic& S = S_;
  const DevPlan& d = dp;
  int step = 0;
  for (int l = 0; l < S.nlevels; ++l) {
    const FactorLevel& L = S.flevels[l];
    if (!L.small.empty()) {
      int smem = 0;
      for (int J : L.small) smem = std::max(smem, S.sn_nrows[J] * S.sn_nrows[J] * 8);
      LAUNCH(k_front_small, (int)L.small.size(), kBlock, smem, st, d, d_small_[l]);
      if (prof_) {
        double f = 0, b = 0;
        for (int J : L.small) {
          const double nJ = S.sn_nrows[J], nc = S.sn_first[J + 1] - S.sn_first[J];
          for (int k = 0; k < nc; ++k) { const double m = nJ - k - 1; f += m * (m + 1) + m; }
          b += 8.0 * nJ * nJ;
        }
        prof_work("k_front_small", f, b);
      }
    }
    if (L.large.empty()) continue;
    const int64_t lo = S.sn_off[L.large.front()];
    const int J1 = L.large.back();
    const int64_t hi = S.sn_off[J1] + (int64_t)S.sn_nrows[J1] * S.sn_nrows[J1];
    HYKKT_CUDA(cudaMemsetAsync(d.front + lo, 0, (hi - lo) * sizeof(double), st));
    LAUNCH(k_front_scatter, dim3((unsigned)L.large.size(), 8), kBlock, 0, st, d, d_large_[l]);
    LAUNCH(k_front_extadd, n_ea_[l], kBlock, 0, st, d, d_ea_sn_[l], d_ea_row0_[l]);
    for (int p = 0; p < L.max_panels; ++p, ++step) {
      const int np = pw_.potrf_off[step + 1] - pw_.potrf_off[step];
      const int nt = pw_.trsm_off[step + 1] - pw_.trsm_off[step];
      const int nu = pw_.upd_off[step + 1] - pw_.upd_off[step];
      if (np) LAUNCH(k_panel_potrf, np, kBlock, 0, st, d, d_potrf_sn_ + pw_.potrf_off[step], p);
      if (nt) LAUNCH(k_panel_trsm, nt, kTrsmRows, 0, st, d, d_trsm_sn_ + pw_.trsm_off[step], d_trsm_row0_ + pw_.trsm_off[step], p);
      if (nu)
        LAUNCH(k_panel_update, nu, kBlock, 0, st, d, d_upd_sn_ + pw_.upd_off[step], d_upd_ti_ + pw_.upd_off[step],
               d_upd_tj_ + pw_.upd_off[step], p);
      if (prof_) {
        // right-looking partial Cholesky: SYRK on the trailing lower triangle,
        // TRSM on the rows below the panel
        double fu = 0, bu = 0, ft = 0;
        for (int J : L.large) {
          const int ncols = S.sn_first[J + 1] - S.sn_first[J];
          const int c0 = p * kPanel;
          if (c0 >= ncols) continue;
          const double w = std::min(kPanel, ncols - c0);
          const double T = S.sn_nrows[J] - c0 - w;
          fu += 2.0 * w * T * (T + 1) / 2;
          bu += 8.0 * (T * (T + 1) + 2 * T * w);  // read+write C (lower), read the panel
          ft += T * w * (w + 1);
        }
        prof_work("k_panel_update", fu, bu);
        prof_work("k_panel_trsm", ft, 0);
      }
    }
  }
  // inverses of the triangular-solve items' diagonal blocks
  if (!iw_.small.empty()) LAUNCH(k_piece_inverse, (int)iw_.small.size(), kBlock, kInvSmem, st, d, d_inv_small_);
  if (!iw_.big.empty()) {
    LAUNCH(k_trtri_init, dim3(64, (unsigned)iw_.big.size()), kBlock, 0, st, d, d_inv_big_);
    const int steps = (int)iw_.diag_off.size() - 1;
    for (int i = 0; i < steps; ++i) {
      const int nd = iw_.diag_off[i + 1] - iw_.diag_off[i];
      const int nu = iw_.upd_off[i + 1] - iw_.upd_off[i];
      if (nd) LAUNCH(k_trtri_diag, nd, kDiagCols, 0, st, d, d_idiag_q_ + iw_.diag_off[i], d_idiag_c_ + iw_.diag_off[i], i);
      if (nu)
        LAUNCH(k_trtri_update, nu, kBlock, 0, st, d, d_iupd_q_ + iw_.upd_off[i], d_iupd_r_ + iw_.upd_off[i],
               d_iupd_c_ + iw_.upd_off[i], i);
    }
    if (prof_) {
      double f = 0;
      for (int q : iw_.big) {
        const double nc = S.sq_c1[q] - S.sq_c0[q];
        f += nc * nc * nc / 3.0;
      }
      prof_work("k_trtri_update", f, 0);
    }
  }
  if (n_pack_) LAUNCH(k_xpanel_pack, n_pack_, kBlock, 0, st, d, d_pack_q_, d_pack_b_, sched_.rows_x);
  for (int q : l21_items_) {  // packed rows-below blocks of the panelized items
    const Symbolic& S = S_;
    const int64_t n = (int64_t)(S.sn_nrows[S.sq_sn[q]] - S.sq_c1[q]) * (S.sq_c1[q] - S.sq_c0[q]);
    LAUNCH(k_l21_pack, (int)std::min<int64_t>(cdiv(n, kBlock), 148 * 16), kBlock, 0, st, d, q, S.sq_l21f[q], S.sq_l21b[q]);
  }
}

// One forward + backward solve pair: x = L^-T L^-1 b.  The dependency
// counters of each direction are cleared by the other direction's kernel;
// `reset` clears both first (a pair that does not follow a pair of the same
// loop body).
void Engine::record_trisolve(cudaStream_t st, const double* b, double* x, int use_stop, bool reset) {
  const Symbolic& S = S_;
  const DevPlan& d = dp;
  if (reset) HYKKT_CUDA(cudaMemsetAsync(sched_.cnt, 0, cnt_ints_ * sizeof(int), st));
  LAUNCH(k_trsv_fwd, grid_f_, kBlock, 0, st, d, sched_, b, x, use_stop);
  LAUNCH(k_trsv_bwd, grid_b_, kBlock, 0, st, d, sched_, x, use_stop);
  if (prof_) {
    // algorithmic work of one direction: every stored entry of L read once,
    // one multiply-add per entry (diagonal blocks: lower triangle)
    double f = 0, b8 = 0;
    for (int q = 0; q < S.nsq; ++q) {
      const double nc = S.sq_c1[q] - S.sq_c0[q], R = S.sn_nrows[S.sq_sn[q]] - S.sq_c1[q];
      f += nc * nc + 2.0 * R * nc;
      b8 += 8.0 * (nc * (nc + 1) / 2 + R * nc);
    }
    prof_work("k_trsv_fwd", f, b8);
    prof_work("k_trsv_bwd", f, b8);
  }
}

// CG right-hand side and start (setup_conjugate_gradient + the first part of
// SchurComplementConjugateGradient::solve, HykktSolver.cpp:814-843,
// SchurCG.cpp:89-144).  zero_x0 for refinement corrections.
void Engine::record_cg_pre(cudaStream_t st, int zero_x0) {
  const DevPlan& d = dp;
  const int gm = std::max(1, std::min(cdiv(d.m_c, kBlock), kRedBlocks));
  const int gn = std::max(1, cdiv(d.n_x, kBlock));
  record_trisolve(st, d.rxp, d.hrxp, 0);
  LAUNCH(k_spmv_jcp, gm, kBlock, 0, st, d, d.hrxp, d.schur, d.ry_s, 0, 0);
  LAUNCH(k_cg_setup, gm, kBlock, 0, st, d, zero_x0);
  // r = b - S x0, gam = r.r
  LAUNCH(k_spmv_jctp, gn, kBlock, 0, st, d, d.cg_x, d.cg_yv, (const double*)nullptr, 0);
  record_trisolve(st, d.cg_yv, d.cg_z, 0);
  LAUNCH(k_spmv_jcp, gm, kBlock, 0, st, d, d.cg_z, d.cg_r, (const double*)nullptr, 4, 0);
  // w = S r, delta = w.r, alpha = gam/delta
  LAUNCH(k_spmv_jctp, gn, kBlock, 0, st, d, d.cg_r, d.cg_yv, (const double*)nullptr, 0);
  record_trisolve(st, d.cg_yv, d.cg_z, 0);
  LAUNCH(k_spmv_jcp, gm, kBlock, 0, st, d, d.cg_z, d.cg_w, (const double*)nullptr, 2, 0);
}

void Engine::record_cg_body(cudaStream_t st, cudaGraphConditionalHandle h, bool with_cond) {
  const DevPlan& d = dp;
  const int gm = std::max(1, std::min(cdiv(d.m_c, kBlock), kRedBlocks));
  // five launches per iteration: the update also decides the loop
  // condition, and the solve pair follows the previous iteration's pair (no
  // counter reset).  (Forming Jc_p^T r inside the forward solve instead of
  // k_spmv_jctp measured slower: it lengthens the leaves' tasks.)
  LAUNCH(k_cg_update, gm, kBlock, 0, st, d, h, with_cond ? 1 : 0);
  LAUNCH(k_spmv_jctp, std::max(1, cdiv(d.n_x, kBlock)), kBlock, 0, st, d, d.cg_r, d.cg_yv, (const double*)nullptr, 1);
  record_trisolve(st, d.cg_yv, d.cg_z, 1, !with_cond);
  LAUNCH(k_spmv_jcp, gm, kBlock, 0, st, d, d.cg_z, d.cg_w, (const double*)nullptr, 3, 1);
}

// Recovery (recover_solution, HykktSolver.cpp:410-457) and the residual.
// correction = 1: recover the refinement correction from the residual
// right-hand side and add it to the solution.
void Engine::record_post(cudaStream_t st, int correction) {
  const DevPlan& d = dp;
  const int gn = std::max(1, cdiv(d.n_x, kBlock));
  const int gb = std::max(1, std::min(cdiv(std::max(d.n_x, std::max(d.m_c, d.m_d)), kBlock), 148 * 8));
  LAUNCH(k_spmv_jctp, gn, kBlock, 0, st, d, d.cg_x, d.rxp, (const double*)d.rxp, 0);
  record_trisolve(st, d.rxp, d.tmp_n, 0);
  if (!correction) {
    LAUNCH(k_recover_x, gb, kBlock, 0, st, d, (const double*)d.tmp_n, d.x, d.y);
    LAUNCH(k_recover_s, std::max(1, cdiv(d.m_d, kBlock)), kBlock, 0, st, d, (const double*)d.x, (const double*)d.ryd,
           (const double*)d.rs, d.s, d.yd);
  } else {
    LAUNCH(k_recover_x, gb, kBlock, 0, st, d, (const double*)d.tmp_n, d.dx, d.dy);
    LAUNCH(k_recover_s, std::max(1, cdiv(d.m_d, kBlock)), kBlock, 0, st, d, (const double*)d.dx,
           (const double*)d.rr_yd, (const double*)d.rr_s, d.ds, d.dyd);
    LAUNCH(k_apply_delta, gb, kBlock, 0, st, d);
  }
  LAUNCH(k_residual, kRedBlocks, kBlock, 0, st, d);
}

// Right-hand-side part of one refinement correction: r~x, Ruiz scaling by
// the aggregated factors, r^x in permuted order.
void Engine::record_correction_rhs(cudaStream_t st) {
  const DevPlan& d = dp;
  const int grid_big = std::max(1, std::min(cdiv(std::max(d.n_x, d.m_c), kBlock), 148 * 16));
  LAUNCH(k_refine_begin, 1, 32, 0, st, d);
  LAUNCH(k_prepare, grid_big, kBlock, 0, st, d, RhsPtrs{d.rr_x, d.rr_s, d.rr_y, d.rr_yd}, 0, 1);
  LAUNCH(k_hgamma, grid_big, kBlock, 0, st, d, 0);
}

// Adds a conditional while node at the capture point of `st`; its body is
// recorded by `body` on stream `bs`.  `pre` records the kernel that sets the
// condition before the node (the default value only applies at graph
// launch, which is too early for a loop nested in another loop's body).
void Engine::capture_while(cudaStream_t st, cudaStream_t bs, int default_value,
                           const std::function<void(cudaStream_t, cudaGraphConditionalHandle)>& pre,
                           const std::function<void(cudaStream_t, cudaGraphConditionalHandle)>& body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  HYKKT_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphConditionalHandle h;
  HYKKT_CUDA(cudaGraphConditionalHandleCreate(&h, g, default_value, cudaGraphCondAssignDefault));
  if (pre) {
    pre(st, h);
    HYKKT_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
  }
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  HYKKT_CUDA(cudaGraphAddNode(&cnode, g, deps, nullptr, nd, &cp));
  cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
  HYKKT_CUDA(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  HYKKT_CUDA(cudaStreamBeginCaptureToGraph(bs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  body(bs, h);
  HYKKT_CUDA(cudaStreamEndCapture(bs, &bodyg));
}

int Engine::ensure_graph() {
  if (exec_dev_) return 0;
  std::lock_guard<std::mutex> lk(cuda_setup_mutex());
  try {
    capture_graph();
  } catch (...) {
    // leave no stream in capture mode and no partial graph behind
    for (cudaStream_t s : {body_stream2_, body_stream_, cap_stream_}) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (s && cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s, &g);
        if (g && s == cap_stream_) cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
    if (exec_dev_) { cudaGraphExecDestroy(exec_dev_); exec_dev_ = nullptr; }
    if (graph_dev_) { cudaGraphDestroy(graph_dev_); graph_dev_ = nullptr; }
    throw;
  }
  return 0;
}

void Engine::capture_graph() {
  if (!cap_stream_) {
    HYKKT_CUDA(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking));
    HYKKT_CUDA(cudaStreamCreateWithFlags(&body_stream_, cudaStreamNonBlocking));
    HYKKT_CUDA(cudaStreamCreateWithFlags(&body_stream2_, cudaStreamNonBlocking));
  }
  cudaStream_t st = cap_stream_;
  kernels_per_solve_ = 0;
  HYKKT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  record_numeric(st);
  record_factor(st);
  record_cg_pre(st, 0);
  int before = kernels_per_solve_;
  auto cg_body = [this](cudaStream_t s, cudaGraphConditionalHandle h) { record_cg_body(s, h, true); };
  auto cg_arm = [this](cudaStream_t s, cudaGraphConditionalHandle h) { LAUNCH(k_cond_arm, 1, 1, 0, s, h); };
  capture_while(st, body_stream_, 0, cg_arm, cg_body);
  kernels_per_iter_ = kernels_per_solve_ - before - 1;  // the arming kernel runs once
  kernels_per_solve_ = before + 1;
  record_post(st, 0);
  if (dp.refine_max > 0) {
    // iterative refinement on the full KKT system, reusing the factorization
    LAUNCH(k_refine_reset, 1, 32, 0, st, dp);
    before = kernels_per_solve_;
    auto pre = [this](cudaStream_t s, cudaGraphConditionalHandle h) { LAUNCH(k_refine_cond, 1, 1, 0, s, dp, h); };
    auto body = [this, cg_body, cg_arm](cudaStream_t s, cudaGraphConditionalHandle h) {
      record_correction_rhs(s);
      record_cg_pre(s, 1);
      capture_while(s, body_stream2_, 0, cg_arm, cg_body);
      record_post(s, 1);
      LAUNCH(k_refine_cond, 1, 1, 0, s, dp, h);
    };
    capture_while(st, body_stream_, 0, pre, body);
    kernels_per_refine_ = kernels_per_solve_ - before - kernels_per_iter_;
    kernels_per_solve_ = before;
  }
  HYKKT_CUDA(cudaStreamEndCapture(st, &graph_dev_));
  HYKKT_CUDA(cudaGraphInstantiate(&exec_dev_, graph_dev_, 0));
}

// Host-driven CG loop of the uncaptured path.
void Engine::direct_cg_loop(cudaStream_t st) {
  bool done = false;
  for (int it = 0; it < dp.cg_itmax; ++it) {
    record_cg_body(st, 0, false);
    HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, dp.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    HYKKT_CUDA(cudaStreamSynchronize(st));
    if (pin_sc_->stop) { done = true; break; }
  }
  if (!done) LAUNCH(k_cg_mark, 1, 1, 0, st, dp);
}

// Direct (uncaptured) execution with events between stages; the loops are
// driven from the host.  Used for stage timing, profiling and partial runs
// in the parity tests.  Stages: numeric, factor, CG setup, CG loop,
// recovery + residual + refinement.
int Engine::run_direct(cudaStream_t st, int upto, float* stage_ms) {
  reload_device();
  cudaEvent_t ev[8];
  for (int i = 0; i < 8; ++i) HYKKT_CUDA(cudaEventCreate(&ev[i]));
  HYKKT_CUDA(cudaEventRecord(ev[0], st));
  record_numeric(st);
  HYKKT_CUDA(cudaEventRecord(ev[1], st));
  if (upto >= 2) record_factor(st);
  HYKKT_CUDA(cudaEventRecord(ev[2], st));
  if (upto >= 3) {
    record_cg_pre(st, 0);
    HYKKT_CUDA(cudaEventRecord(ev[3], st));
    direct_cg_loop(st);
    HYKKT_CUDA(cudaEventRecord(ev[4], st));
    record_post(st, 0);
    if (dp.refine_max > 0) {
      LAUNCH(k_refine_reset, 1, 32, 0, st, dp);
      for (int r = 0; r < dp.refine_max; ++r) {
        LAUNCH(k_refine_decide, 1, 1, 0, st, dp);
        HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, dp.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
        HYKKT_CUDA(cudaStreamSynchronize(st));
        if (pin_sc_->solve_flags & 2) break;
        record_correction_rhs(st);
        record_cg_pre(st, 1);
        direct_cg_loop(st);
        record_post(st, 1);
      }
    }
  } else {
    HYKKT_CUDA(cudaEventRecord(ev[3], st));
    HYKKT_CUDA(cudaEventRecord(ev[4], st));
  }
  HYKKT_CUDA(cudaEventRecord(ev[5], st));
  HYKKT_CUDA(cudaStreamSynchronize(st));
  if (stage_ms)
    for (int i = 0; i < 5; ++i) HYKKT_CUDA(cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]));
  for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
  return 0;
}

// Persistent solve grids: every resident CTA slot of the GPU, or a 1/share
// part of them (at least 16 CTAs) when `share` plans solve at once, so that
// the plans' solve kernels can be resident together.
void Engine::size_solve_grids() {
  const int f = std::max(16, sms_ * occ_f_ / share_), b = std::max(16, sms_ * occ_b_ / share_);
  grid_f_ = std::max(1, std::min(sched_.ntasks_f, f));
  grid_b_ = std::max(1, std::min(sched_.ntasks_b, b));
}

void Engine::set_concurrency(int share) {
  if (share < 1) throw std::invalid_argument("concurrency must be >= 1");
  share_ = share;
  size_solve_grids();
  drop_graph();
}

void Engine::debug_set(const std::string& what, double value) {
  if (what == "spin_limit") {
    if (!(value >= 0.0) || value > 4294967295.0) throw std::invalid_argument("spin_limit out of range");
    dp.spin_limit = value == 0.0 ? kSpinLimit : (unsigned)value;
  } else if (what == "unsatisfiable_waits") {
    dp.dbg_unsatisfiable = value != 0.0 ? 1 : 0;
  } else {
    throw std::invalid_argument("unknown debug setting: " + what);
  }
  drop_graph();  // the graph's kernels hold the plan by value
}

void Engine::set_delta(double delta) {
  if (!(delta >= 0.0) || !(delta < 1e300)) throw std::invalid_argument("delta must be finite and >= 0");
  dp.delta = delta;
  drop_graph();  // the graph holds the launch (or not) and the value
}

void Engine::set_refine_rtol(double rtol) {
  dp.cg_rtol_refine = rtol;
  drop_graph();
}

void Engine::set_accuracy(int cg_itmax, double cg_rtol, int refine_max, double refine_target) {
  dp.cg_itmax = cg_itmax;
  dp.cg_rtol = cg_rtol;
  dp.cg_rtol_refine = cg_rtol;
  dp.refine_max = refine_max;
  dp.refine_target = refine_target;
  drop_graph();
}

int Engine::upload(const double* h_v, const double* ds_v, const double* jc_v, const double* jd_v, const double* rx,
                   const double* rs, const double* ry, const double* ryd, const double* y0, bool on_device,
                   cudaStream_t st) {
  const Symbolic& S = S_;
  struct Item { double* dst; const double* src; int64_t n; };
  const int64_t nds = S.nnz_ds;
  Item items[9] = {{dp.h_v, h_v, S.nnz_h}, {dp.ds_v, ds_v, nds}, {dp.jc_v, jc_v, S.nnz_jc}, {dp.jd_v, jd_v, S.nnz_jd},
                   {dp.rx, rx, S.n_x}, {dp.rs, rs, S.m_d}, {dp.ry, ry, S.m_c}, {dp.ryd, ryd, S.m_d},
                   {dp.y0, y0, S.m_c}};
  if (on_device) {
    for (auto& it : items) {
      if (it.n == 0) continue;
      if (it.src) HYKKT_CUDA(cudaMemcpyAsync(it.dst, it.src, it.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      else HYKKT_CUDA(cudaMemsetAsync(it.dst, 0, it.n * sizeof(double), st));
    }
    return 0;
  }
  // host inputs: pageable user memory -> pinned staging -> one DMA per block
  int64_t off = 0;
  for (auto& it : items) {
    if (it.n == 0) continue;
    if (it.src) std::memcpy(pin_in_ + off, it.src, it.n * sizeof(double));
    else std::memset(pin_in_ + off, 0, it.n * sizeof(double));
    HYKKT_CUDA(cudaMemcpyAsync(it.dst, pin_in_ + off, it.n * sizeof(double), cudaMemcpyHostToDevice, st));
    off += it.n;
  }
  return 0;
}

int Engine::solve(const double* h_v, const double* ds_v, const double* jc_v, const double* jd_v, const double* rx,
                  const double* rs, const double* ry, const double* ryd, const double* y0, bool on_device,
                  cudaStream_t st, bool sync) {
  reload_device();  // a released plan takes its device storage back first
  upload(h_v, ds_v, jc_v, jd_v, rx, rs, ry, ryd, y0, on_device, st);
  ensure_graph();
  HYKKT_CUDA(cudaGraphLaunch(exec_dev_, st));
  if (!last_launch_) HYKKT_CUDA(cudaEventCreateWithFlags(&last_launch_, cudaEventDisableTiming));
  HYKKT_CUDA(cudaEventRecord(last_launch_, st));
  if (!sync) return 0;
  return finish(st);
}

int Engine::finish(cudaStream_t st) {
  if (!resident_) throw std::invalid_argument("the plan's device storage is released (its last solution with it)");
  HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, dp.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
  HYKKT_CUDA(cudaStreamSynchronize(st));
  last_sc_ = *pin_sc_;
  const bool refined_ok = dp.refine_max > 0 && last_sc_.rel_res_full <= dp.refine_target;
  if (last_sc_.solve_flags & 1) last_status_ = ST_TIMEOUT;
  else if (last_sc_.pivot_col != INT_MAX) last_status_ = ST_NOT_SPD;
  else if (last_sc_.stop_main > 0 && !refined_ok) last_status_ = ST_CG_NOT_CONVERGED;
  // with refinement on, the caller asked for a residual target: a solve that
  // ends above it (or with a residual that is not a number) is not a success
  else if (dp.refine_max > 0 && !refined_ok) last_status_ = ST_ACCURACY_NOT_MET;
  else last_status_ = ST_OK;
  return last_status_;
}

int Engine::get_solution(double* x, double* s, double* y, double* yd, bool to_device, cudaStream_t st) {
  if (!resident_) throw std::invalid_argument("the plan's device storage is released (its last solution with it)");
  const Symbolic& S = S_;
  struct Item { double* dst; const double* src; int64_t n; };
  Item items[4] = {{x, dp.x, S.n_x}, {s, dp.s, S.m_d}, {y, dp.y, S.m_c}, {yd, dp.yd, S.m_d}};
  if (to_device) {
    for (auto& it : items)
      if (it.dst && it.n) HYKKT_CUDA(cudaMemcpyAsync(it.dst, it.src, it.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    HYKKT_CUDA(cudaStreamSynchronize(st));
    return 0;
  }
  int64_t off = 0;
  for (auto& it : items) {
    if (it.dst && it.n) HYKKT_CUDA(cudaMemcpyAsync(pin_out_ + off, it.src, it.n * sizeof(double), cudaMemcpyDeviceToHost, st));
    off += it.n;
  }
  HYKKT_CUDA(cudaStreamSynchronize(st));
  off = 0;
  for (auto& it : items) {
    if (it.dst && it.n) std::memcpy(it.dst, pin_out_ + off, it.n * sizeof(double));
    off += it.n;
  }
  return 0;
}

int Engine::debug_read(const char* what, double* out, int64_t n) {
  if (!resident_) throw std::invalid_argument("the plan's device storage is released (its last solution with it)");
  struct Arr { const char* name; const double* p; int64_t n; };
  const Symbolic& S = S_;
  Arr arrs[] = {{"ht_v", dp.ht_v, S.Ht.nnz()}, {"jc_s", dp.jc_s, S.nnz_jc}, {"ry_s", dp.ry_s, S.m_c},
                {"rxt", dp.rxt, S.n_x}, {"max_d", dp.max_d, S.n_x + S.m_c}, {"scale", dp.scale, S.n_x + S.m_c},
                {"lp_v", dp.lp_v, S.lp_cp[S.n_x]}, {"rxp", dp.rxp, S.n_x}, {"hrxp", dp.hrxp, S.n_x},
                {"schur", dp.schur, S.m_c}, {"cg_x", dp.cg_x, S.m_c}, {"front", dp.front, S.front_arena},
                {"x", dp.x, S.n_x}, {"s", dp.s, S.m_d}, {"y", dp.y, S.m_c}, {"yd", dp.yd, S.m_d},
                {"tmp_n", dp.tmp_n, S.n_x}, {"rr_x", dp.rr_x, S.n_x}, {"rr_s", dp.rr_s, S.m_d},
                {"rr_y", dp.rr_y, S.m_c}, {"rr_yd", dp.rr_yd, S.m_d}, {"dx", dp.dx, S.n_x}, {"ds", dp.ds, S.m_d},
                {"dy", dp.dy, S.m_c}, {"dyd", dp.dyd, S.m_d}};
  for (auto& a : arrs)
    if (std::strcmp(a.name, what) == 0) {
      if (n > a.n) return ST_INVALID;
      HYKKT_CUDA(cudaDeviceSynchronize());
      HYKKT_CUDA(cudaMemcpy(out, a.p, n * sizeof(double), cudaMemcpyDeviceToHost));
      return 0;
    }
  return ST_INVALID;
}

// Average time (ms) of one forward+backward solve pair with the current factor.
float Engine::time_trisolve(cudaStream_t st, int nrep) {
  reload_device();
  cudaEvent_t a, b;
  HYKKT_CUDA(cudaEventCreate(&a));
  HYKKT_CUDA(cudaEventCreate(&b));
  record_trisolve(st, dp.rxp, dp.tmp_n, 0);  // warm-up
  HYKKT_CUDA(cudaEventRecord(a, st));
  for (int i = 0; i < nrep; ++i) record_trisolve(st, dp.rxp, dp.tmp_n, 0);
  HYKKT_CUDA(cudaEventRecord(b, st));
  HYKKT_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  HYKKT_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / std::max(nrep, 1);
}

float Engine::time_trisolve_group(const std::vector<Engine*>& es, int nrep, int mode, cudaStream_t st) {
#ifndef HYKKT_MEASURE
  (void)es, (void)nrep, (void)mode, (void)st;
  throw std::invalid_argument("group solve timing is in measurement builds only (HYKKT_MEASURE=1)");
#else
  const int n = (int)es.size();
  if (n == 0) return 0.0f;
  for (Engine* e : es)
    if (e->sched_.ntasks_f != es[0]->sched_.ntasks_f || e->sched_.ntasks_b != es[0]->sched_.ntasks_b)
      throw std::invalid_argument("plans of different patterns");
  std::vector<DevPlan> hd(n);
  std::vector<SolveSched> hs(n);
  std::vector<const double*> hb(n);
  std::vector<double*> hx(n);
  for (int i = 0; i < n; ++i) {
    hd[i] = es[i]->dp;
    hs[i] = es[i]->sched_;
    hb[i] = es[i]->dp.rxp;
    hx[i] = es[i]->dp.tmp_n;
  }
  DevPlan* dd = nullptr;
  SolveSched* ds = nullptr;
  const double** db = nullptr;
  double** dx = nullptr;
  int* head = nullptr;
  HYKKT_CUDA(cudaMalloc(&dd, n * sizeof(DevPlan)));
  HYKKT_CUDA(cudaMalloc(&ds, n * sizeof(SolveSched)));
  HYKKT_CUDA(cudaMalloc(&db, n * sizeof(double*)));
  HYKKT_CUDA(cudaMalloc(&dx, n * sizeof(double*)));
  HYKKT_CUDA(cudaMalloc(&head, 2 * sizeof(int)));
  HYKKT_CUDA(cudaMemcpy(dd, hd.data(), n * sizeof(DevPlan), cudaMemcpyHostToDevice));
  HYKKT_CUDA(cudaMemcpy(ds, hs.data(), n * sizeof(SolveSched), cudaMemcpyHostToDevice));
  HYKKT_CUDA(cudaMemcpy(db, hb.data(), n * sizeof(double*), cudaMemcpyHostToDevice));
  HYKKT_CUDA(cudaMemcpy(dx, hx.data(), n * sizeof(double*), cudaMemcpyHostToDevice));
  MultiTrsv m{dd, ds, db, dx, n, head, 0};
  const int gf = es[0]->sms_ * es[0]->occ_f_, gb = es[0]->sms_ * es[0]->occ_b_;
  std::vector<cudaStream_t> sts(n, nullptr);
  std::vector<cudaEvent_t> evs(n, nullptr);
  cudaEvent_t fork;
  HYKKT_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  if (mode == 1)
    for (int i = 0; i < n; ++i) {
      HYKKT_CUDA(cudaStreamCreateWithFlags(&sts[i], cudaStreamNonBlocking));
      HYKKT_CUDA(cudaEventCreateWithFlags(&evs[i], cudaEventDisableTiming));
    }
  auto one = [&]() {
    if (mode == 0) {
      for (Engine* e : es) HYKKT_CUDA(cudaMemsetAsync(e->sched_.cnt, 0, e->cnt_ints_ * sizeof(int), st));
      HYKKT_CUDA(cudaMemsetAsync(head, 0, 2 * sizeof(int), st));
      k_trsv_fwd_multi<<<gf, kBlock, 0, st>>>(m);
      k_trsv_bwd_multi<<<gb, kBlock, 0, st>>>(m);
    } else if (mode == 1) {
      HYKKT_CUDA(cudaEventRecord(fork, st));
      for (int i = 0; i < n; ++i) {
        HYKKT_CUDA(cudaStreamWaitEvent(sts[i], fork, 0));
        es[i]->record_trisolve(sts[i], es[i]->dp.rxp, es[i]->dp.tmp_n, 0);
        HYKKT_CUDA(cudaEventRecord(evs[i], sts[i]));
        HYKKT_CUDA(cudaStreamWaitEvent(st, evs[i], 0));
      }
    } else {
      for (Engine* e : es) e->record_trisolve(st, e->dp.rxp, e->dp.tmp_n, 0);
    }
    HYKKT_CUDA(cudaGetLastError());
  };
  cudaEvent_t a, b;
  HYKKT_CUDA(cudaEventCreate(&a));
  HYKKT_CUDA(cudaEventCreate(&b));
  one();  // warm-up
  HYKKT_CUDA(cudaEventRecord(a, st));
  for (int r = 0; r < nrep; ++r) one();
  HYKKT_CUDA(cudaEventRecord(b, st));
  HYKKT_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  HYKKT_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaEventDestroy(fork);
  for (int i = 0; i < n; ++i) {
    if (sts[i]) cudaStreamDestroy(sts[i]);
    if (evs[i]) cudaEventDestroy(evs[i]);
  }
  cudaFree(dd);
  cudaFree(ds);
  cudaFree(db);
  cudaFree(dx);
  cudaFree(head);
  return ms / std::max(nrep, 1);
#endif
}

void Engine::trace_trisolve(cudaStream_t st, std::vector<unsigned long long>& out) {
#ifndef HYKKT_MEASURE
  (void)st, (void)out;
  throw std::invalid_argument("the solve timeline is in measurement builds only (HYKKT_MEASURE=1)");
#else
  const int64_t n = 4LL * (sched_.ntasks_f + sched_.ntasks_b);
  unsigned long long* buf = nullptr;
  HYKKT_CUDA(cudaMallocAsync(&buf, std::max<int64_t>(n, 1) * sizeof(unsigned long long), st));
  HYKKT_CUDA(cudaMemsetAsync(buf, 0, std::max<int64_t>(n, 1) * sizeof(unsigned long long), st));
  record_trisolve(st, dp.rxp, dp.tmp_n, 0);  // warm-up, untraced
  DevPlan saved = dp;
  dp.trace = buf;
  try {
    record_trisolve(st, dp.rxp, dp.tmp_n, 0);
  } catch (...) {
    dp = saved;
    throw;
  }
  dp = saved;
  out.assign(n, 0);
  HYKKT_CUDA(cudaMemcpyAsync(out.data(), buf, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  HYKKT_CUDA(cudaFreeAsync(buf, st));
  HYKKT_CUDA(cudaStreamSynchronize(st));
#endif
}

// Triangular solve of the current factor on a device vector (component API).
int Engine::trisolve(const double* b, double* x, cudaStream_t st) {
  reload_device();
  record_trisolve(st, b, x, 0);
  HYKKT_CUDA(cudaStreamSynchronize(st));
  return 0;
}

// ---------------------------------------------------------------------------
// Cholesky component: the plan of a single SPD matrix (no Jc/Jd blocks).
// ---------------------------------------------------------------------------
int Engine::factor_values(const double* lower_vals_host, cudaStream_t st) {
  reload_device();
  const int nlo = S_.lp_cp[S_.n_x];
  HYKKT_CUDA(cudaMemcpyAsync(dp.lp_v, lower_vals_host, (size_t)nlo * sizeof(double), cudaMemcpyHostToDevice, st));
  DevScalars init{};
  init.pivot_col = INT_MAX;
  HYKKT_CUDA(cudaMemcpyAsync(dp.sc, &init, sizeof(DevScalars), cudaMemcpyHostToDevice, st));
  record_factor(st);
  HYKKT_CUDA(cudaGetLastError());
  HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, dp.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
  HYKKT_CUDA(cudaStreamSynchronize(st));
  last_sc_ = *pin_sc_;
  last_status_ = last_sc_.pivot_col != INT_MAX ? ST_NOT_SPD : ST_OK;
  return last_status_;
}

// CG on S = Jc H^{-1} Jc^T with this engine's factor (same recurrence and
// stopping test as the product path; host-driven loop).
int Engine::schur_cg(int m, const std::vector<int>& jc_rp, const std::vector<int>& jc_ci, const double* jc_v_host,
                     const double* b_host, double* x_host, int itmax, double tol, int* iters, double* err,
                     cudaStream_t st) {
  reload_device();
  const int n = S_.n_x;
  const int nnz = jc_rp[m];
  // Jc with permuted columns, Jc^T with permuted rows
  std::vector<int> jcp(nnz), tp(n + 1, 0), tci(nnz), tsrc(nnz);
  for (int p = 0; p < nnz; ++p) jcp[p] = S_.rev_perm[jc_ci[p]];
  for (int p = 0; p < nnz; ++p) tp[jcp[p] + 1]++;
  for (int i = 0; i < n; ++i) tp[i + 1] += tp[i];
  {
    std::vector<int> next(tp.begin(), tp.end() - 1);
    for (int k = 0; k < m; ++k)
      for (int p = jc_rp[k]; p < jc_rp[k + 1]; ++p) {
        int q = next[jcp[p]]++;
        tci[q] = k;
        tsrc[q] = p;
      }
  }
  std::vector<void*> tmp;
  auto up_i = [&](const std::vector<int>& v) {
    int* p = nullptr;
    HYKKT_CUDA(cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(int)));
    tmp.push_back(p);
    // on the stream of the kernels that read it (a non-blocking stream does
    // not wait for the legacy default stream)
    if (!v.empty()) HYKKT_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    return p;
  };
  auto up_d = [&](const double* v, int64_t k) {
    double* p = nullptr;
    HYKKT_CUDA(cudaMalloc(&p, std::max<int64_t>(k, 1) * sizeof(double)));
    tmp.push_back(p);
    if (v) HYKKT_CUDA(cudaMemcpyAsync(p, v, k * sizeof(double), cudaMemcpyHostToDevice, st));
    else HYKKT_CUDA(cudaMemsetAsync(p, 0, std::max<int64_t>(k, 1) * sizeof(double), st));
    return p;
  };
  DevPlan d = dp;
  d.m_c = m;
  d.nnz_jc = nnz;
  d.jc_rp = up_i(jc_rp);
  d.jc_ci = up_i(jc_ci);
  d.jcp_ci = up_i(jcp);
  d.jctp_rp = up_i(tp);
  d.jctp_ci = up_i(tci);
  d.jctp_src = up_i(tsrc);
  d.jc_s = up_d(jc_v_host, nnz);
  d.schur = up_d(b_host, m);
  d.y0 = up_d(x_host, m);
  d.cg_x = up_d(nullptr, m);
  d.cg_r = up_d(nullptr, m);
  d.cg_w = up_d(nullptr, m);
  d.cg_p = up_d(nullptr, m);
  d.cg_s = up_d(nullptr, m);
  d.cg_tol = tol;
  d.cg_itmax = itmax;
  const int gm = std::max(1, std::min((m + kBlock - 1) / kBlock, kRedBlocks));
  const int gn = std::max(1, (n + kBlock - 1) / kBlock);
  k_cg_setup<<<gm, kBlock, 0, st>>>(d, 0);
  k_spmv_jctp<<<gn, kBlock, 0, st>>>(d, d.cg_x, d.cg_yv, nullptr, 0);
  record_trisolve(st, d.cg_yv, d.cg_z, 0);
  k_spmv_jcp<<<gm, kBlock, 0, st>>>(d, d.cg_z, d.cg_r, nullptr, 4, 0);
  k_spmv_jctp<<<gn, kBlock, 0, st>>>(d, d.cg_r, d.cg_yv, nullptr, 0);
  record_trisolve(st, d.cg_yv, d.cg_z, 0);
  k_spmv_jcp<<<gm, kBlock, 0, st>>>(d, d.cg_z, d.cg_w, nullptr, 2, 0);
  for (int it = 0; it < itmax; ++it) {
    k_cg_update<<<gm, kBlock, 0, st>>>(d, 0, 0);
    k_spmv_jctp<<<gn, kBlock, 0, st>>>(d, d.cg_r, d.cg_yv, nullptr, 1);
    record_trisolve(st, d.cg_yv, d.cg_z, 1);
    k_spmv_jcp<<<gm, kBlock, 0, st>>>(d, d.cg_z, d.cg_w, nullptr, 3, 1);
    HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, d.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    HYKKT_CUDA(cudaStreamSynchronize(st));
    if (pin_sc_->stop) break;
  }
  HYKKT_CUDA(cudaGetLastError());
  HYKKT_CUDA(cudaMemcpyAsync(x_host, d.cg_x, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, st));
  HYKKT_CUDA(cudaMemcpyAsync(pin_sc_, d.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
  HYKKT_CUDA(cudaStreamSynchronize(st));
  if (iters) *iters = pin_sc_->it;
  if (err) *err = pin_sc_->cg_err;
  const int st_out = pin_sc_->stop == 1 ? ST_OK : ST_CG_NOT_CONVERGED;
  for (void* p : tmp) cudaFree(p);
  return st_out;
}

}  // namespace hykkt
