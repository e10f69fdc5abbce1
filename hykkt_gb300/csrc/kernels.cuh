// Device kernels of the KKT solve path (sm_103a, FP64 throughout).
//
// Conventions shared with the oracle (oracle/hykkt_oracle.c) so that the
// integer work and the formation steps are bit-identical to it:
//   * products of products are evaluated left to right, e.g. (a*b)*c;
//   * sums of products accumulate from 0 in list order with separate
//     multiply and add (__dmul_rn/__dadd_rn: no contraction to FMA);
//   * Ruiz uses 1.0/sqrt(max) and v *= (s_i*s_j), as adapt_row_max /
//     adapt_diag_scale do (reference src/matrix_vector_ops.cu:146-266).
// The factorization, the triangular solves and the CG reductions use a
// different summation order than the oracle; they are compared within a
// relative tolerance.
#pragma once

#include <cuda_runtime.h>
#include <climits>
#include <cstdint>

#include "engine.hpp"

namespace hykkt {

constexpr int kBlock = 256;
constexpr int kPanel = 32;        // panel width of the blocked large-front factorization
constexpr int kTile = 64;         // trailing-update tile
constexpr int kTrsmRows = 64;     // rows per TRSM CTA (one thread per row: small CTAs spread a front's
                                  // dependent FMA chains over more SMs)
constexpr int kDiagCols = 64;     // columns per CTA of the inverse's diagonal-block step (same reason)
constexpr int kEaRows = 32;       // rows per extend-add CTA
constexpr int kPiece = 64;        // max columns of a small triangular-solve item
constexpr int kRedBlocks = 296;   // CTAs of the reduction kernels (2 x 148)

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// ---------------------------------------------------------------------------
// Deterministic reductions: every CTA writes its partial sums, the last CTA
// to finish (ticket) adds them in CTA order.
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_reduce_sum(double (&v)[NV], double* sh /* NV*32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = dadd(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) sh[k * 32 + warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = dadd(x, __shfl_down_sync(0xffffffffu, x, o));
      v[k] = x;  // valid in thread 0
    }
  }
  __syncthreads();
}

// Writes the CTA partials; returns true in thread 0 of the last CTA, with the
// totals in out[] (summed in CTA order).  The last CTA loads every partial at
// once into shared memory (one round trip to L2 instead of one per CTA) and
// sums each total there in CTA order, the same additions in the same order.
template <int NV>
__device__ bool grid_reduce_last(double (&v)[NV], double* partials, unsigned int* ticket, double (&out)[NV]) {
  __shared__ double sh[NV * 32];
  __shared__ double gath[kRedBlocks * NV];
  __shared__ bool last;
  block_reduce_sum<NV>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[blockIdx.x * NV + k] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  if (gridDim.x <= (unsigned)kRedBlocks) {
    __threadfence();
    const int n = (int)gridDim.x * NV;
    for (int i = threadIdx.x; i < n; i += blockDim.x) gath[i] = __ldcg(&partials[i]);
    __syncthreads();
    if (threadIdx.x < NV) {
      double acc = 0.0;
      for (unsigned int b = 0; b < gridDim.x; ++b) acc = dadd(acc, gath[b * NV + threadIdx.x]);
      sh[threadIdx.x] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) out[k] = sh[k];
      *ticket = 0u;  // reset for the next launch
      return true;
    }
    return false;
  }
  if (threadIdx.x == 0) {  // more CTAs than the gather buffer holds
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) {
#pragma unroll
      for (int k = 0; k < NV; ++k) out[k] = dadd(out[k], ((volatile double*)partials)[b * NV + k]);
    }
    *ticket = 0u;  // reset for the next launch
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Step a2: H~ = H + Jd^T Ds Jd and r~x = rx + Jd^T (Ds rd + rs)
// (reference HykktSolver.cpp:289-337, row_scale matrix_vector_ops.cu:490-509)
// ---------------------------------------------------------------------------
struct RhsPtrs {
  const double *rx, *rs, *ry, *ryd;
};

// matrix = 1: also form H~ and reset the per-solve state (first solve of a
// system).  scale = 1: right-hand side of a refinement correction, scaled
// by the aggregated Ruiz factors of the factorized system.
__global__ void k_prepare(DevPlan d, RhsPtrs r, int matrix, int scale) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (matrix) {
    for (int q = tid; q < d.nnz_ht; q += stride) {
      double h = d.ht_hsrc[q] >= 0 ? d.h_v[d.ht_hsrc[q]] : 0.0;
      double acc = 0.0;
      for (int t = d.ht_cp[q]; t < d.ht_cp[q + 1]; ++t)
        acc = dadd(acc, dmul(dmul(d.jd_v[d.ht_ca[t]], d.jd_v[d.ht_cb[t]]), d.ds_v[d.ht_ck[t]]));
      d.ht_v[q] = dadd(h, acc);
    }
    for (int p = tid; p < d.nnz_jc; p += stride) d.jc_s[p] = d.jc_v[p];
    for (int k = tid; k < d.n_x + d.m_c; k += stride) d.max_d[k] = 1.0;
    if (tid == 0) {
      d.sc->pivot_col = INT_MAX;
      d.sc->stop = 0;
      d.sc->it = 0;
      d.sc->it_total = 0;
      d.sc->refine_it = 0;
      d.sc->stop_main = 0;
      d.sc->solve_flags = 0;
    }
  }
  // r~x = rx + Jd^T (Ds rd + rs)
  for (int i = tid; i < d.n_x; i += stride) {
    double acc = 0.0;
    if (d.jd_flag) {
      for (int q = d.jdt_rp[i]; q < d.jdt_rp[i + 1]; ++q) {
        int k = d.jdt_ci[q];
        double ryds = dadd(dmul(r.ryd[k], d.ds_v[k]), r.rs[k]);
        acc = dadd(acc, dmul(d.jd_v[d.jdt_src[q]], ryds));
      }
    }
    double v = dadd(r.rx[i], acc);
    d.rxt[i] = scale ? dmul(v, d.max_d[i]) : v;
  }
  for (int k = tid; k < d.m_c; k += stride) d.ry_s[k] = scale ? dmul(r.ry[k], d.max_d[d.n_x + k]) : r.ry[k];
}

// ---------------------------------------------------------------------------
// Step a3: Ruiz equilibration of [H~ Jc^T; Jc 0] (RuizClass.cpp:54-88).
// One warp per row of the 2x2 block system.
// ---------------------------------------------------------------------------
__global__ void k_ruiz_rowmax(DevPlan d) {
  const int lane = threadIdx.x & 31;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nrow = d.n_x + d.m_c;
  if (row >= nrow) return;
  double ml = 0.0, mu = 0.0;
  if (row < d.n_x) {
    for (int p = d.ht_rp[row] + lane; p < d.ht_rp[row + 1]; p += 32) {
      double e = fabs(d.ht_v[p]);
      if (e > ml) ml = e;
    }
    for (int p = d.jct_rp[row] + lane; p < d.jct_rp[row + 1]; p += 32) {
      double e = fabs(d.jc_s[d.jct_src[p]]);
      if (e > mu) mu = e;
    }
  } else {
    const int k = row - d.n_x;
    for (int p = d.jc_rp[k] + lane; p < d.jc_rp[k + 1]; p += 32) {
      double e = fabs(d.jc_s[p]);
      if (e > ml) ml = e;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double a = __shfl_xor_sync(0xffffffffu, ml, o);
    double b = __shfl_xor_sync(0xffffffffu, mu, o);
    if (a > ml) ml = a;
    if (b > mu) mu = b;
  }
  if (lane == 0) {
    double m = (row < d.n_x) ? (ml > mu ? ml : mu) : ml;
    d.scale[row] = 1.0 / sqrt(m);
  }
}

__global__ void k_ruiz_scale(DevPlan d) {
  const int lane = threadIdx.x & 31;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nrow = d.n_x + d.m_c;
  if (row >= nrow) return;
  const double si = d.scale[row];
  if (row < d.n_x) {
    for (int p = d.ht_rp[row] + lane; p < d.ht_rp[row + 1]; p += 32)
      d.ht_v[p] = dmul(d.ht_v[p], dmul(si, d.scale[d.ht_ci[p]]));
    if (lane == 0) {
      d.rxt[row] = dmul(d.rxt[row], si);
      d.max_d[row] = dmul(d.max_d[row], si);
    }
  } else {
    const int k = row - d.n_x;
    for (int p = d.jc_rp[k] + lane; p < d.jc_rp[k + 1]; p += 32)
      d.jc_s[p] = dmul(d.jc_s[p], dmul(si, d.scale[d.jc_ci[p]]));
    if (lane == 0) {
      d.ry_s[k] = dmul(d.ry_s[k], si);
      d.max_d[row] = dmul(d.max_d[row], si);
    }
  }
}

// ---------------------------------------------------------------------------
// Steps a4+a5: Hgamma = H~ + gamma Jc^T Jc written straight into the permuted
// lower-triangular CSC layout, and r^x = r~x + gamma Jc^T ry gathered into
// permuted order (compute_spgemm_hgamma + apply_permutation,
// HykktSolver.cpp:370-395).
// ---------------------------------------------------------------------------
__global__ void k_hgamma(DevPlan d, int matrix) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (matrix)
  for (int q = tid; q < d.nnz_lo; q += stride) {
    double h = d.lp_htsrc[q] >= 0 ? d.ht_v[d.lp_htsrc[q]] : 0.0;
    double acc = 0.0;
    for (int t = d.lp_ccp[q]; t < d.lp_ccp[q + 1]; ++t) acc = dadd(acc, dmul(d.jc_s[d.lp_ca[t]], d.jc_s[d.lp_cb[t]]));
    d.lp_v[q] = dadd(h, dmul(d.gamma, acc));
  }
  for (int i = tid; i < d.n_x; i += stride) {
    double acc = 0.0;
    for (int p = d.jctp_rp[i]; p < d.jctp_rp[i + 1]; ++p) acc = dadd(acc, dmul(d.jc_s[d.jctp_src[p]], d.ry_s[d.jctp_ci[p]]));
    d.rxp[i] = dadd(d.rxt[d.perm[i]], dmul(d.gamma, acc));
  }
}

// add_diag (HykktSolver.cpp:392, matrix_vector_ops.cu:344-358): delta added
// to the diagonal entries of the permuted lower Hgamma that the pattern holds
// (none inserted).  The reference passes 0; delta != 0 gives the regularized
// H_delta = Hgamma + delta I of an interior-point method's inertia correction.
__global__ void k_add_diag(DevPlan d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.n_x) return;
  const int q = d.lp_cp[j];
  if (q < d.lp_cp[j + 1] && d.lp_row[q] == j) d.lp_v[q] = dadd(d.lp_v[q], d.delta);
}

// ---------------------------------------------------------------------------
// Step a7: multifrontal supernodal Cholesky of the permuted Hgamma
// (replaces cusolverSpDcsrcholFactor, CholeskyClass.cpp:71-90).
// Front J is an n_J x n_J column-major block (ld n_J) at front + sn_off[J];
// its first ncols columns hold L(rows(J), cols(J)) after factorization, the
// trailing (n_J-ncols)^2 block holds the update (contribution) matrix that
// the parent front adds in.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void note_pivot(DevPlan& d, int col, double piv) {
  if (!(piv > d.pivot_tol) || !(piv <= 1.79e308)) atomicMin(&d.sc->pivot_col, col);
}

// Small fronts: one CTA per front, whole front in shared memory.
__global__ void __launch_bounds__(kBlock) k_front_small(DevPlan d, const int* __restrict__ list) {
  extern __shared__ double F[];
  const int J = list[blockIdx.x];
  const int first = d.sn_first[J];
  const int ncols = d.sn_first[J + 1] - first;
  const int nJ = d.sn_nrows[J];
  const int tid = threadIdx.x;
  const int nn = nJ * nJ;
  for (int i = tid; i < nn; i += blockDim.x) F[i] = 0.0;
  __syncthreads();
  // original entries of the supernode's columns
  const int q0 = d.lp_cp[first], q1 = d.lp_cp[first + ncols];
  for (int q = q0 + tid; q < q1; q += blockDim.x) {
    // column of entry q: search the (short) column pointer range
    int c = 0;
    while (d.lp_cp[first + c + 1] <= q) ++c;
    F[c * nJ + d.lp_lrow[q]] = d.lp_v[q];
  }
  __syncthreads();
  // extend-add of the children's update matrices, children in order
  for (int cc = d.sn_child_rp[J]; cc < d.sn_child_rp[J + 1]; ++cc) {
    const int ch = d.sn_children[cc];
    const int nc = d.sn_nrows[ch];
    const int ncc = d.sn_first[ch + 1] - d.sn_first[ch];
    const int R = nc - ncc;
    const int* rel = d.sn_rel + d.sn_relp[ch];
    const double* CB = d.front + d.sn_off[ch] + (int64_t)ncc * nc + ncc;
    for (int idx = tid; idx < R * R; idx += blockDim.x) {
      const int a = idx % R, b = idx / R;
      if (a >= b) F[rel[b] * nJ + rel[a]] += CB[(int64_t)b * nc + a];
    }
    __syncthreads();
  }
  // right-looking partial Cholesky of the first ncols columns
  __shared__ double piv;
  for (int k = 0; k < ncols; ++k) {
    if (tid == 0) {
      double dk = F[k * nJ + k];
      note_pivot(d, first + k, dk);
      piv = sqrt(dk);
      F[k * nJ + k] = piv;
    }
    __syncthreads();
    const double pk = piv;
    for (int i = k + 1 + tid; i < nJ; i += blockDim.x) F[k * nJ + i] = F[k * nJ + i] / pk;
    __syncthreads();
    const int m = nJ - k - 1;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int ii = idx % m, jj = idx / m;
      if (ii >= jj) {
        const int i = k + 1 + ii, j = k + 1 + jj;
        F[j * nJ + i] = fma(-F[k * nJ + i], F[k * nJ + j], F[j * nJ + i]);
      }
    }
    __syncthreads();
  }
  double* G = d.front + d.sn_off[J];
  for (int i = tid; i < nn; i += blockDim.x) G[i] = F[i];
}

// Large fronts: scatter original entries (front zeroed by a memset before).
__global__ void k_front_scatter(DevPlan d, const int* __restrict__ list) {
  const int J = list[blockIdx.x];
  const int first = d.sn_first[J];
  const int ncols = d.sn_first[J + 1] - first;
  const int nJ = d.sn_nrows[J];
  double* G = d.front + d.sn_off[J];
  for (int c = 0; c < ncols; ++c) {
    const int q0 = d.lp_cp[first + c], q1 = d.lp_cp[first + c + 1];
    for (int q = q0 + threadIdx.x + blockIdx.y * blockDim.x; q < q1; q += blockDim.x * gridDim.y)
      G[(int64_t)c * nJ + d.lp_lrow[q]] = d.lp_v[q];
  }
}

// Large fronts: extend-add, one CTA per 32-row chunk of the parent front,
// children in order (deterministic; no atomics).
__global__ void __launch_bounds__(kBlock) k_front_extadd(DevPlan d, const int* __restrict__ ea_sn, const int* __restrict__ ea_row0) {
  const int J = ea_sn[blockIdx.x];
  const int row0 = ea_row0[blockIdx.x];
  const int nJ = d.sn_nrows[J];
  double* G = d.front + d.sn_off[J];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  __shared__ int s_lo, s_hi;
  for (int cc = d.sn_child_rp[J]; cc < d.sn_child_rp[J + 1]; ++cc) {
    const int ch = d.sn_children[cc];
    const int nc = d.sn_nrows[ch];
    const int ncc = d.sn_first[ch + 1] - d.sn_first[ch];
    const int R = nc - ncc;
    const int* rel = d.sn_rel + d.sn_relp[ch];
    if (threadIdx.x == 0) {
      int lo = 0, hi = R;
      while (lo < hi) { int mid = (lo + hi) >> 1; if (rel[mid] < row0) lo = mid + 1; else hi = mid; }
      int a_lo = lo;
      hi = R;
      while (lo < hi) { int mid = (lo + hi) >> 1; if (rel[mid] < row0 + kEaRows) lo = mid + 1; else hi = mid; }
      s_lo = a_lo;
      s_hi = lo;
    }
    __syncthreads();
    const int a_lo = s_lo, a_hi = s_hi;
    if (a_hi > a_lo) {
      const double* CB = d.front + d.sn_off[ch] + (int64_t)ncc * nc + ncc;
      const int a = a_lo + lane;
      const int ra = a < a_hi ? rel[a] : 0;
      for (int b = warp; b < a_hi; b += nwarp) {
        if (a < a_hi && a >= b) {
          G[(int64_t)rel[b] * nJ + ra] += CB[(int64_t)b * nc + a];
        }
      }
    }
    __syncthreads();
  }
}

// Panel p of the blocked factorization: Cholesky of the diagonal block.
__global__ void __launch_bounds__(kBlock) k_panel_potrf(DevPlan d, const int* __restrict__ sn, int p) {
  __shared__ double A[kPanel * kPanel];
  __shared__ double piv;
  const int J = sn[blockIdx.x];
  const int first = d.sn_first[J];
  const int ncols = d.sn_first[J + 1] - first;
  const int nJ = d.sn_nrows[J];
  const int c0 = p * kPanel;
  const int w = min(kPanel, ncols - c0);
  double* G = d.front + d.sn_off[J];
  const int tid = threadIdx.x;
  for (int idx = tid; idx < w * w; idx += blockDim.x) {
    const int i = idx % w, j = idx / w;
    A[j * kPanel + i] = (i >= j) ? G[(int64_t)(c0 + j) * nJ + c0 + i] : 0.0;
  }
  __syncthreads();
  for (int k = 0; k < w; ++k) {
    if (tid == 0) {
      double dk = A[k * kPanel + k];
      note_pivot(d, first + c0 + k, dk);
      piv = sqrt(dk);
      A[k * kPanel + k] = piv;
    }
    __syncthreads();
    const double pk = piv;
    for (int i = k + 1 + tid; i < w; i += blockDim.x) A[k * kPanel + i] = A[k * kPanel + i] / pk;
    __syncthreads();
    const int m = w - k - 1;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int ii = idx % m, jj = idx / m;
      if (ii >= jj) {
        const int i = k + 1 + ii, j = k + 1 + jj;
        A[j * kPanel + i] = fma(-A[k * kPanel + i], A[k * kPanel + j], A[j * kPanel + i]);
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < w * w; idx += blockDim.x) {
    const int i = idx % w, j = idx / w;
    if (i >= j) G[(int64_t)(c0 + j) * nJ + c0 + i] = A[j * kPanel + i];
  }
}

// Panel p: rows below the diagonal block, X = B L11^{-T}; one thread per row.
__global__ void __launch_bounds__(kTrsmRows) k_panel_trsm(DevPlan d, const int* __restrict__ sn, const int* __restrict__ row0s, int p) {
  __shared__ double A[kPanel * kPanel];
  const int J = sn[blockIdx.x];
  const int first = d.sn_first[J];
  const int ncols = d.sn_first[J + 1] - first;
  const int nJ = d.sn_nrows[J];
  const int c0 = p * kPanel;
  const int w = min(kPanel, ncols - c0);
  const double* __restrict__ Gc = d.front + d.sn_off[J];
  double* G = d.front + d.sn_off[J];
  for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
    const int i = idx % w, j = idx / w;
    A[j * kPanel + i] = (i >= j) ? Gc[(int64_t)(c0 + j) * nJ + c0 + i] : 0.0;
  }
  __syncthreads();
  const int r = row0s[blockIdx.x] + threadIdx.x;
  if (r >= nJ) return;
  double x[kPanel];
#pragma unroll
  for (int t = 0; t < kPanel; ++t) x[t] = t < w ? Gc[(int64_t)(c0 + t) * nJ + r] : 0.0;
#pragma unroll
  for (int j = 0; j < kPanel; ++j) {
    if (j < w) {
      double v = x[j];
#pragma unroll
      for (int t = 0; t < kPanel; ++t)
        if (t < j) v = fma(-x[t], A[t * kPanel + j], v);
      x[j] = v / A[j * kPanel + j];
    }
  }
#pragma unroll
  for (int t = 0; t < kPanel; ++t)
    if (t < w) G[(int64_t)(c0 + t) * nJ + r] = x[t];
}

// Panel p: trailing update C -= A_i A_j^T on 64x64 lower tiles.
__global__ void __launch_bounds__(kBlock) k_panel_update(DevPlan d, const int* __restrict__ sn, const int* __restrict__ tis,
                                                          const int* __restrict__ tjs, int p) {
  __shared__ double As[kPanel][kTile + 1];
  __shared__ double Bs[kPanel][kTile + 1];
  const int J = sn[blockIdx.x];
  const int first = d.sn_first[J];
  const int ncols = d.sn_first[J + 1] - first;
  const int nJ = d.sn_nrows[J];
  const int c0 = p * kPanel;
  const int w = min(kPanel, ncols - c0);
  const int ti = tis[blockIdx.x], tj = tjs[blockIdx.x];
  double* G = d.front + d.sn_off[J];
  for (int idx = threadIdx.x; idx < kPanel * kTile; idx += blockDim.x) {
    const int r = idx % kTile, t = idx / kTile;
    double a = 0.0, b = 0.0;
    if (t < w) {
      if (ti + r < nJ) a = G[(int64_t)(c0 + t) * nJ + ti + r];
      if (tj + r < nJ) b = G[(int64_t)(c0 + t) * nJ + tj + r];
    }
    As[t][r] = a;
    Bs[t][r] = b;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int t = 0; t < w; ++t) {
    double a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = As[t][tx + 16 * i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = Bs[t][ty + 16 * j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = tj + ty + 16 * j;
    if (c >= nJ) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ti + tx + 16 * i;
      if (r < nJ && r >= c) {
        double* g = G + (int64_t)c * nJ + r;
        *g = *g - acc[i][j];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Inverses of the items' diagonal blocks, computed once per factorization:
// the solves then apply X_q = L_qq^{-1} as dense products instead of serial
// substitutions with FP64 divisions.
//   * items with <= 64 columns: one CTA each (k_piece_inverse), column j of
//     X by X[j][j] = 1/L[j][j], X[i][j] = -(sum_{k=j}^{i-1} L[i][k] X[k][j]) / L[i][i];
//   * larger items: blocked, by 32-row steps i over all of them at once:
//     X starts as the identity; k_trtri_diag solves L_ii X_i = X_i on the
//     step's block row (columns < 32(i+1)), k_trtri_update subtracts
//     L_ri X_i from every block row r below (64x64 tiles).
// X is stored column-major, nc x nc, at sq_doff[q] in the inverse arena.
// ---------------------------------------------------------------------------
constexpr int kInvSmem = (2 * kPiece * (kPiece + 1) + kPiece) * 8;  // dynamic shared memory of k_piece_inverse

__global__ void __launch_bounds__(kBlock) k_piece_inverse(DevPlan d, const int* __restrict__ items) {
  extern __shared__ double inv_smem[];
  double* Ls = inv_smem;
  double* Xs = Ls + kPiece * (kPiece + 1);
  double* rdiag = Xs + kPiece * (kPiece + 1);
  const int q = items[blockIdx.x];
  const int J = d.sq_sn[q], c0 = d.sq_c0[q], c1 = d.sq_c1[q];
  const int nc = c1 - c0;
  const int nJ = d.sn_nrows[J];
  const double* L = d.front + d.sn_off[J] + (int64_t)c0 * nJ + c0;
  constexpr int ld = kPiece + 1;
  for (int idx = threadIdx.x; idx < nc * nc; idx += blockDim.x) {
    const int r = idx % nc, t = idx / nc;
    Ls[t * ld + r] = (r >= t) ? L[(int64_t)t * nJ + r] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < nc) rdiag[threadIdx.x] = 1.0 / Ls[threadIdx.x * ld + threadIdx.x];
  __syncthreads();
  // one thread per column j; rows i ascending
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    Xs[j * ld + j] = rdiag[j];
    for (int i = j + 1; i < nc; ++i) {
      double acc = 0.0;
      for (int k = j; k < i; ++k) acc = fma(Ls[k * ld + i], Xs[j * ld + k], acc);
      Xs[j * ld + i] = -acc * rdiag[i];
    }
  }
  __syncthreads();
  double* X = d.dinv + d.dinv_off[q];
  for (int idx = threadIdx.x; idx < nc * nc; idx += blockDim.x) {
    const int r = idx % nc, t = idx / nc;
    X[(int64_t)t * nc + r] = (r >= t) ? Xs[t * ld + r] : 0.0;
  }
}

__global__ void k_trtri_init(DevPlan d, const int* __restrict__ items) {
  const int q = items[blockIdx.y];
  const int64_t nc = d.sq_c1[q] - d.sq_c0[q];
  double* X = d.dinv + d.dinv_off[q];
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nc * nc; idx += (int64_t)gridDim.x * blockDim.x)
    X[idx] = (idx % nc == idx / nc) ? 1.0 : 0.0;
}

// Step i, block row [32i, 32i+w): X_i = L_ii^{-1} X_i for the columns
// [c0t, c0t+256) of the tile (columns < 32(i+1)); one thread per column.
__global__ void __launch_bounds__(kDiagCols) k_trtri_diag(DevPlan d, const int* __restrict__ items, const int* __restrict__ ctile, int i) {
  __shared__ double A[kPanel * (kPanel + 1)];
  const int q = items[blockIdx.x];
  const int J = d.sq_sn[q], c0 = d.sq_c0[q];
  const int nc = d.sq_c1[q] - c0;
  const int nJ = d.sn_nrows[J];
  const int b0 = i * kPanel;
  const int w = min(kPanel, nc - b0);
  const double* Lq = d.front + d.sn_off[J] + (int64_t)c0 * nJ + c0;
  for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
    const int r = idx % w, t = idx / w;
    A[t * (kPanel + 1) + r] = (r >= t) ? Lq[(int64_t)(b0 + t) * nJ + b0 + r] : 0.0;
  }
  __syncthreads();
  const int c = ctile[blockIdx.x] + threadIdx.x;
  if (c >= min(nc, b0 + w)) return;
  double* Xc = d.dinv + d.dinv_off[q] + (int64_t)c * nc + b0;
  double x[kPanel];
#pragma unroll
  for (int t = 0; t < kPanel; ++t) x[t] = t < w ? Xc[t] : 0.0;
#pragma unroll
  for (int j = 0; j < kPanel; ++j) {
    if (j < w) {
      double v = x[j];
#pragma unroll
      for (int t = 0; t < kPanel; ++t)
        if (t < j) v = fma(-A[t * (kPanel + 1) + j], x[t], v);
      x[j] = v / A[j * (kPanel + 1) + j];
    }
  }
#pragma unroll
  for (int t = 0; t < kPanel; ++t)
    if (t < w) Xc[t] = x[t];
}

// Step i: X[r0:r0+64, c0t:c0t+64] -= L[r0:r0+64, 32i:32i+32] X[32i:32i+32, c0t:c0t+64]
// for block rows below the step (r0 >= 32(i+1)) and columns < 32(i+1).
__global__ void __launch_bounds__(kBlock) k_trtri_update(DevPlan d, const int* __restrict__ items, const int* __restrict__ trow,
                                                          const int* __restrict__ tcol, int i) {
  __shared__ double As[kPanel][kTile + 1];
  __shared__ double Bs[kPanel][kTile + 1];
  const int q = items[blockIdx.x];
  const int J = d.sq_sn[q], c0 = d.sq_c0[q];
  const int nc = d.sq_c1[q] - c0;
  const int nJ = d.sn_nrows[J];
  const int b0 = i * kPanel;
  const int w = min(kPanel, nc - b0);
  const int cmax = min(nc, b0 + w);
  const int r0 = trow[blockIdx.x], ct = tcol[blockIdx.x];
  const double* Lq = d.front + d.sn_off[J] + (int64_t)c0 * nJ + c0;
  double* X = d.dinv + d.dinv_off[q];
  for (int idx = threadIdx.x; idx < kPanel * kTile; idx += blockDim.x) {
    const int r = idx % kTile, t = idx / kTile;
    As[t][r] = (t < w && r0 + r < nc) ? Lq[(int64_t)(b0 + t) * nJ + r0 + r] : 0.0;
  }
  for (int idx = threadIdx.x; idx < kPanel * kTile; idx += blockDim.x) {
    const int t = idx % kPanel, c = idx / kPanel;
    Bs[t][c] = (t < w && ct + c < cmax) ? X[(int64_t)(ct + c) * nc + b0 + t] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int t = 0; t < w; ++t) {
    double a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = As[t][tx + 16 * k];
#pragma unroll
    for (int k = 0; k < 4; ++k) b[k] = Bs[t][ty + 16 * k];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
  }
#pragma unroll
  for (int y = 0; y < 4; ++y) {
    const int c = ct + ty + 16 * y;
    if (c >= cmax) continue;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const int r = r0 + tx + 16 * x;
      if (r < nc) {
        double* g = X + (int64_t)c * nc + r;
        *g = *g - acc[x][y];
      }
    }
  }
}

// Packed copies of a panelized item's rows-below block L21 (R x nc, from the
// front): forward 16-row chunks [row chunk][col][16] and backward 16-column
// panels [panel][row][16]; rows past R and columns past nc are zeros.
__global__ void k_l21_pack(DevPlan d, int q, int64_t off_f, int64_t off_b) {
  const int J = d.sq_sn[q], c0 = d.sq_c0[q], c1 = d.sq_c1[q];
  const int nc = c1 - c0, nJ = d.sn_nrows[J], R = nJ - c1;
  const double* L = d.front + d.sn_off[J] + (int64_t)c0 * nJ + c1;  // L21(i, t) = L[t * nJ + i]
  const int64_t nf = (int64_t)((R + 15) / 16) * 16 * nc, nb = (int64_t)((nc + 15) / 16) * 16 * R;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nf; e += stride) {
    const int r = (int)(e & 15);
    const int64_t rest = e >> 4;
    const int t = (int)(rest % nc), c = (int)(rest / nc);
    const int i = c * 16 + r;
    d.l21f[off_f + e] = i < R ? L[(int64_t)t * nJ + i] : 0.0;
  }
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nb; e += stride) {
    const int tt = (int)(e & 15);
    const int64_t rest = e >> 4;
    const int i = (int)(rest % R), b = (int)(rest / R);
    const int t = b * 16 + tt;
    d.l21b[off_b + e] = t < nc ? L[(int64_t)t * nJ + i] : 0.0;
  }
}

// Row panels of a large item's X (layout: xpanel_fwd / xpanel_bwd in
// symbolic.hpp), copied from the column-major inverse; entries outside the
// triangle and rows past nc are stored as zeros.  One CTA per (item, panel).
__global__ void __launch_bounds__(kBlock) k_xpanel_pack(DevPlan d, const int* __restrict__ pq, const int* __restrict__ pb,
                                                         const int* __restrict__ rows_x) {
  const int q = pq[blockIdx.x], b = pb[blockIdx.x];
  const int nc = d.sq_c1[q] - d.sq_c0[q];
  const int RT = rows_x[q];
  const int r0 = b * RT;
  const double* X = d.dinv + d.dinv_off[q];
  double* P = d.xpanel + d.xp_off[q];
  {  // forward: P[k*RT + rl] = X[r0+rl][k], k < min(nc, r0+RT)
    double* F = P + xpanel_fwd(RT, nc, b);
    const int K = min(nc, r0 + RT);
    for (int64_t idx = threadIdx.x; idx < (int64_t)K * RT; idx += kBlock) {
      const int k = (int)(idx / RT), r = r0 + (int)(idx % RT);
      F[idx] = (r < nc && k <= r) ? X[(int64_t)k * nc + r] : 0.0;
    }
  }
  {  // backward: P[(k-r0)*RT + rl] = X[k][r0+rl], k in [r0, nc)
    double* Bk = P + xpanel_bwd(RT, nc, b);
    const int K = nc - r0;
    for (int64_t idx = threadIdx.x; idx < (int64_t)K * RT; idx += kBlock) {
      const int k = r0 + (int)(idx / RT), t = r0 + (int)(idx % RT);
      Bk[idx] = (t < nc && k >= t) ? X[(int64_t)t * nc + k] : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Step a8: triangular solves with the supernodal factor
// (replaces cusolverSpDcsrcholSolve, CholeskyClass.cpp:93-101).
//
// Items are supernodes (or column pieces of them, an option of the symbolic
// plan).  Forward item q:
//   b'_q = b_q - (updates u of the descendant items whose rows are q's columns)
//   x_q  = X_q b'_q            u_q = L21_q x_q   (L21: the rows below the item)
// Backward item q:
//   y'_q = x_q - L21_q^T x_R   x_q = X_q^T y'_q
// No step is a serial substitution: every step is a gather or a dense
// product.  A small item (n_J - c0 <= 256 rows, <= 64 columns) is one task
// per direction; a large item is split into stages whose tasks run on many
// SMs at once (SolveTask in symbolic.hpp: GATHER / INV / L21 forward, L21T /
// REDUCE / INVT backward).
// One persistent launch per direction: CTAs claim tasks in topological order
// from a global counter and wait (bounded) on dependency counters.  A task
// only waits on tasks claimed before it, by CTAs that are running, so the
// scheme cannot deadlock whatever the number of resident CTAs.  Data written
// by other CTAs of the same launch is read with ld.global.cg (__ldcg).
// Every sum is taken in a fixed order, so a solve is bit-reproducible.
// ---------------------------------------------------------------------------
// resident CTAs per SM the persistent solve kernels are compiled for (the
// register budget per thread follows from it: 48 at 5).  Five rather than
// four measured 4.49 -> 4.63 solves/s with 8 plans sharing the GPU (more
// CTAs of different plans per SM keep its FP64 pipe busier) and the same
// single-plan time.
#ifndef HYKKT_TRSV_MIN_BLOCKS
#define HYKKT_TRSV_MIN_BLOCKS 5
#endif
constexpr int kLs = kPiece + 1;      // padded column stride of a small X block in shared memory
constexpr unsigned kSpinLimit = 1u << 24;
constexpr int kStage = 2048;         // doubles of a staged vector segment
// shared memory of the solve kernels (doubles): a small X block, one vector
// of its columns, one of the rows below it and a reduction buffer; or a
// stage + reduction buffer
constexpr int kTrsvSmem = kPiece * kLs + kPiece + kSmallItemRows + kBlock;
static_assert(kStage + kBlock <= kTrsvSmem, "stage + reduction buffer must fit the shared buffer");
static_assert(kStage >= kMaxUnitCols, "a panel unit's vector segment must fit one stage");
static_assert(kMaxUnitCols + kMaxUnitCols / 2 + kBlock <= kTrsvSmem, "panel product scratch must fit the shared buffer");
static_assert(kSmallItemRows + kBlock + 32 * (128 + 1) <= kTrsvSmem, "L21T tile must fit the shared buffer");
static_assert(kSmallItemRows <= kBlock, "a fused item's rows are one thread each");

// back-off between polls of a dependency counter (ns; 0: none)
#ifndef HYKKT_SPIN_NS
#define HYKKT_SPIN_NS 64
#endif

// Waits until *p >= need.  Bounded: after d.spin_limit polls it records the
// timeout in solve_flags (the solve then reports HYKKT_TIMEOUT, its results
// invalid) and continues; once any wait of the solve has given up, the others
// return at once and the CG and refinement loops stop, so a solve with a
// missing signal ends after one spin limit.  d.dbg_unsatisfiable (a test
// hook, 0 in use) raises every count to one that no task reaches.
__device__ __forceinline__ void wait_ge(const int* p, int need, const DevPlan& d) {
  need += d.dbg_unsatisfiable;
  if (need <= 0) return;
  volatile const int* flags = &d.sc->solve_flags;
  for (unsigned it = 0; *(volatile const int*)p < need; ++it) {
    if (it > d.spin_limit || (*flags & 1)) {
      atomicOr(&d.sc->solve_flags, 1);
      break;
    }
    if (HYKKT_SPIN_NS > 0) __nanosleep(HYKKT_SPIN_NS);
  }
  __threadfence();
}

// thread 0 waits, then the whole CTA proceeds
__device__ __forceinline__ void cta_wait_ge(const int* p, int need, const DevPlan& d) {
  if (threadIdx.x == 0) wait_ge(p, need, d);
  __syncthreads();
}

// optional timeline: slot e of task k (0 claimed, 1 dependencies met, 2 done,
// 3 SM id).  Compiled in only for measurement builds (HYKKT_MEASURE); the
// shipped library's solve kernels carry no timer reads.
__device__ __forceinline__ void trace_mark(const DevPlan& d, int k, int e) {
#ifndef HYKKT_MEASURE
  (void)d, (void)k, (void)e;
#else
  if (d.trace && threadIdx.x == 0) {
    unsigned long long t;
    if (e == 3) {
      unsigned int sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      t = sm;
    } else {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    }
    d.trace[4 * (int64_t)k + e] = t;
  }
#endif
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = dadd(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }

// out[i] = sum_{k<K} M[k*ld + r0 + i] v[k] for i < nr: RT (a power of two,
// 16..256) rows per CTA, kBlock/RT column parts per row, NB loads in flight
// per thread (eight accumulators), v staged through shared memory in kStage
// segments, the parts summed in order.  With ld == RT (a row panel) each
// step of the CTA reads one contiguous block of kBlock doubles.
template <int NB = 8>
__device__ void rows_times_vec(const double* __restrict__ M, int64_t ld, int r0, int nr, int RT, int K,
                               const double* v, double* out, double* sm, double* out2 = nullptr) {
  static_assert(NB % 8 == 0, "loads in flight: a multiple of the eight accumulators");
  double* stage = sm;
  double* red = sm + kStage;
  const int rl = threadIdx.x & (RT - 1);
  const int part = threadIdx.x / RT;
  const int KP = kBlock / RT;
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = 0.0;
  for (int kb = 0; kb < K; kb += kStage) {
    const int kn = min(kStage, K - kb);
    __syncthreads();
    for (int t = threadIdx.x; t < kn; t += kBlock) stage[t] = __ldcg(&v[kb + t]);
    __syncthreads();
    const double* Mr = M + (int64_t)kb * ld + r0 + rl;
    int k = part;
    for (; k + (NB - 1) * KP < kn; k += NB * KP) {
      double m[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j) m[j] = Mr[(int64_t)(k + j * KP) * ld];
#pragma unroll
      for (int j = 0; j < NB; ++j) a[j % 8] = fma(m[j], stage[k + j * KP], a[j % 8]);
    }
    for (; k + 7 * KP < kn; k += 8 * KP) {
      double m[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) m[j] = Mr[(int64_t)(k + j * KP) * ld];
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] = fma(m[j], stage[k + j * KP], a[j]);
    }
    for (; k < kn; k += KP) a[0] = fma(Mr[(int64_t)k * ld], stage[k], a[0]);
  }
  red[threadIdx.x] = dadd(dadd(dadd(a[0], a[1]), dadd(a[2], a[3])), dadd(dadd(a[4], a[5]), dadd(a[6], a[7])));
  __syncthreads();
  if (part == 0 && rl < nr) {
    double s = red[rl];
    for (int p = 1; p < KP; ++p) s = dadd(s, red[p * RT + rl]);
    out[rl] = s;
    if (out2) out2[rl] = s;
  }
}

// f(t, sum_{i<nr} M[t*ld + i] v[i]) for t < nc (column dot products, v in
// shared memory): TC = min(nc, kBlock) column lanes x kBlock/TC row parts,
// eight loads in flight per thread, the parts summed in order through `red`
// (kBlock doubles of shared memory); f runs in the thread of part 0.
template <class F>
__device__ __forceinline__ void column_dots(const double* __restrict__ M, int64_t ld, int nc, int nr, const double* v,
                                            double* red, F f) {
  const int TC = nc < kBlock ? nc : kBlock;
  const int P = kBlock / TC;
  const int tl = threadIdx.x % TC, p = threadIdx.x / TC;
  for (int c0 = 0; c0 < nc; c0 += TC) {
    const int t = c0 + tl;
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 0.0;
    if (p < P && t < nc) {
      const double* Mt = M + (int64_t)t * ld;
      int i = p;
      for (; i + 7 * P < nr; i += 8 * P) {
        double m[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) m[j] = Mt[i + j * P];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(m[j], v[i + j * P], a[j]);
      }
      for (; i < nr; i += P) a[0] = fma(Mt[i], v[i], a[0]);
    }
    __syncthreads();
    red[threadIdx.x] = dadd(dadd(dadd(a[0], a[1]), dadd(a[2], a[3])), dadd(dadd(a[4], a[5]), dadd(a[6], a[7])));
    __syncthreads();
    if (p == 0 && t < nc) {
      double sum = red[tl];
      for (int j = 1; j < P; ++j) sum = dadd(sum, red[j * TC + tl]);
      f(t, sum);
    }
  }
}

// f(t, sum_{i<nr} M[t*ld + i] v[i]) for t < nc, M column-major: 32-row x
// 128-column tiles of M are copied to shared memory with coalesced loads (a
// warp reads 32 consecutive rows of a column), then each thread sums its
// column's rows from shared memory (two threads per column, the halves
// added in order).  `tile` holds kTileR x (kTileC + 1) doubles, `red` kBlock.
constexpr int kTileR = 32, kTileC = 128;
template <class F>
__device__ void column_dots_tiled(const double* __restrict__ M, int64_t ld, int nc, int nr, const double* v,
                                  double* tile, double* red, F f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tc = threadIdx.x % kTileC, part = threadIdx.x / kTileC;  // 2 parts
  for (int c0 = 0; c0 < nc; c0 += kTileC) {
    const int cn = min(kTileC, nc - c0);
    double acc = 0.0;
    for (int r0 = 0; r0 < nr; r0 += kTileR) {
      const int rn = min(kTileR, nr - r0);
      __syncthreads();
      for (int c = warp; c < cn; c += kBlock / 32)
        tile[lane * (kTileC + 1) + c] = lane < rn ? M[(int64_t)(c0 + c) * ld + r0 + lane] : 0.0;
      __syncthreads();
      if (tc < cn)
        for (int r = part; r < rn; r += 2) acc = fma(tile[r * (kTileC + 1) + tc], v[r0 + r], acc);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    if (part == 0 && tc < cn) f(c0 + tc, dadd(red[tc], red[kTileC + tc]));
    __syncthreads();
  }
}

// Copies the nr x nc block L (column-major, leading dimension ld) to shared
// memory Ls with leading dimension lds (>= nr).  All loads are independent,
// so a task issues them before it waits on its dependencies.
__device__ __forceinline__ void stage_block(const double* __restrict__ L, int64_t ld, int nr, int nc, double* Ls, int lds) {
  for (int idx = threadIdx.x; idx < nr * nc; idx += kBlock) {
    const int t = idx / nr, i = idx - t * nr;
    Ls[t * lds + i] = L[(int64_t)t * ld + i];
  }
}

// out[i] = sum_{t<nc} Ls[t*nr + i] v[t] for i < nr (Ls and v in shared
// memory): kBlock/nr parts per row, the parts summed in order through `red`.
__device__ __forceinline__ void block_rows_times_vec(const double* Ls, int nr, int nc, const double* v, double* red,
                                                     double* out) {
  const int P = kBlock / nr;
  const int i = threadIdx.x % nr, p = threadIdx.x / nr;
  double a0 = 0.0, a1 = 0.0;
  if (p < P) {
    int t = p;
    for (; t + P < nc; t += 2 * P) {
      a0 = fma(Ls[t * nr + i], v[t], a0);
      a1 = fma(Ls[(t + P) * nr + i], v[t + P], a1);
    }
    if (t < nc) a0 = fma(Ls[t * nr + i], v[t], a0);
  }
  red[threadIdx.x] = dadd(a0, a1);
  __syncthreads();
  if (threadIdx.x < nr) {
    double s = red[i];
    for (int j = 1; j < P; ++j) s = dadd(s, red[j * nr + i]);
    out[i] = s;
  }
}

// Sum over the chunks c = c_beg + g, c_beg + g + G, ... < c_end of
// part[base + (c - c0) * stride], in that order, eight loads in flight.
__device__ __forceinline__ double strided_chunk_sum(const double* part, int64_t base, int64_t stride, int c0, int c_beg,
                                                    int c_end, int G) {
  double acc = 0.0;
  int c = c_beg;
  for (; c + 7 * G < c_end; c += 8 * G) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __ldcg(&part[base + (int64_t)(c + j * G - c0) * stride]);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc = dadd(acc, v[j]);
  }
  for (; c < c_end; c += G) acc = dadd(acc, __ldcg(&part[base + (int64_t)(c - c0) * stride]));
  return acc;
}

// Dependency counters, one block per direction:
//   forward  [head_f, diag_cnt, g_done, inv_done, child_done (nsq each), panel_f (npanels),
//             fch_cnt (forward chunks)]
//   backward [head_b, bg_cnt (nchunks), bd_cnt, red_done, invt_done (nsq each), panel_b (npanels)]
// A solve pair needs each block at zero when its kernel starts: the forward
// kernel clears the backward block and the backward kernel the forward one
// (the other kernel of the pair does not touch them), so consecutive pairs
// need no reset in between.  Both kernels of a pair skip together when the
// CG has stopped, which keeps that invariant.
__device__ __host__ inline int64_t trsv_fwd_counters(int nsq, int npanels, int nfch) {
  return 1 + 4LL * nsq + npanels + nfch;
}
__device__ __host__ inline int64_t trsv_bwd_counters(int nsq, int nchunks, int npanels) {
  return 1 + (int64_t)nchunks + 3LL * nsq + npanels;
}
struct TrsvCounters {
  int *head_f, *head_b, *diag_cnt, *g_done, *inv_done, *bg_cnt, *bd_cnt, *red_done, *invt_done, *panel_f, *panel_b,
      *child_done, *fch_cnt;
  __device__ explicit TrsvCounters(const SolveSched& s) {
    head_f = s.cnt;
    diag_cnt = head_f + 1;
    g_done = diag_cnt + s.nsq;
    inv_done = g_done + s.nsq;
    child_done = inv_done + s.nsq;
    panel_f = child_done + s.nsq;
    fch_cnt = panel_f + s.npanels;
    head_b = fch_cnt + s.nfchunks;
    bg_cnt = head_b + 1;
    bd_cnt = bg_cnt + s.nchunks;
    red_done = bd_cnt + s.nsq;
    invt_done = red_done + s.nsq;
    panel_b = invt_done + s.nsq;
  }
  __device__ void clear_range(int* p, int n) const {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
  }
  __device__ void clear_fwd(const SolveSched& s) const {
    clear_range(head_f, (int)trsv_fwd_counters(s.nsq, s.npanels, s.nfchunks));
  }
  __device__ void clear_bwd(const SolveSched& s) const {
    clear_range(head_b, (int)trsv_bwd_counters(s.nsq, s.nchunks, s.npanels));
  }
};

// loads in flight per thread in the panel units (the FP64-bound products of
// the widest items)
#ifndef HYKKT_UNIT_LOADS
#define HYKKT_UNIT_LOADS 16
#endif
constexpr int kUnitLoads = HYKKT_UNIT_LOADS;

// One unit (columns [k0, k0+kn) of a row panel P with leading dimension RT)
// of a panel product into `out` (nr rows).  A panel with one unit writes
// out directly; otherwise the unit stores its partial sums in the panel's
// slot and the last unit to finish adds the slot's partials in unit order.
// Returns true in every thread of the CTA that completed the panel.
// out2 (optional): a second copy of the panel's rows
__device__ bool panel_unit(const double* __restrict__ P, int RT, int nr, int K, int unit, int seg, const double* v,
                           double* out, double* slot, int* panel_cnt, double* sm, int* flag, double* out2 = nullptr) {
  const int nunits = ceil_div(K, seg);
  const int k0 = unit * seg;
  const int kn = min(seg, K - k0);
  if (nunits == 1) {
    rows_times_vec<kUnitLoads>(P, RT, 0, nr, RT, K, v, out, sm, out2);
    return true;
  }
  rows_times_vec<kUnitLoads>(P + (int64_t)k0 * RT, RT, 0, nr, RT, kn, v + k0, slot + (int64_t)unit * RT, sm);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *flag = atomicAdd(panel_cnt, 1) == nunits - 1;
  __syncthreads();
  if (!*flag) return false;
  __threadfence();
  if (threadIdx.x < nr) {
    double acc = __ldcg(&slot[threadIdx.x]);
    for (int u = 1; u < nunits; ++u) acc = dadd(acc, __ldcg(&slot[(int64_t)u * RT + threadIdx.x]));
    out[threadIdx.x] = acc;
    if (out2) out2[threadIdx.x] = acc;
  }
  return true;
}

// make the CTA's global writes visible, then one signal per target item of
// chunk ch (target lists t_rp / t_item)
__device__ __forceinline__ void signal_chunk_items(const int* t_rp, const int* t_item, int ch, int* diag_cnt) {
  __threadfence();
  __syncthreads();
  for (int p = t_rp[ch] + threadIdx.x; p < t_rp[ch + 1]; p += kBlock) atomicAdd(&diag_cnt[t_item[p]], 1);
}

__device__ __forceinline__ void signal_count(int* c) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(c, 1);
}

// item q finished in the backward direction: notify the chunks with rows in
// its columns (an item near the root notifies thousands: spread over the CTA)
__device__ __forceinline__ void signal_item_done(const SolveSched& s, int q, int* bg_cnt) {
  __threadfence();
  __syncthreads();
  for (int p = s.ic_rp[q] + threadIdx.x; p < s.ic_rp[q + 1]; p += kBlock) atomicAdd(&bg_cnt[s.ic_chunk[p]], 1);
}

// forward product tasks of a head item: one (it wrote all of x_q)
__device__ __forceinline__ int inv_tasks(const SolveSched& s, int q, int nc) {
  return s.mode[q] == ITEM_HEAD ? 1 : ceil_div(nc, s.rows_x[q]);
}

// L2 prefetch hints, issued by a task before it waits on its dependencies so
// that the factor data it streams is on chip when they are met.  One 128-byte
// line per instruction, spread over the threads [0, nt) of the calling group
// (tid = index in the group); every address lies inside the given range.
__device__ __forceinline__ void prefetch_bytes(const void* p, int64_t bytes, int tid, int nt) {
  if (bytes <= 0) return;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p), e = a + (uintptr_t)bytes;
  for (uintptr_t l = (a & ~uintptr_t(127)) + (uintptr_t)tid * 128; l < e; l += (uintptr_t)nt * 128) {
    const uintptr_t q = l < a ? a : l;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
  }
}

// rows [r0, r0 + nrows) of the columns [0, ncols) of a column-major block
__device__ __forceinline__ void prefetch_cols(const double* M, int64_t ld, int ncols, int r0, int nrows, int tid,
                                              int nt) {
  if (nrows <= 0) return;
  const int lpc = (nrows * 8 + 127) / 128 + 1;  // lines a column segment can touch
  for (int w = tid; w < ncols * lpc; w += nt) {
    const int t = w / lpc, j = w % lpc;
    const uintptr_t a = reinterpret_cast<uintptr_t>(M + (int64_t)t * ld + r0), e = a + (uintptr_t)nrows * 8;
    const uintptr_t l = (a & ~uintptr_t(127)) + (uintptr_t)j * 128;
    if (l < e) {
      const uintptr_t q = l < a ? a : l;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
    }
  }
}

struct ItemView {
  int nc, c1, col0, nJ;
  const double* L;    // column c0 of the front (leading dimension nJ)
  const int* rows;    // rows(J) of the item's supernode
  const double* X;    // inverse of the diagonal block (nc x nc, column-major)
  __device__ ItemView(const DevPlan& d, int q) {
    const int J = d.sq_sn[q], c0 = d.sq_c0[q];
    c1 = d.sq_c1[q];
    nc = c1 - c0;
    col0 = d.sn_first[J] + c0;
    nJ = d.sn_nrows[J];
    L = d.front + d.sn_off[J] + (int64_t)c0 * nJ;
    rows = d.sn_rows + d.sn_rp[J];
    X = d.dinv + d.dinv_off[q];
  }
};

// Warp items: every warp of a T_WARP task owns kWarpSmem doubles of the
// task's shared memory.  While it waits on its item's dependencies it stages
// X and the rows-below block there (when they fit, nc*(nc+R) doubles),
// together with the gather positions, b and x values it will need, so that
// after the wait only the freshly produced values are fetched.
constexpr int kWarpSmem = kTrsvSmem / kWarpsPerTask;

// Forward warp item (n_J - c0 <= 32): lane t holds column t's values.
// grouped: a member of a warp subtree -- no waits (its contributors are
// earlier members of the same CTA) and no signals (the subtree task sends
// them once all members are done).
__device__ __forceinline__ void warp_item_fwd(const DevPlan& d, const SolveSched& s, const TrsvCounters& C, int q,
                                              const double* b, double* x, double* ws, bool grouped = false) {
  const int lane = threadIdx.x & 31;
  const ItemView it(d, q);
  const int nc = it.nc, R = it.nJ - it.c1;
  const bool fit = nc * (nc + R) <= kWarpSmem;
  double* Xs = ws;            // X, column-major (nc x nc)
  double* Ls = ws + nc * nc;  // L21 as Ls[t*R + i]
  if (fit) {
    for (int idx = lane; idx < nc * nc; idx += 32) Xs[idx] = it.X[idx];
    for (int idx = lane; idx < nc * R; idx += 32) Ls[idx] = it.L[(int64_t)(idx / R) * it.nJ + it.c1 + idx % R];
  } else {
    prefetch_bytes(it.X, (int64_t)nc * nc * 8, lane, 32);
    prefetch_cols(it.L, it.nJ, nc, it.c1, R, lane, 32);
  }
  // lane t: b_t and the first four update positions of column t
  int g0 = 0, g1 = 0;
  double bcol = 0.0;
  int64_t gp[4] = {-1, -1, -1, -1};
  if (lane < nc) {
    const int col = it.col0 + lane;
    g0 = d.g_rp[col];
    g1 = d.g_rp[col + 1];
    bcol = __ldcg(&b[col]);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (g0 + j < g1) gp[j] = d.g_pos[g0 + j];
  }
  if (lane == 0 && !grouped) {
    wait_ge(&C.diag_cnt[q], s.fdiag_need[q], d);
    wait_ge(&C.child_done[q], s.nchild[q], d);
  }
  __syncwarp();
  double bt = 0.0;  // b'_t, lane t: its column's updates in list order
  if (lane < nc) {
    double uv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) uv[j] = gp[j] >= 0 ? __ldcg(&d.u[gp[j]]) : 0.0;
    double s0 = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) s0 = dadd(s0, uv[j]);
    for (int p = g0 + 4; p < g1; ++p) s0 = dadd(s0, __ldcg(&d.u[d.g_pos[p]]));
    bt = dsub(bcol, s0);
  }
  double acc = 0.0;  // x_r = sum_{k<=r} X[r][k] b'_k, lane r
  for (int k = 0; k < nc; ++k) {
    const double bk = __shfl_sync(0xffffffffu, bt, k);
    if (lane < nc && k <= lane) acc = fma(fit ? Xs[k * nc + lane] : it.X[(int64_t)k * nc + lane], bk, acc);
  }
  if (lane < nc) x[it.col0 + lane] = acc;
  double u = 0.0;  // u_i = L21(i,:) x_q, lane i
  for (int t = 0; t < nc; ++t) {
    const double xt = __shfl_sync(0xffffffffu, acc, t);
    if (lane < R) u = fma(fit ? Ls[t * R + lane] : it.L[(int64_t)t * it.nJ + it.c1 + lane], xt, u);
  }
  if (lane < R) d.u[d.sq_uoff[q] + lane] = u;
  if (grouped) return;
  __threadfence();
  __syncwarp();
  for (int ch = s.fch0[q]; ch < s.fch0[q] + s.nfch[q]; ++ch)
    for (int p = s.fct_rp[ch] + lane; p < s.fct_rp[ch + 1]; p += 32) atomicAdd(&C.diag_cnt[s.fct_item[p]], 1);
  if (lane == 0 && s.sq_parent[q] >= 0) atomicAdd(&C.child_done[s.sq_parent[q]], 1);
}

// Backward warp item: lane i holds x_R[i], then lane t column t.
__device__ __forceinline__ void warp_item_bwd(const DevPlan& d, const SolveSched& s, const TrsvCounters& C, int q,
                                              double* x, double* ws, bool grouped = false) {
  const int lane = threadIdx.x & 31;
  const ItemView it(d, q);
  const int nc = it.nc, R = it.nJ - it.c1;
  const bool fit = nc * (nc + R) <= kWarpSmem;
  double* Xs = ws;
  double* Ls = ws + nc * nc;
  if (fit) {
    for (int idx = lane; idx < nc * nc; idx += 32) Xs[idx] = it.X[idx];
    for (int idx = lane; idx < nc * R; idx += 32) Ls[idx] = it.L[(int64_t)(idx / R) * it.nJ + it.c1 + idx % R];
  } else {
    prefetch_bytes(it.X, (int64_t)nc * nc * 8, lane, 32);
    prefetch_cols(it.L, it.nJ, nc, it.c1, R, lane, 32);
  }
  const int ridx = lane < R ? it.rows[it.c1 + lane] : 0;
  const double xown = lane < nc ? __ldcg(&x[it.col0 + lane]) : 0.0;  // x_q from the forward solve
  if (s.nch[q] > 0 && lane == 0 && !grouped) {
    const int ch = s.ch0[q];
    wait_ge(&C.bg_cnt[ch], s.ct_rp[ch + 1] - s.ct_rp[ch], d);
  }
  __syncwarp();
  const double xr = lane < R ? __ldcg(&x[ridx]) : 0.0;
  double acc = 0.0;  // L21(:,t)^T x_R, lane t
  for (int i = 0; i < R; ++i) {
    const double xi = __shfl_sync(0xffffffffu, xr, i);
    if (lane < nc) acc = fma(fit ? Ls[lane * R + i] : it.L[(int64_t)lane * it.nJ + it.c1 + i], xi, acc);
  }
  const double ys = lane < nc ? dsub(xown, acc) : 0.0;
  double xo = 0.0;  // x_t = sum_{k>=t} X[k][t] y'_k, lane t
  for (int k = 0; k < nc; ++k) {
    const double yk = __shfl_sync(0xffffffffu, ys, k);
    if (lane < nc && k >= lane) xo = fma(fit ? Xs[lane * nc + k] : it.X[(int64_t)lane * nc + k], yk, xo);
  }
  if (lane < nc) x[it.col0 + lane] = xo;
  if (grouped) return;
  __threadfence();
  __syncwarp();
  for (int p = s.ic_rp[q] + lane; p < s.ic_rp[q + 1]; p += 32) atomicAdd(&C.bg_cnt[s.ic_chunk[p]], 1);
}

// One forward task k of the plan (d, s); sm, flag and g_lo are the CTA's
// shared scratch.
__device__ __forceinline__ void fwd_task(const DevPlan& d, const SolveSched& s, const TrsvCounters& C, int k,
                                         const double* __restrict__ b, double* x, double* sm, int* flag, int* g_lo) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  trace_mark(d, k, 0);
  trace_mark(d, k, 3);
  const int kind = s.tf_kind[k], q = s.tf_item[k], arg = s.tf_arg[k];
  if (kind == T_WARP) {
    const int g0 = s.wg_rp[arg], gn = s.wg_rp[arg + 1] - g0;
    if (warp < gn) warp_item_fwd(d, s, C, s.wg_item[g0 + warp], b, x, sm + warp * kWarpSmem);
    trace_mark(d, k, 2);
    return;
  }
  if (kind == T_WSUB) {
    // a warp subtree, leaves first: the members of one level on the warps,
    // a barrier between levels (a member's contributors are earlier
    // members), then every member's signals to the items above
    const int g0 = s.sg_rp[arg], g1 = s.sg_rp[arg + 1];
    for (int i = g0; i < g1;) {
      int j = i;
      while (j < g1 && s.sg_lvl[j] == s.sg_lvl[i]) ++j;
      for (int t = i + warp; t < j; t += kWarpsPerTask) {
        warp_item_fwd(d, s, C, s.sg_item[t], b, x, sm + warp * kWarpSmem, true);
        __syncwarp();  // the warp's staging area is reused by its next member
      }
      __syncthreads();
      i = j;
    }
    __threadfence();
    __syncthreads();
    for (int t = g0 + warp; t < g1; t += kWarpsPerTask) {
      const int qq = s.sg_item[t];
      for (int ch = s.fch0[qq]; ch < s.fch0[qq] + s.nfch[qq]; ++ch)
        for (int p = s.fct_rp[ch] + lane; p < s.fct_rp[ch + 1]; p += 32) atomicAdd(&C.diag_cnt[s.fct_item[p]], 1);
      if (lane == 0 && s.sq_parent[qq] >= 0) atomicAdd(&C.child_done[s.sq_parent[qq]], 1);
    }
    trace_mark(d, k, 2);
    return;
  }
  const ItemView it(d, q);
  const int nc = it.nc, c1 = it.c1, col0 = it.col0, nJ = it.nJ;
  if (kind == T_FUSED || kind == T_HEAD) {
    // everything that does not depend on this solve's updates is staged
    // while the task waits: X in shared memory (column stride nc + 1), a
    // fused item's rows below (column stride R + 1) when they fit, b, each
    // column's first gather entry, the gather lists (update arena positions)
    // when they fit the rest of the shared memory, and the children's rows
    // in these columns (factor data, into L2)
    double* xs = sm;
    double* xq = sm + kPiece;
    double* Ls = sm + 2 * kPiece;
    const int ldx = nc + 1, R = nJ - c1;
    double* Lb = Ls + nc * ldx;
    const bool lfit = kind == T_FUSED && 2 * kPiece + nc * ldx + nc * (R + 1) <= kTrsvSmem;
    int64_t* gpos = reinterpret_cast<int64_t*>(lfit ? Lb + nc * (R + 1) : Lb);
    const int g0 = d.g_rp[col0], gE = d.g_rp[col0 + nc] - g0;
    const bool staged = gE <= kTrsvSmem - (int)(reinterpret_cast<double*>(gpos) - sm);
    if (lfit) stage_block(it.L + c1, nJ, R, nc, Lb, R + 1);
    else if (kind == T_FUSED) prefetch_cols(it.L, nJ, nc, c1, R, threadIdx.x, kBlock);
    for (int idx = threadIdx.x; idx < nc * nc; idx += kBlock) Ls[(idx / nc) * ldx + idx % nc] = it.X[idx];
    if (staged) {
      for (int e = threadIdx.x; e < gE; e += kBlock) gpos[e] = d.g_pos[g0 + e];
    } else {
      prefetch_bytes(d.g_pos + g0, (int64_t)gE * 8, threadIdx.x, kBlock);
    }
    if (threadIdx.x < nc) xs[threadIdx.x] = __ldcg(&b[col0 + threadIdx.x]);
    if (threadIdx.x <= nc) g_lo[threadIdx.x] = d.g_rp[col0 + threadIdx.x] - g0;
    for (int ce = s.cd_rp[col0] + (threadIdx.x >> 3); ce < s.cd_rp[col0 + nc]; ce += kBlock / 8) {
      const double* Lc = d.front + s.cd_L[ce];
      const int64_t ld = s.cd_ld[ce];
      for (int tt = threadIdx.x & 7; tt < s.cd_nc[ce]; tt += 8)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(Lc + tt * ld));
    }
    if (threadIdx.x == 0) wait_ge(&C.diag_cnt[q], s.fdiag_need[q], d);
    cta_wait_ge(&C.child_done[q], s.nchild[q], d);
    trace_mark(d, k, 1);
    {
      // b'_t = b_t - (the column's updates) - (its children's products from
      // their fresh x): every column at once, tpc threads per column, the
      // partial sums combined in a fixed order
      const int lg = nc <= 32 ? 3 : 2, tpc = 1 << lg;
      const int t = threadIdx.x >> lg, j = threadIdx.x & (tpc - 1);
      double a0 = 0.0, a1 = 0.0;
      if (t < nc) {
        const int e1 = g_lo[t + 1];
        int e = g_lo[t] + j;
        for (; e + tpc < e1; e += 2 * tpc) {
          const int64_t p0 = staged ? gpos[e] : d.g_pos[g0 + e];
          const int64_t p1 = staged ? gpos[e + tpc] : d.g_pos[g0 + e + tpc];
          a0 = dadd(a0, __ldcg(&d.u[p0]));
          a1 = dadd(a1, __ldcg(&d.u[p1]));
        }
        if (e < e1) a0 = dadd(a0, __ldcg(&d.u[staged ? gpos[e] : d.g_pos[g0 + e]]));
        for (int ce = s.cd_rp[col0 + t]; ce < s.cd_rp[col0 + t + 1]; ++ce) {
          const double* Lc = d.front + s.cd_L[ce];
          const int ld = s.cd_ld[ce], ncc = s.cd_nc[ce];
          const double* xc = x + s.cd_x[ce];
          for (int tt = j; tt < ncc; tt += tpc) a1 = fma(Lc[(int64_t)tt * ld], __ldcg(&xc[tt]), a1);
        }
      }
      double v = dadd(a0, a1);
      if (lg == 3) v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 4));
      v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 2));
      v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 1));
      if (j == 0 && t < nc) xs[t] = dsub(xs[t], v);
    }
    __syncthreads();
    {  // x_q = X_q b'_q: four threads per row
      const int row = threadIdx.x >> 2, part = threadIdx.x & 3;
      double acc = 0.0;
      if (row < nc)
        for (int kk = part; kk <= row; kk += 4) acc = fma(Ls[kk * ldx + row], xs[kk], acc);
      acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 1));
      acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 2));
      if (row < nc && part == 0) {
        x[col0 + row] = acc;
        xq[row] = acc;
      }
    }
    if (kind == T_HEAD) {
      signal_count(&C.inv_done[q]);
    } else {
      __syncthreads();
      // u_q = L21 x_q for the rows below the parent's: one thread per row,
      // two or four (columns split, then summed in order) when the rows are
      // few, for shorter load chains
      const int r0 = s.sq_rpar[q], nrow = R - r0;
      const int lr = nrow <= kBlock / 4 ? 2 : nrow <= kBlock / 2 ? 1 : 0;
      const int row = threadIdx.x >> lr, part = threadIdx.x & ((1 << lr) - 1);
      double acc = 0.0;
      if (row < nrow) {
        if (lfit) {
          const double* Lr = Lb + r0 + row;
#pragma unroll 8
          for (int t = part; t < nc; t += 1 << lr) acc = fma(Lr[t * (R + 1)], xq[t], acc);
        } else {
          const double* Lr = it.L + c1 + r0 + row;
#pragma unroll 8
          for (int t = part; t < nc; t += 1 << lr) acc = fma(Lr[(int64_t)t * nJ], xq[t], acc);
        }
      }
      if (lr == 2) acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 2));
      if (lr >= 1) acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 1));
      if (row < nrow && part == 0) d.u[d.sq_uoff[q] + r0 + row] = acc;
      if (s.nfch[q] > 0) signal_chunk_items(s.fct_rp, s.fct_item, s.fch0[q], C.diag_cnt);
      else __threadfence();
    }
    // x_q is complete: the parent may take its products
    __syncthreads();
    if (threadIdx.x == 0 && s.sq_parent[q] >= 0) atomicAdd(&C.child_done[s.sq_parent[q]], 1);
  } else if (kind == T_GATHER) {
    // b' of a chunk of kColChunk columns, eight threads per column, all
    // columns at once.  Staged while waiting: each column's first entry,
    // the update positions (when they fit) and b.
    static_assert(kColChunk * 8 == kBlock, "eight threads per gathered column");
    const int cb = col0 + arg, ncol = min(nc - arg, kColChunk);
    const int gb = d.g_rp[cb], gE = d.g_rp[cb + ncol] - gb;
    constexpr int kGatherPos = kTrsvSmem - kColChunk;  // int64 positions after the b values
    double* bs = sm;
    int64_t* gpos = reinterpret_cast<int64_t*>(sm + kColChunk);
    const bool staged = gE <= kGatherPos;
    if (staged) {
      for (int e = threadIdx.x; e < gE; e += kBlock) gpos[e] = d.g_pos[gb + e];
    } else {
      prefetch_bytes(d.g_pos + gb, (int64_t)gE * 8, threadIdx.x, kBlock);
    }
    if (threadIdx.x <= ncol) g_lo[threadIdx.x] = d.g_rp[cb + threadIdx.x] - gb;
    if (threadIdx.x < ncol) bs[threadIdx.x] = __ldcg(&b[cb + threadIdx.x]);
    if (threadIdx.x == 0) wait_ge(&C.diag_cnt[q], s.fdiag_need[q], d);
    cta_wait_ge(&C.child_done[q], s.nchild[q], d);
    trace_mark(d, k, 1);
    const int t = threadIdx.x >> 3, j = threadIdx.x & 7;
    double a0 = 0.0, a1 = 0.0;
    if (t < ncol) {
      const int e1 = g_lo[t + 1];
      int e = g_lo[t] + j;
      for (; e + 8 < e1; e += 16) {
        const int64_t p0 = staged ? gpos[e] : d.g_pos[gb + e];
        const int64_t p1 = staged ? gpos[e + 8] : d.g_pos[gb + e + 8];
        a0 = dadd(a0, __ldcg(&d.u[p0]));
        a1 = dadd(a1, __ldcg(&d.u[p1]));
      }
      if (e < e1) a0 = dadd(a0, __ldcg(&d.u[staged ? gpos[e] : d.g_pos[gb + e]]));
      // children's products for this column, from their fresh x
      for (int ce = s.cd_rp[cb + t]; ce < s.cd_rp[cb + t + 1]; ++ce) {
        const double* Lc = d.front + s.cd_L[ce];
        const int ld = s.cd_ld[ce], ncc = s.cd_nc[ce];
        const double* xc = x + s.cd_x[ce];
        for (int tt = j; tt < ncc; tt += 8) a1 = fma(Lc[(int64_t)tt * ld], __ldcg(&xc[tt]), a1);
      }
    }
    // the eight partial sums of a column in a fixed order
    double v = dadd(a0, a1);
    v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 4));
    v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 2));
    v = dadd(v, __shfl_xor_sync(0xffffffffu, v, 1));
    if (j == 0 && t < ncol) d.sv[cb + t] = dsub(bs[t], v);
    signal_count(&C.g_done[q]);
  } else if (kind == T_INV) {
    const int RT = s.rows_x[q];
    const int b = arg & ((1 << kUnitShift) - 1), unit = arg >> kUnitShift;
    const int r0 = b * RT, nr = min(RT, nc - r0);
    const double* P = d.xpanel + d.xp_off[q] + xpanel_fwd(RT, nc, b);
    {
      const int K = min(nc, r0 + RT), k0 = unit * s.unit_cols;
      prefetch_bytes(P + (int64_t)k0 * RT, (int64_t)min(s.unit_cols, K - k0) * RT * 8, threadIdx.x, kBlock);
    }
    cta_wait_ge(&C.g_done[q], ceil_div(nc, kColChunk), d);
    trace_mark(d, k, 1);
    double* slot = d.ppart + s.ppoff[q] + (int64_t)b * ceil_div(nc, s.unit_cols) * RT;
    // an item without rows below keeps a copy of its x for the backward pass
    double* keep = s.nch[q] == 0 ? d.sv2 + col0 + r0 : nullptr;
    if (panel_unit(P, RT, nr, min(nc, r0 + RT), unit, s.unit_cols, d.sv + col0, x + col0 + r0, slot, &C.panel_f[s.pcoff[q] + b],
                   sm, flag, keep)) {
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) {
        // the CTA completing the last panel tells the parent that x_q is complete
        const bool all = atomicAdd(&C.inv_done[q], 1) == ceil_div(nc, RT) - 1;
        if (all && s.sq_parent[q] >= 0) {
          __threadfence();
          atomicAdd(&C.child_done[s.sq_parent[q]], 1);
        }
      }
    }
  } else {  // T_L21
    const int RT = s.rows_x[q];
    const int ch = arg & ((1 << kUnitShift) - 1), unit = arg >> kUnitShift;
    const int row0 = s.fch_row0[ch], nr = s.fch_rows[ch];
    const int64_t slot0 = s.fch_slot[ch];
    if (slot0 >= 0) {
      // a wide item's chunk in column units: this unit's partial sums go to
      // the chunk's slot; the last unit adds them in unit order
      const int seg = s.unit_cols, nunits = ceil_div(nc, seg), k0 = unit * seg, kn = min(seg, nc - k0);
      const int64_t lf = s.l21f_off[q];
      // panelized item: the chunk's packed block [col][16]; otherwise the front
      const double* Lk = lf >= 0 ? d.l21f + lf + (int64_t)row0 * nc + (int64_t)k0 * 16 : it.L + (int64_t)k0 * nJ;
      const int64_t ldk = lf >= 0 ? 16 : nJ;
      const int rk = lf >= 0 ? 0 : c1 + row0;
      if (lf >= 0) prefetch_bytes(Lk, (int64_t)kn * 16 * 8, threadIdx.x, kBlock);
      else prefetch_cols(Lk, nJ, kn, c1 + row0, nr, threadIdx.x, kBlock);
      cta_wait_ge(&C.inv_done[q], inv_tasks(s, q, nc), d);
      trace_mark(d, k, 1);
      double* slot = s.fslot + slot0;
      rows_times_vec<kUnitLoads>(Lk, ldk, rk, nr, RT, kn, x + col0 + k0, slot + (int64_t)unit * RT, sm);
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) *flag = atomicAdd(&C.fch_cnt[ch], 1) == nunits - 1;
      __syncthreads();
      if (*flag) {
        __threadfence();
        if (threadIdx.x < nr) {
          double acc = __ldcg(&slot[threadIdx.x]);
          for (int u = 1; u < nunits; ++u) acc = dadd(acc, __ldcg(&slot[(int64_t)u * RT + threadIdx.x]));
          d.u[d.sq_uoff[q] + row0 + threadIdx.x] = acc;
        }
        signal_chunk_items(s.fct_rp, s.fct_item, ch, C.diag_cnt);
      }
      trace_mark(d, k, 2);
      return;
    }
    // a block that fits shared memory is staged there while waiting
    const bool fit = nr * nc + nc + kBlock <= kTrsvSmem;
    double* Ls = sm;
    double* xv = sm + nr * nc;
    if (fit) stage_block(it.L + c1 + row0, nJ, nr, nc, Ls, nr);
    else prefetch_cols(it.L, nJ, nc, c1 + row0, nr, threadIdx.x, kBlock);
    cta_wait_ge(&C.inv_done[q], inv_tasks(s, q, nc), d);
    trace_mark(d, k, 1);
    if (fit) {
      for (int t = threadIdx.x; t < nc; t += kBlock) xv[t] = __ldcg(&x[col0 + t]);
      __syncthreads();
      block_rows_times_vec(Ls, nr, nc, xv, xv + nc, d.u + d.sq_uoff[q] + row0);
    } else {
      rows_times_vec(it.L, nJ, c1 + row0, nr, RT, nc, x + col0, d.u + d.sq_uoff[q] + row0, sm);
    }
    signal_chunk_items(s.fct_rp, s.fct_item, ch, C.diag_cnt);
  }
  trace_mark(d, k, 2);
}

__global__ void __launch_bounds__(kBlock, HYKKT_TRSV_MIN_BLOCKS) k_trsv_fwd(DevPlan d, SolveSched s, const double* __restrict__ b, double* x,
                                                     int use_stop) {
  if (use_stop && d.sc->stop) return;
  __shared__ double sm[kTrsvSmem];
  __shared__ int task;
  __shared__ int flag;
  __shared__ int g_lo[kPiece + 1];  // staged gather: each column's first entry
  const TrsvCounters C(s);
  C.clear_bwd(s);  // for the backward solve that follows
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) task = atomicAdd(C.head_f, 1);
    __syncthreads();
    const int k = task;
    if (k >= s.ntasks_f) return;
    fwd_task(d, s, C, k, b, x, sm, &flag, g_lo);
  }
}

// x_q = X_q^T y'_q for an item of at most 64 columns: X staged in shared
// memory at column stride ldx (row t of X^T is column t of X), four threads
// per row, their partial sums combined in a fixed order.
__device__ __forceinline__ void apply_xt(const double* Ls, int ldx, int nc, const double* ys, double* xq) {
  const int row = threadIdx.x >> 2, part = threadIdx.x & 3;
  double acc = 0.0;
  if (row < nc)
    for (int kk = row + part; kk < nc; kk += 4) acc = fma(Ls[row * ldx + kk], ys[kk], acc);
  acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 1));
  acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, 2));
  if (row < nc && part == 0) xq[row] = acc;
}

// Backward tail of head item q, run by the task that completed its last
// L21^T chunk (every chunk's partial products are written and fenced):
// y'_t = x_t - (sum over the item's chunks, kBlock/64 groups of chunks per
// column, each in chunk order, then the groups in order), x_q = X_q^T y',
// then the item is done.
__device__ void head_tail(const DevPlan& d, const SolveSched& s, const ItemView& it, int q, double* x, double* sm) {
  const int nc = it.nc, col0 = it.col0;
  double* ys = sm;
  double* red = ys + kPiece + kSmallItemRows;  // kBlock doubles
  double* Ls = red + kBlock;                   // X, column stride nc + 1
  const int ldx = nc + 1;
  __syncthreads();  // the caller's shared-memory use is over
  for (int idx = threadIdx.x; idx < nc * nc; idx += kBlock) Ls[(idx / nc) * ldx + idx % nc] = it.X[idx];
  constexpr int G = kBlock / kPiece;
  const int tl = threadIdx.x % kPiece, g = threadIdx.x / kPiece;
  const int cq = s.ch0[q], ncq = s.nch[q];
  const double acc =
      tl < nc && ncq > 0 ? strided_chunk_sum(d.part, s.ch_poff[cq] + tl, nc, cq, cq + g, cq + ncq, G) : 0.0;
  red[threadIdx.x] = acc;
  __syncthreads();
  if (g == 0 && tl < nc) {
    double tot = red[tl];
    for (int j = 1; j < G; ++j) tot = dadd(tot, red[j * kPiece + tl]);
    ys[tl] = dsub(__ldcg(&x[col0 + tl]), tot);
  }
  __syncthreads();
  apply_xt(Ls, ldx, nc, ys, x + col0);
  const TrsvCounters C(s);
  signal_item_done(s, q, C.bg_cnt);
}

// One backward task k of the plan (d, s); sm, flag and ridx are the CTA's
// shared scratch.
__device__ __forceinline__ void bwd_task(const DevPlan& d, const SolveSched& s, const TrsvCounters& C, int k, double* x,
                                         double* sm, int* flag, int* ridx) {
  const int warp = threadIdx.x >> 5;
  const int kt = s.ntasks_f + k;  // timeline slot
  trace_mark(d, kt, 0);
  trace_mark(d, kt, 3);
  const int kind = s.tb_kind[k], q = s.tb_item[k], arg = s.tb_arg[k];
  if (kind == T_WARP) {
    const int g0 = s.wg_rp[arg], gn = s.wg_rp[arg + 1] - g0;
    if (warp < gn) warp_item_bwd(d, s, C, s.wg_item[g0 + warp], x, sm + warp * kWarpSmem);
    trace_mark(d, kt, 2);
    return;
  }
  if (kind == T_WSUB) {
    // a warp subtree, root first: the root's rows below cover every row of
    // the members outside the subtree, so one wait on the root's chunk
    // opens the whole subtree; then the levels top-down with barriers
    const int g0 = s.sg_rp[arg], g1 = s.sg_rp[arg + 1];
    if (s.nch[q] > 0) {
      const int ch = s.ch0[q];
      cta_wait_ge(&C.bg_cnt[ch], s.ct_rp[ch + 1] - s.ct_rp[ch], d);
    }
    trace_mark(d, kt, 1);
    for (int i = g1; i > g0;) {
      int j = i;
      while (j > g0 && s.sg_lvl[j - 1] == s.sg_lvl[i - 1]) --j;
      for (int t = j + warp; t < i; t += kWarpsPerTask) {
        warp_item_bwd(d, s, C, s.sg_item[t], x, sm + warp * kWarpSmem, true);
        __syncwarp();
      }
      __syncthreads();
      i = j;
    }
    trace_mark(d, kt, 2);
    return;
  }
  const ItemView it(d, q);
  const int nc = it.nc, c1 = it.c1, col0 = it.col0, nJ = it.nJ;
  if (kind == T_TAIL) {
    // a head item's tail runs in its last L21^T chunk task (head_tail);
    // only an item without chunks is finished here
    trace_mark(d, kt, 1);
    if (s.nch[q] == 0) head_tail(d, s, it, q, x, sm);
  } else if (kind == T_FUSED) {
    double* ys = sm;
    double* xR = ys + kPiece;           // the ancestors' values x_R (R <= 256 - nc)
    double* red = xR + kSmallItemRows;  // kBlock doubles
    double* Ls = red + kBlock;          // X, column stride nc + 1
    const int ldx = nc + 1;
    // staged while waiting: X in shared memory, the rows below (column stride
    // R + 1, when they fit), their row indices and x_q from the forward solve
    for (int idx = threadIdx.x; idx < nc * nc; idx += kBlock) Ls[(idx / nc) * ldx + idx % nc] = it.X[idx];
    const int R = nJ - c1;
    double* Lb = Ls + nc * ldx;
    const bool lfit = kPiece + kSmallItemRows + kBlock + nc * ldx + nc * (R + 1) <= kTrsvSmem;
    if (lfit) stage_block(it.L + c1, nJ, R, nc, Lb, R + 1);
    else prefetch_cols(it.L, nJ, nc, c1, R, threadIdx.x, kBlock);
    for (int i = threadIdx.x; i < R; i += kBlock) ridx[i] = it.rows[c1 + i];
    if (threadIdx.x < nc) ys[threadIdx.x] = __ldcg(&x[col0 + threadIdx.x]);
    if (s.nch[q] > 0) {
      const int ch = s.ch0[q];
      cta_wait_ge(&C.bg_cnt[ch], s.ct_rp[ch + 1] - s.ct_rp[ch], d);
    } else {
      __syncthreads();
    }
    trace_mark(d, kt, 1);
    for (int i = threadIdx.x; i < R; i += kBlock) xR[i] = __ldcg(&x[ridx[i]]);
    __syncthreads();
    // y'_t = x_t - L21(:,t)^T x_R
    if (lfit) column_dots(Lb, R + 1, nc, R, xR, red, [&](int t, double v) { ys[t] = dsub(ys[t], v); });
    else column_dots(it.L + c1, nJ, nc, R, xR, red, [&](int t, double v) { ys[t] = dsub(ys[t], v); });
    __syncthreads();
    apply_xt(Ls, ldx, nc, ys, x + col0);
    signal_item_done(s, q, C.bg_cnt);
  } else if (kind == T_L21T && s.l21b_off[q] >= 0) {
    // panelized item: columns [16 b, 16 b + 16) over the chunk's rows, from
    // the packed panel [row][16]
    const int ch = arg & ((1 << kUnitShift) - 1), b = arg >> kUnitShift;
    const int r0 = s.ch_row0[ch], nr = s.ch_rows[ch], R = nJ - c1;
    const double* P = d.l21b + s.l21b_off[q] + (int64_t)b * R * 16 + (int64_t)r0 * 16;
    double* xR = sm;                                  // nr <= unit_cols doubles
    int* rix = reinterpret_cast<int*>(sm + kMaxUnitCols);  // nr row indices
    double* red = sm + kMaxUnitCols + kMaxUnitCols / 2;
    prefetch_bytes(P, (int64_t)nr * 16 * 8, threadIdx.x, kBlock);
    for (int i = threadIdx.x; i < nr; i += kBlock) rix[i] = it.rows[c1 + r0 + i];
    cta_wait_ge(&C.bg_cnt[ch], s.ct_rp[ch + 1] - s.ct_rp[ch], d);
    trace_mark(d, kt, 1);
    for (int i = threadIdx.x; i < nr; i += kBlock) xR[i] = __ldcg(&x[rix[i]]);
    __syncthreads();
    {
      // thread (column tt, part p): rows i = p, p + 16, ...; eight loads in flight
      const int tt = threadIdx.x & 15, p = threadIdx.x >> 4;
      double a[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] = 0.0;
      int i = p;
      for (; i + 7 * 16 < nr; i += 8 * 16) {
        double m[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) m[j] = P[(int64_t)(i + 16 * j) * 16 + tt];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(m[j], xR[i + 16 * j], a[j]);
      }
      for (; i < nr; i += 16) a[0] = fma(P[(int64_t)i * 16 + tt], xR[i], a[0]);
      red[threadIdx.x] = dadd(dadd(dadd(a[0], a[1]), dadd(a[2], a[3])), dadd(dadd(a[4], a[5]), dadd(a[6], a[7])));
      __syncthreads();
      const int t = b * 16 + tt;
      if (p == 0 && t < nc) {
        double sum = red[tt];
        for (int j = 1; j < 16; ++j) sum = dadd(sum, red[j * 16 + tt]);
        d.part[s.ch_poff[ch] + t] = sum;
      }
    }
    signal_count(&C.bd_cnt[q]);
  } else if (kind == T_L21T) {
    const int row0 = c1 + s.ch_row0[arg], nr = s.ch_rows[arg];
    double* part = d.part + s.ch_poff[arg];
    // a block that fits shared memory (padded columns: conflict-free column
    // dots) is staged there with its row indices while waiting
    const bool fit = (nr + 1) * nc + nr + kBlock <= kTrsvSmem;
    if (fit) {
      stage_block(it.L + row0, nJ, nr, nc, sm, nr + 1);
      for (int i = threadIdx.x; i < nr; i += kBlock) ridx[i] = it.rows[row0 + i];
    } else {
      prefetch_cols(it.L, nJ, nc, row0, nr, threadIdx.x, kBlock);
      prefetch_bytes(it.rows + row0, (int64_t)nr * 4, threadIdx.x, kBlock);
    }
    cta_wait_ge(&C.bg_cnt[arg], s.ct_rp[arg + 1] - s.ct_rp[arg], d);
    trace_mark(d, kt, 1);
    if (fit) {
      double* xR = sm + (nr + 1) * nc;
      for (int i = threadIdx.x; i < nr; i += kBlock) xR[i] = __ldcg(&x[ridx[i]]);
      __syncthreads();
      column_dots(sm, nr + 1, nc, nr, xR, xR + nr, [&](int t, double v) { part[t] = v; });
    } else {
      double* xR = sm;
      double* red = sm + kSmallItemRows;
      double* tile = red + kBlock;
      for (int i = threadIdx.x; i < nr; i += kBlock) xR[i] = __ldcg(&x[it.rows[row0 + i]]);
      __syncthreads();
      // wide items: shared-memory tiles (coalesced); narrow ones: rows split over the threads
      if (nc >= 64) column_dots_tiled(it.L + row0, nJ, nc, nr, xR, tile, red, [&](int t, double v) { part[t] = v; });
      else column_dots(it.L + row0, nJ, nc, nr, xR, red, [&](int t, double v) { part[t] = v; });
    }
    if (s.mode[q] == ITEM_HEAD) {
      // the chunk that completes a head item's partials finishes the item
      // itself: one dependency round trip less per level of head items
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) *flag = atomicAdd(&C.bd_cnt[q], 1) == s.nch[q] - 1;
      __syncthreads();
      if (*flag) {
        __threadfence();
        head_tail(d, s, it, q, x, sm);
      }
    } else {
      signal_count(&C.bd_cnt[q]);
    }
  } else if (kind == T_REDUCE) {
    cta_wait_ge(&C.bd_cnt[q], s.bd_need[q], d);
    trace_mark(d, kt, 1);
    // kBlock/kColChunk groups of chunks per column, each summed in chunk
    // order, then the groups in order
    static_assert(kBlock % kColChunk == 0, "column chunk must divide the CTA");
    constexpr int G = kBlock / kColChunk;
    double* red = sm;
    const int tl = threadIdx.x % kColChunk, g = threadIdx.x / kColChunk;
    const int t = arg + tl;
    const bool col_ok = t < min(nc, arg + kColChunk);
    // an item's chunk partials are consecutive, nc doubles apart
    const int cq = s.ch0[q], ncq = s.nch[q];
    const double acc = col_ok && ncq > 0 ? strided_chunk_sum(d.part, s.ch_poff[cq] + t, nc, cq, cq + g, cq + ncq, G) : 0.0;
    red[threadIdx.x] = acc;
    __syncthreads();
    if (g == 0 && col_ok) {
      double tot = red[tl];
      for (int j = 1; j < G; ++j) tot = dadd(tot, red[j * kColChunk + tl]);
      d.sv[col0 + t] = dsub(__ldcg(&x[col0 + t]), tot);
    }
    signal_count(&C.red_done[q]);
  } else {  // T_INVT
    const int RT = s.rows_x[q];
    const int b = arg & ((1 << kUnitShift) - 1), unit = arg >> kUnitShift;
    const int r0 = b * RT, nr = min(RT, nc - r0);
    const double* P = d.xpanel + d.xp_off[q] + xpanel_bwd(RT, nc, b);
    {
      const int K = nc - r0, k0 = unit * s.unit_cols;
      prefetch_bytes(P + (int64_t)k0 * RT, (int64_t)min(s.unit_cols, K - k0) * RT * 8, threadIdx.x, kBlock);
    }
    // an item without rows below has y' = x, copied by the forward pass (no
    // REDUCE tasks: nothing to wait for); the others wait for their y'
    const bool own = s.nch[q] == 0;
    cta_wait_ge(&C.red_done[q], own ? 0 : ceil_div(nc, kColChunk), d);
    trace_mark(d, kt, 1);
    double* slot = d.ppart + s.ppoff[q] + (int64_t)b * ceil_div(nc, s.unit_cols) * RT;
    if (panel_unit(P, RT, nr, nc - r0, unit, s.unit_cols, (own ? d.sv2 : d.sv) + col0 + r0, x + col0 + r0, slot,
                   &C.panel_b[s.pcoff[q] + b], sm, flag)) {
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) *flag = atomicAdd(&C.invt_done[q], 1) == ceil_div(nc, RT) - 1;
      __syncthreads();
      if (*flag) signal_item_done(s, q, C.bg_cnt);
    }
  }
  trace_mark(d, kt, 2);
}

__global__ void __launch_bounds__(kBlock, HYKKT_TRSV_MIN_BLOCKS) k_trsv_bwd(DevPlan d, SolveSched s, double* x, int use_stop) {
  if (use_stop && d.sc->stop) return;
  __shared__ double sm[kTrsvSmem];
  __shared__ int task;
  __shared__ int flag;
  __shared__ int ridx[kSmallItemRows];  // staged row indices below a fused item
  const TrsvCounters C(s);
  C.clear_fwd(s);  // for the next forward solve
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) task = atomicAdd(C.head_b, 1);
    __syncthreads();
    const int k = task;
    if (k >= s.ntasks_b) return;
    bwd_task(d, s, C, k, x, sm, &flag, ridx);
  }
}

#ifdef HYKKT_MEASURE
// Measurement builds only (measured slower than concurrent plans on their
// own streams, kept to repeat that comparison).
// Triangular solves of several plans of one pattern in one launch.  The
// plans' task queues are interleaved (task k of every plan before task k+1
// of any), so every task's dependencies -- earlier tasks of its own plan --
// are claimed before it, as in the single-plan kernels.  Plans whose CG has
// stopped (use_stop) skip their tasks.  Each plan's counter blocks must be
// clear at launch.
struct MultiTrsv {
  const DevPlan* d;        // per plan, device memory
  const SolveSched* s;     // per plan, device memory
  const double* const* b;  // per plan right-hand side (forward)
  double* const* x;        // per plan solution
  int nplan;
  int* head;               // shared claim counters: [forward, backward]
  int use_stop;
};

__global__ void __launch_bounds__(kBlock, 4) k_trsv_fwd_multi(MultiTrsv m) {
  __shared__ double sm[kTrsvSmem];
  __shared__ int task;
  __shared__ int flag;
  __shared__ int g_lo[kPiece + 1];
  const int ntasks = m.s[0].ntasks_f;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) task = atomicAdd(&m.head[0], 1);
    __syncthreads();
    const int t = task, p = t % m.nplan, k = t / m.nplan;
    if (k >= ntasks) return;
    const DevPlan& d = m.d[p];
    if (m.use_stop && d.sc->stop) continue;
    const SolveSched& s = m.s[p];
    const TrsvCounters C(s);
    fwd_task(d, s, C, k, m.b[p], m.x[p], sm, &flag, g_lo);
  }
}

__global__ void __launch_bounds__(kBlock, 4) k_trsv_bwd_multi(MultiTrsv m) {
  __shared__ double sm[kTrsvSmem];
  __shared__ int task;
  __shared__ int flag;
  __shared__ int ridx[kSmallItemRows];
  const int ntasks = m.s[0].ntasks_b;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) task = atomicAdd(&m.head[1], 1);
    __syncthreads();
    const int t = task, p = t % m.nplan, k = t / m.nplan;
    if (k >= ntasks) return;
    const DevPlan& d = m.d[p];
    if (m.use_stop && d.sc->stop) continue;
    const SolveSched& s = m.s[p];
    const TrsvCounters C(s);
    bwd_task(d, s, C, k, m.x[p], sm, &flag, ridx);
  }
}
#endif  // HYKKT_MEASURE

// ---------------------------------------------------------------------------
// Step a9: Schur-complement CG, scalars on the device
// (SchurComplementConjugateGradient::solve, SchurCG.cpp:102-194).
// ---------------------------------------------------------------------------
// sum_p vals[vidx(p)] x[ci[p]] over p in [p0, p1), in order: the index and
// value loads of four entries are issued before their products (the loads
// of a row do not wait on one another; the sum keeps the entry order)
template <class VIdx>
__device__ __forceinline__ double sparse_row_dot(int p0, int p1, const double* __restrict__ vals, VIdx vidx,
                                                 const int* __restrict__ ci, const double* __restrict__ x) {
  double acc = 0.0;
  int p = p0;
  for (; p + 4 <= p1; p += 4) {
    int c[4], s[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      c[j] = ci[p + j];
      s[j] = vidx(p + j);
    }
    double a[4], b[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      a[j] = vals[s[j]];
      b[j] = x[c[j]];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) acc = fma(a[j], b[j], acc);
  }
  for (; p < p1; ++p) acc = fma(vals[vidx(p)], x[ci[p]], acc);
  return acc;
}

// y (n_x, permuted) = Jc_p^T v  (+ optional: out = base - Jc_p^T v)
__global__ void k_spmv_jctp(DevPlan d, const double* __restrict__ v, double* out, const double* base, int use_stop) {
  if (use_stop && d.sc->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_x) return;
  const int* src = d.jctp_src;
  const double acc = sparse_row_dot(d.jctp_rp[i], d.jctp_rp[i + 1], d.jc_s, [src](int p) { return src[p]; }, d.jctp_ci, v);
  out[i] = base ? base[i] - acc : acc;
}

// mode 0: out = Jc_p z - sub            (CG right-hand side, setup_conjugate_gradient)
// mode 1: out = out - Jc_p z            (r = b - S x0)
// mode 2: w = Jc_p z, delta = w.r, alpha = gam/delta          (CG start)
// mode 3: w = Jc_p z, delta = w.r, recurrence for alpha/beta  (CG iteration)
// mode 4: r.r of out = out - Jc_p z into gam                  (start residual)
__global__ void __launch_bounds__(kBlock) k_spmv_jcp(DevPlan d, const double* __restrict__ z, double* out, const double* sub,
                                                     int mode, int use_stop) {
  if (use_stop && d.sc->stop) return;
  double part[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.m_c; k += gridDim.x * blockDim.x) {
    const double acc = sparse_row_dot(d.jc_rp[k], d.jc_rp[k + 1], d.jc_s, [](int p) { return p; }, d.jcp_ci, z);
    if (mode == 0) out[k] = acc - sub[k];
    else if (mode == 1 || mode == 4) {
      double v = out[k] - acc;
      out[k] = v;
      part[0] = fma(v, v, part[0]);
    } else {
      out[k] = acc;
      part[0] = fma(acc, d.cg_r[k], part[0]);
    }
  }
  if (mode == 0 || mode == 1) return;
  double tot[1];
  if (grid_reduce_last<1>(part, d.red, &d.sc->ticket[0], tot)) {
    DevScalars* s = d.sc;
    if (mode == 4) {
      s->gam = tot[0];
      s->gam0 = tot[0];
    } else if (mode == 2) {
      s->delta = tot[0];
      s->alpha = s->gam / s->delta;
      s->beta = 0.0;
    } else {
      s->delta = tot[0];
      s->beta = s->gam1 / s->gam;
      s->gam = s->gam1;
      s->alpha = s->gam / (s->delta - s->beta * s->gam / s->alpha);
    }
  }
}

// p = r + beta p; s = w + beta s; x += alpha p; r -= alpha s; gam1 = r.r.
// Stops when sqrt(r.r) < rtol * ||r0|| (rtol = cg_rtol, or cg_rtol_refine
// for a refinement correction; > 0), else when
// sqrt(r.r) < cg_tol, the reference's absolute test (SchurCG.cpp:156), or
// when the iteration budget is spent.  In the graph (with_cond) it also sets
// the CG while node's condition: the rest of a body that stops is skipped
// (its kernels test `stop`) and the loop ends after it.
__global__ void __launch_bounds__(kBlock) k_cg_update(DevPlan d, cudaGraphConditionalHandle h, int with_cond) {
  DevScalars* s = d.sc;
  if (s->stop || (s->solve_flags & 1)) {  // stopped, or a triangular-solve wait gave up
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (!s->stop) s->stop = 3;
      if (with_cond) cudaGraphSetConditional(h, 0u);
    }
    return;
  }
  const double alpha = s->alpha, beta = s->beta;
  double part[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.m_c; k += gridDim.x * blockDim.x) {
    const double r = d.cg_r[k];
    const double p = fma(beta, d.cg_p[k], r);
    const double sv = fma(beta, d.cg_s[k], d.cg_w[k]);
    d.cg_p[k] = p;
    d.cg_s[k] = sv;
    d.cg_x[k] = fma(alpha, p, d.cg_x[k]);
    const double rn = fma(-alpha, sv, r);
    d.cg_r[k] = rn;
    part[0] = fma(rn, rn, part[0]);
  }
  double tot[1];
  if (grid_reduce_last<1>(part, d.red, &s->ticket[1], tot)) {
    s->gam1 = tot[0];
    s->it += 1;
    s->it_total += 1;
    s->cg_err = sqrt(tot[0]);
    // relative mode (refinement corrections have tiny right-hand sides, an
    // absolute floor would stop them early); absolute mode = the reference
    const double thr = s->rtol_cur > 0.0 ? s->rtol_cur * sqrt(s->gam0) : d.cg_tol;
    if (sqrt(tot[0]) < thr) s->stop = 1;
    // iteration budget; an independent count of loop bodies bounds the
    // while node even if the iteration counter stalled
    s->cond_calls += 1;
    if (!s->stop && (s->it >= d.cg_itmax || s->cond_calls >= d.cg_itmax)) {
      s->stop = 2;
      s->stop_main += 1;
    }
    if (with_cond) cudaGraphSetConditional(h, s->stop ? 0u : 1u);
  }
}

// Opens a while loop whose body runs at least once: a conditional handle's
// default value is applied only when the whole graph is launched, so a loop
// nested in another loop's body is re-armed by this kernel every time.
__global__ void k_cond_arm(cudaGraphConditionalHandle h) { cudaGraphSetConditional(h, 1u); }

// host-driven loop: mark a CG run that used its whole budget
__global__ void k_cg_mark(DevPlan d) {
  DevScalars* s = d.sc;
  if (!s->stop) {
    s->stop = 2;
    s->stop_main += 1;
  }
}

// setup(): r = w = p = s = b, x = x0 (SchurCG.cpp:89-100); zero_x0 for a
// refinement correction.
__global__ void k_cg_setup(DevPlan d, int zero_x0) {
  const int stride = gridDim.x * blockDim.x;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.m_c; k += stride) {
    const double b = d.schur[k];
    d.cg_r[k] = b;
    d.cg_w[k] = b;
    d.cg_p[k] = b;
    d.cg_s[k] = b;
    d.cg_x[k] = zero_x0 ? 0.0 : d.y0[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    DevScalars* s = d.sc;
    s->beta = 0.0;
    s->it = 0;
    s->rtol_cur = zero_x0 ? d.cg_rtol_refine : d.cg_rtol;  // refinement corrections start from 0
    s->cond_calls = 0;
    s->stop = d.m_c == 0 ? 1 : 0;
    s->gam1 = 0.0;
    s->cg_err = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Step a10: recovery of dx, ds, dy, dyd (recover_solution, HykktSolver.cpp:410-457)
// into (x, y) / (s, yd) or, for a refinement correction, into the delta
// buffers with the residual as right-hand side.
// ---------------------------------------------------------------------------
__global__ void k_recover_x(DevPlan d, const double* __restrict__ zp, double* x, double* y) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = tid; i < d.n_x; i += stride) x[i] = dmul(zp[d.rev_perm[i]], d.max_d[i]);
  for (int k = tid; k < d.m_c; k += stride) y[k] = dmul(d.cg_x[k], d.max_d[d.n_x + k]);
}

__global__ void k_recover_s(DevPlan d, const double* __restrict__ x, const double* __restrict__ ryd,
                            const double* __restrict__ rs, double* s_out, double* yd_out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.m_d) return;
  double s;
  if (d.jd_flag) {
    double acc = 0.0;
    for (int p = d.jd_rp[k]; p < d.jd_rp[k + 1]; ++p) acc = fma(d.jd_v[p], x[d.jd_ci[p]], acc);
    s = acc - ryd[k];
  } else {
    s = -ryd[k];
  }
  s_out[k] = s;
  yd_out[k] = dmul(s, d.ds_v[k]) - rs[k];
}

// z += dz after a refinement correction
__global__ void k_apply_delta(DevPlan d) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = tid; i < d.n_x; i += stride) d.x[i] += d.dx[i];
  for (int k = tid; k < d.m_c; k += stride) d.y[k] += d.dy[k];
  for (int k = tid; k < d.m_d; k += stride) {
    d.s[k] += d.ds[k];
    d.yd[k] += d.dyd[k];
  }
}

// ---------------------------------------------------------------------------
// Step a11: residual of the full 4x4 KKT system (check_error,
// HykktSolver.cpp:846-930, extended with the rows the reference assumes 0).
// Writes the four residual blocks (the right-hand side of a refinement
// correction) and their squared norms.
// ---------------------------------------------------------------------------
// (s, c) += a*b with the rounding errors of the product (FMA) and of the sum
// (two-sum) carried in c: residuals of large, nearly cancelling terms come
// out as if accumulated in twice the working precision (Ogita, Rump and
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).
__device__ __forceinline__ void acc2(double& s, double& c, double a, double b) {
  const double p = __dmul_rn(a, b);
  const double pe = fma(a, b, -p);
  const double t = __dadd_rn(s, p);
  const double z = __dsub_rn(t, s);
  const double e = __dadd_rn(__dsub_rn(s, __dsub_rn(t, z)), __dsub_rn(p, z));
  s = t;
  c = __dadd_rn(c, __dadd_rn(e, pe));
}

__global__ void __launch_bounds__(kBlock) k_residual(DevPlan d) {
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = 0.0;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = tid; i < d.n_x; i += stride) {  // r1 = rx - H x - Jd^T yd - Jc^T y
    const double rx = d.rx[i];
    v[0] = fma(rx, rx, v[0]);
    double sh = rx, c = 0.0;
    for (int p = d.h_rp[i]; p < d.h_rp[i + 1]; ++p) acc2(sh, c, -d.h_v[p], d.x[d.h_ci[p]]);
    if (d.jd_flag)
      for (int q = d.jdt_rp[i]; q < d.jdt_rp[i + 1]; ++q) acc2(sh, c, -d.jd_v[d.jdt_src[q]], d.yd[d.jdt_ci[q]]);
    for (int q = d.jct_rp[i]; q < d.jct_rp[i + 1]; ++q) acc2(sh, c, -d.jc_v[d.jct_src[q]], d.y[d.jct_ci[q]]);
    const double r = __dadd_rn(sh, c);
    d.rr_x[i] = r;
    v[4] = fma(r, r, v[4]);
  }
  for (int k = tid; k < d.m_d; k += stride) {
    const double rs = d.rs[k], rd = d.ryd[k];
    v[1] = fma(rs, rs, v[1]);
    v[3] = fma(rd, rd, v[3]);
    double s2 = rs, c2 = 0.0;  // r2 = rs - (Ds s - yd)
    acc2(s2, c2, -d.ds_v[k], d.s[k]);
    acc2(s2, c2, d.yd[k], 1.0);
    const double r2 = __dadd_rn(s2, c2);
    v[5] = fma(r2, r2, v[5]);
    double s4 = rd, c4 = 0.0;  // r4 = ryd - (Jd x - s)
    if (d.jd_flag)
      for (int p = d.jd_rp[k]; p < d.jd_rp[k + 1]; ++p) acc2(s4, c4, -d.jd_v[p], d.x[d.jd_ci[p]]);
    acc2(s4, c4, d.s[k], 1.0);
    const double r4 = __dadd_rn(s4, c4);
    v[7] = fma(r4, r4, v[7]);
    d.rr_s[k] = r2;
    d.rr_yd[k] = r4;
  }
  for (int k = tid; k < d.m_c; k += stride) {  // r3 = ry - Jc x
    const double rc = d.ry[k];
    v[2] = fma(rc, rc, v[2]);
    double s3 = rc, c3 = 0.0;
    for (int p = d.jc_rp[k]; p < d.jc_rp[k + 1]; ++p) acc2(s3, c3, -d.jc_v[p], d.x[d.jc_ci[p]]);
    const double r3 = __dadd_rn(s3, c3);
    d.rr_y[k] = r3;
    v[6] = fma(r3, r3, v[6]);
  }
  double tot[8];
  if (grid_reduce_last<8>(v, d.red, &d.sc->ticket[2], tot)) {
    DevScalars* s = d.sc;
    for (int k = 0; k < 8; ++k) s->nrm[k] = tot[k];
    const double nb = sqrt(tot[0] + tot[1] + tot[2] + tot[3]);
    s->rel_res_ref = sqrt(tot[4] + tot[6]) / nb;
    s->rel_res_full = sqrt(tot[4] + tot[5] + tot[6] + tot[7]) / nb;
    if (s->refine_it == 0) s->rel_res_first = s->rel_res_full;
  }
}

// Iterative refinement on the full KKT system: continue while the relative
// residual is above the target, the last step at least halved it (a step
// that does not has met the floor that rounding the solution to FP64 sets)
// and the step budget is not used up.
__device__ __forceinline__ bool refine_continue(const DevPlan& d, const DevScalars* s) {
  const double r = s->rel_res_full;
  return r > d.refine_target && r == r && s->refine_it < d.refine_max && !(s->solve_flags & 1) &&
         (s->refine_it == 0 || r < 0.5 * s->rel_res_prev);
}

__global__ void k_refine_cond(DevPlan d, cudaGraphConditionalHandle h) {
  DevScalars* s = d.sc;
  s->refine_calls += 1;
  const unsigned int cont = (refine_continue(d, s) && s->refine_calls <= d.refine_max + 1) ? 1u : 0u;
  s->rel_res_prev = s->rel_res_full;
  cudaGraphSetConditional(h, cont);
}

// host-driven refinement loop: the same decision, written to solve_flags bit 1
__global__ void k_refine_decide(DevPlan d) {
  DevScalars* s = d.sc;
  if (refine_continue(d, s)) s->solve_flags &= ~2;
  else s->solve_flags |= 2;
  s->rel_res_prev = s->rel_res_full;
}

__global__ void k_refine_begin(DevPlan d) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    d.sc->refine_it += 1;
  }
}

__global__ void k_refine_reset(DevPlan d) {
  if (threadIdx.x == 0 && blockIdx.x == 0) d.sc->refine_calls = 0;
}

}  // namespace hykkt
