// Component-level device entry points mirroring the reference's component
// kernels and the tests that drive them:
//   * map_idx gather                   (src/permcheck.cu:4-19)
//   * RuizClass on explicit arrays     (src/RuizClass.cpp:54-88, kernels
//                                       src/matrix_vector_ops.cu:146-266)
// The Cholesky and Schur-CG components run on the Engine (engine.cu).
#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "components.hpp"
#include "engine.hpp"

namespace hykkt {

__global__ void k_map_idx(int n, const int* __restrict__ map, const double* __restrict__ oldv, double* __restrict__ newv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) newv[i] = oldv[map[i]];
}

void map_index(int n, const int* d_map, const double* d_old, double* d_new, cudaStream_t st) {
  if (n <= 0) return;
  k_map_idx<<<(n + 255) / 256, 256, 0, st>>>(n, d_map, d_old, d_new);
  HYKKT_CUDA(cudaGetLastError());
}

// One warp per row of [A B^T; B 0]; the same operation order as the
// product path (1/sqrt of the row max, v *= s_i*s_j).
__global__ void k_ruizc_rowmax(int n, int m, const double* a_v, const int* a_i, const double* bt_v, const int* bt_i,
                               const double* b_v, const int* b_i, double* scale) {
  const int lane = threadIdx.x & 31;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= n + m) return;
  double ml = 0.0, mu = 0.0;
  if (row < n) {
    for (int p = a_i[row] + lane; p < a_i[row + 1]; p += 32) { double e = fabs(a_v[p]); if (e > ml) ml = e; }
    for (int p = bt_i[row] + lane; p < bt_i[row + 1]; p += 32) { double e = fabs(bt_v[p]); if (e > mu) mu = e; }
  } else {
    const int k = row - n;
    for (int p = b_i[k] + lane; p < b_i[k + 1]; p += 32) { double e = fabs(b_v[p]); if (e > ml) ml = e; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double a = __shfl_xor_sync(0xffffffffu, ml, o), b = __shfl_xor_sync(0xffffffffu, mu, o);
    if (a > ml) ml = a;
    if (b > mu) mu = b;
  }
  if (lane == 0) scale[row] = 1.0 / sqrt(row < n ? (ml > mu ? ml : mu) : ml);
}

__global__ void k_ruizc_scale(int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v, const int* bt_i,
                              const int* bt_j, double* b_v, const int* b_i, const int* b_j, const double* scale,
                              double* rhs1, double* rhs2, double* max_d) {
  const int lane = threadIdx.x & 31;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= n + m) return;
  const double si = scale[row];
  if (row < n) {
    for (int p = a_i[row] + lane; p < a_i[row + 1]; p += 32) a_v[p] = __dmul_rn(a_v[p], __dmul_rn(si, scale[a_j[p]]));
    for (int p = bt_i[row] + lane; p < bt_i[row + 1]; p += 32)
      bt_v[p] = __dmul_rn(bt_v[p], __dmul_rn(si, scale[n + bt_j[p]]));
    if (lane == 0) {
      rhs1[row] = __dmul_rn(rhs1[row], si);
      max_d[row] = __dmul_rn(max_d[row], si);
    }
  } else {
    const int k = row - n;
    for (int p = b_i[k] + lane; p < b_i[k + 1]; p += 32) b_v[p] = __dmul_rn(b_v[p], __dmul_rn(si, scale[b_j[p]]));
    if (lane == 0) {
      rhs2[k] = __dmul_rn(rhs2[k], si);
      max_d[row] = __dmul_rn(max_d[row], si);
    }
  }
}

__global__ void k_fill(int n, double v, double* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

void ruiz_scale(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v, const int* bt_i,
                const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1, double* rhs2, double* max_d,
                cudaStream_t st) {
  if (its < 0 || n < 0 || m < 0) throw std::invalid_argument("ruiz_scale: negative size or sweep count");
  const int tot = n + m;
  if (tot <= 0) return;
  double* scale = nullptr;
  HYKKT_CUDA(cudaMallocAsync(&scale, tot * sizeof(double), st));
  k_fill<<<(tot + 255) / 256, 256, 0, st>>>(tot, 1.0, max_d);  // reset_scaling (RuizClass.cpp:95-98)
  const int grid = (int)(((int64_t)tot * 32 + 255) / 256);
  for (int s = 0; s < its; ++s) {
    k_ruizc_rowmax<<<grid, 256, 0, st>>>(n, m, a_v, a_i, bt_v, bt_i, b_v, b_i, scale);
    k_ruizc_scale<<<grid, 256, 0, st>>>(n, m, a_v, a_i, a_j, bt_v, bt_i, bt_j, b_v, b_i, b_j, scale, rhs1, rhs2, max_d);
  }
  HYKKT_CUDA(cudaGetLastError());
  HYKKT_CUDA(cudaFreeAsync(scale, st));
}

// ---------------------------------------------------------------------------
// Ruiz scaling that allocates nothing.
//
// ruiz_scale() above takes its n+m scale vector from the stream-ordered pool
// on every call.  Some callers cannot allocate where they scale: an
// interior-point loop that reserves all of its device memory before the
// first iteration and must not touch the allocator inside it (a pool
// allocation there can fail under a fixed memory budget, or wait on other
// streams' frees).  This variant takes the scale vector from a fixed array
// compiled into the library.
//   * limit: n + m <= kRuizNoAllocMaxRows (1,048,576 rows, 8 MiB of
//     doubles); larger systems are rejected before anything is enqueued;
//   * set-up: the first call on a device resolves the array's address on
//     that device (cudaGetSymbolAddress, with that device current) and
//     caches it; make that first call before any stream capture.  The cache
//     lives as long as the process's context on the device: after
//     cudaDeviceReset the module is loaded again at another address, so a
//     process that resets a device must not call this entry point after it;
//   * nothing has to start at zero: each sweep's row-max kernel writes all
//     n+m entries before the scaling kernel of the sweep reads them;
//   * all calls on one device share the one array, so calls that overlap in
//     time (from other host threads, or on other streams whose work is still
//     in flight) race on it: the caller serialises them, e.g. on one stream.
// ---------------------------------------------------------------------------
constexpr int kRuizNoAllocMaxRows = 1 << 20;
static __device__ __align__(256) double g_ruiz_scale_scratch[kRuizNoAllocMaxRows];

static double* ruiz_scratch_on_current_device() {
  static std::mutex mu;
  static std::unordered_map<int, double*> addr;
  int dev = 0;
  HYKKT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = addr.find(dev);
  if (it != addr.end()) return it->second;
  void* p = nullptr;
  HYKKT_CUDA(cudaGetSymbolAddress(&p, g_ruiz_scale_scratch));
  addr[dev] = static_cast<double*>(p);
  return static_cast<double*>(p);
}

int ruiz_noalloc_max_rows() { return kRuizNoAllocMaxRows; }

void ruiz_scale_noalloc(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v,
                        const int* bt_i, const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1,
                        double* rhs2, double* max_d, cudaStream_t st) {
  if (its < 0 || n < 0 || m < 0) throw std::invalid_argument("ruiz_scale_noalloc: negative size or sweep count");
  const int64_t tot = (int64_t)n + m;
  if (tot > kRuizNoAllocMaxRows)
    throw std::invalid_argument("ruiz_scale_noalloc: n + m = " + std::to_string(tot) +
                                " exceeds the fixed scratch of " + std::to_string(kRuizNoAllocMaxRows) + " rows");
  double* scale = ruiz_scratch_on_current_device();
  if (tot == 0) return;
  k_fill<<<(int)((tot + 255) / 256), 256, 0, st>>>((int)tot, 1.0, max_d);  // reset_scaling (RuizClass.cpp:95-98)
  const int grid = (int)((tot * 32 + 255) / 256);
  for (int s = 0; s < its; ++s) {
    k_ruizc_rowmax<<<grid, 256, 0, st>>>(n, m, a_v, a_i, bt_v, bt_i, b_v, b_i, scale);
    k_ruizc_scale<<<grid, 256, 0, st>>>(n, m, a_v, a_i, a_j, bt_v, bt_i, bt_j, b_v, b_i, b_j, scale, rhs1, rhs2, max_d);
  }
  HYKKT_CUDA(cudaGetLastError());
}

// FP64 throughput probe: 8 independent FMA chains per thread.
__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// FP64 tensor-pipe probe: eight independent accumulator chains per warp of
// mma.sync m8n8k4 (FP64 operands and accumulators; 512 flops per warp
// instruction).  mode 1: every warp issues mma; mode 2: even warps mma, odd
// warps the DFMA chains of k_dfma_peak (do the two share one pipe?).
__global__ void k_fp64_probe(double* out, int iters, double a, double b, int mode) {
  const int warp = threadIdx.x >> 5;
  double s = 0.0;
  if (mode == 1 || (mode == 2 && (warp & 1) == 0)) {
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = threadIdx.x + k;
    const double av = a + 1e-9 * threadIdx.x, bv = b;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[k][0]), "+d"(c[k][1])
                     : "d"(av), "d"(bv));
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  } else {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    // 4x the chain steps of an mma warp's loop: a DFMA warp instruction does
    // 64 flops, an m8n8k4 one 512, so both kinds issue about equal work
    for (int i = 0; i < 4 * iters; ++i) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  }
  if (s == 12345.678) out[0] = s;
}

double fp64_probe_tflops(int mode) {
  if (mode < 0 || mode > 2) throw std::invalid_argument("fp64 probe mode must be 0, 1 or 2");
  if (mode == 0) return fp64_peak_tflops();
  int dev = 0, sms = 0;
  HYKKT_CUDA(cudaGetDevice(&dev));
  HYKKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  HYKKT_CUDA(cudaMalloc(&out, sizeof(double)));
  const int blocks = sms * 8, threads = 256, iters = 1024;
  cudaEvent_t a, b;
  HYKKT_CUDA(cudaEventCreate(&a));
  HYKKT_CUDA(cudaEventCreate(&b));
  k_fp64_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7, mode);  // warm-up
  HYKKT_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    HYKKT_CUDA(cudaEventRecord(a));
    k_fp64_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7, mode);
    HYKKT_CUDA(cudaEventRecord(b));
    HYKKT_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    HYKKT_CUDA(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double warps = (double)blocks * threads / 32;
  // mma warps: 8 chains x iters x 512 flops; DFMA warps: 32 lanes x 8 chains x 4 iters x 2 flops
  const double per_mma_warp = 8.0 * iters * 512.0, per_dfma_warp = 32.0 * 8.0 * 4.0 * iters * 2.0;
  const double flops = mode == 1 ? warps * per_mma_warp : warps / 2 * (per_mma_warp + per_dfma_warp);
  return flops / (best * 1e-3) / 1e12;
}

double fp64_peak_tflops() {
  int dev = 0, sms = 0;
  HYKKT_CUDA(cudaGetDevice(&dev));
  HYKKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  HYKKT_CUDA(cudaMalloc(&out, sizeof(double)));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  HYKKT_CUDA(cudaEventCreate(&a));
  HYKKT_CUDA(cudaEventCreate(&b));
  k_dfma_peak<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    HYKKT_CUDA(cudaEventRecord(a));
    k_dfma_peak<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    HYKKT_CUDA(cudaEventRecord(b));
    HYKKT_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    HYKKT_CUDA(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace hykkt
