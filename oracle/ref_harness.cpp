// Timing and solution-dump harness for the reference's own GPU solve path.
//
// MEASUREMENT INFRASTRUCTURE ONLY: linked against the reference's sources as
// staged and built by oracle/ref_build.py (oracle/_ref/); the product never
// uses it.  It drives the reference through its public API exactly as the
// reference's two-system driver does (examples/cuSolver_driver_solver.cpp:
// 96-137): borrowed host CSR buffers set once with set_H/set_Ds/set_Jc/set_Jd,
// right-hand sides with set_rx/rs/ry/ryd, zero initial guesses with
// set_*_host, then execute() per system with the values overwritten in
// place (same sparsity).  The reference keeps its solution on the device
// with no accessor (src/HykktSolver.cpp:451-456); the harness reads the four
// device vectors d_x_, d_s_, d_y_, d_yd_ directly, for which it opens the
// class's private members to this translation unit only.
//
// Input: a binary file (oracle/refgpu.py writes it):
//   int32 magic 0x4b4b5442, n_x, m_c, m_d, nnz_h, nnz_jc, nnz_jd, nsys
//   double gamma
//   int32 h_rp[n_x+1] h_ci[nnz_h] ds_rp[m_d+1] ds_ci[m_d] jc_rp[m_c+1]
//         jc_ci[nnz_jc] jd_rp[m_d+1] jd_ci[nnz_jd]
//   per system: double h_v[nnz_h] ds_v[m_d] jc_v[nnz_jc] jd_v[nnz_jd]
//                      rx[n_x] rs[m_d] ry[m_c] ryd[m_d]
// Calls: the first execute() (system 0: symbolic set-up + numeric solve,
// src/HykktSolver.cpp:240-286), then one execute() per system 0..nsys-1
// (numeric only).  --itmax N raises the Schur CG budget after the first call
// (SchurComplementConjugateGradient::set_solver_itmax; the reference's value
// is 100, SchurComplementConjugateGradient.hpp:125).
// Output: one JSON line per call on stdout: wall-clock and CUDA-event time of
// execute() (device synchronised before and after; the reference runs on the
// legacy default stream and synchronises on the host inside every CG
// iteration), its return value, the CG iterations and error and the relative
// residual it printed (SchurCG.cpp:157,188-190, HykktSolver.cpp:914).  The
// reference's own prints go to a temporary file and are parsed.  --dump DIR
// writes DIR/sol_<k>.bin (x, s, y, yd as doubles) after numeric call k.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusparse.h>
#include <fcntl.h>
#include <unistd.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "SchurComplementConjugateGradient.hpp"
#define private public
#include "HykktSolver.hpp"
#undef private

namespace {

struct Input {
  int n_x = 0, m_c = 0, m_d = 0, nnz_h = 0, nnz_jc = 0, nnz_jd = 0, nsys = 0;
  double gamma = 0;
  std::vector<int> h_rp, h_ci, ds_rp, ds_ci, jc_rp, jc_ci, jd_rp, jd_ci;
  std::vector<double> vals;  // nsys value sets, back to back
  int64_t per_sys() const { return (int64_t)nnz_h + m_d + nnz_jc + nnz_jd + n_x + m_d + m_c + m_d; }
};

bool read_input(const char* path, Input& in) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  int hdr[8];
  bool ok = std::fread(hdr, sizeof(int), 8, f) == 8 && hdr[0] == 0x4b4b5442;
  if (ok) {
    in.n_x = hdr[1], in.m_c = hdr[2], in.m_d = hdr[3], in.nnz_h = hdr[4], in.nnz_jc = hdr[5], in.nnz_jd = hdr[6];
    in.nsys = hdr[7];
    ok = std::fread(&in.gamma, sizeof(double), 1, f) == 1;
  }
  auto rd = [&](std::vector<int>& v, int64_t n) {
    v.resize(n);
    if (ok && n) ok = std::fread(v.data(), sizeof(int), n, f) == (size_t)n;
  };
  rd(in.h_rp, in.n_x + 1);
  rd(in.h_ci, in.nnz_h);
  rd(in.ds_rp, in.m_d + 1);
  rd(in.ds_ci, in.m_d);
  rd(in.jc_rp, in.m_c + 1);
  rd(in.jc_ci, in.nnz_jc);
  rd(in.jd_rp, in.m_d + 1);
  rd(in.jd_ci, in.nnz_jd);
  if (ok) {
    in.vals.resize(in.per_sys() * in.nsys);
    ok = std::fread(in.vals.data(), sizeof(double), in.vals.size(), f) == in.vals.size();
  }
  std::fclose(f);
  return ok;
}

// execute() with stdout sent to a file (HYKKT_REF_CAPTURE, else a temporary
// one); returns what it printed.  The reference exits on its own errors
// (cuda_check_errors.hpp) with the reason printed to stdout, so a named
// capture file keeps that reason for the caller.
int run_quiet(HykktSolver& hs, std::string& printed) {
  std::fflush(stdout);
  std::cout.flush();
  const char* named = std::getenv("HYKKT_REF_CAPTURE");
  char tmpl[] = "/tmp/ref_harness_XXXXXX";
  const int fd = named ? open(named, O_CREAT | O_TRUNC | O_WRONLY, 0644) : mkstemp(tmpl);
  const char* path = named ? named : tmpl;
  const int saved = dup(1);
  dup2(fd, 1);
  const int rc = hs.execute();
  std::fflush(stdout);
  std::cout.flush();
  dup2(saved, 1);
  close(saved);
  close(fd);
  std::ifstream t(path);
  std::stringstream ss;
  ss << t.rdbuf();
  printed = ss.str();
  if (!named) unlink(tmpl);
  return rc;
}

// last value printed after `key` (or fallback)
double parse_after(const std::string& s, const char* key, double fallback) {
  const size_t p = s.rfind(key);
  if (p == std::string::npos) return fallback;
  return std::strtod(s.c_str() + p + std::strlen(key), nullptr);
}

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "ref_harness: %s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_harness <system.bin> [--itmax N] [--dump DIR] [--calls K]\n");
    return 2;
  }
  int itmax = 0, max_calls = -1;
  std::string dump;
  for (int a = 2; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--itmax") && a + 1 < argc) itmax = std::atoi(argv[++a]);
    else if (!std::strcmp(argv[a], "--dump") && a + 1 < argc) dump = argv[++a];
    else if (!std::strcmp(argv[a], "--calls") && a + 1 < argc) max_calls = std::atoi(argv[++a]);
  }
  Input in;
  if (!read_input(argv[1], in)) {
    std::fprintf(stderr, "ref_harness: cannot read %s\n", argv[1]);
    return 2;
  }
  // borrowed buffers, as the reference's API expects (HykktSolver.hpp:49-116)
  std::vector<double> h_v(in.nnz_h), ds_v(in.m_d), jc_v(in.nnz_jc), jd_v(in.nnz_jd);
  std::vector<double> rx(in.n_x), rs(in.m_d), ry(in.m_c), ryd(in.m_d);
  std::vector<double> x0(in.n_x, 0.0), s0(in.m_d, 0.0), y0(in.m_c, 0.0), yd0(in.m_d, 0.0);
  auto load = [&](int k) {
    const double* p = in.vals.data() + in.per_sys() * k;
    for (std::vector<double>* v : {&h_v, &ds_v, &jc_v, &jd_v, &rx, &rs, &ry, &ryd}) {
      std::memcpy(v->data(), p, v->size() * sizeof(double));
      p += v->size();
    }
  };
  load(0);
  check(cudaFree(nullptr), "context");
  HykktSolver* hs = new HykktSolver(in.gamma);
  hs->set_H(in.h_rp.data(), in.h_ci.data(), h_v.data(), in.n_x, in.n_x, in.nnz_h);
  hs->set_Ds(in.ds_rp.data(), in.ds_ci.data(), ds_v.data(), in.m_d, in.m_d, in.m_d);
  hs->set_Jc(in.jc_rp.data(), in.jc_ci.data(), jc_v.data(), in.m_c, in.n_x, in.nnz_jc);
  hs->set_Jd(in.jd_rp.data(), in.jd_ci.data(), jd_v.data(), in.m_d, in.n_x, in.nnz_jd);
  hs->set_rx(rx.data(), in.n_x);
  hs->set_rs(rs.data(), in.m_d);
  hs->set_ry(ry.data(), in.m_c);
  hs->set_ryd(ryd.data(), in.m_d);
  hs->set_x_host(x0.data(), in.n_x);
  hs->set_s_host(s0.data(), in.m_d);
  hs->set_y_host(y0.data(), in.m_c);
  hs->set_yd_host(yd0.data(), in.m_d);

  cudaEvent_t e0, e1;
  check(cudaEventCreate(&e0), "event");
  check(cudaEventCreate(&e1), "event");
  const int ncalls = 1 + (max_calls >= 0 ? std::min(max_calls, in.nsys) : in.nsys);
  for (int c = 0; c < ncalls; ++c) {
    const int k = c == 0 ? 0 : c - 1;  // call 0: first call on system 0; then systems 0..nsys-1
    load(k);
    if (c == 1 && itmax > 0) hs->sccg_->set_solver_itmax(itmax);
    check(cudaDeviceSynchronize(), "sync");
    const auto t0 = std::chrono::steady_clock::now();
    check(cudaEventRecord(e0, 0), "record");
    std::string out;
    const int rc = run_quiet(*hs, out);
    check(cudaEventRecord(e1, 0), "record");
    check(cudaEventSynchronize(e1), "sync");
    const auto t1 = std::chrono::steady_clock::now();
    check(cudaGetLastError(), "execute");
    float ev_ms = 0;
    check(cudaEventElapsedTime(&ev_ms, e0, e1), "elapsed");
    const double wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const bool converged = out.rfind("Convergence occured at iteration") != std::string::npos;
    int its = converged ? (int)parse_after(out, "Convergence occured at iteration", -1)
                        : (int)parse_after(out, "No CG convergence in", -1);
    const double cg_err = parse_after(out, "Error is", -1);
    const double res = parse_after(out, "||Ax-b||/||b|| =", -1);
    if (!dump.empty() && c > 0) {
      std::vector<double> sol((size_t)in.n_x + 2 * in.m_d + in.m_c);
      double* p = sol.data();
      check(cudaMemcpy(p, hs->d_x_, sizeof(double) * in.n_x, cudaMemcpyDeviceToHost), "d_x_");
      check(cudaMemcpy(p + in.n_x, hs->d_s_, sizeof(double) * in.m_d, cudaMemcpyDeviceToHost), "d_s_");
      check(cudaMemcpy(p + in.n_x + in.m_d, hs->d_y_, sizeof(double) * in.m_c, cudaMemcpyDeviceToHost), "d_y_");
      check(cudaMemcpy(p + in.n_x + in.m_d + in.m_c, hs->d_yd_, sizeof(double) * in.m_d, cudaMemcpyDeviceToHost),
            "d_yd_");
      const std::string path = dump + "/sol_" + std::to_string(k) + ".bin";
      FILE* f = std::fopen(path.c_str(), "wb");
      if (!f || std::fwrite(sol.data(), sizeof(double), sol.size(), f) != sol.size()) {
        std::fprintf(stderr, "ref_harness: cannot write %s\n", path.c_str());
        return 2;
      }
      std::fclose(f);
    }
    std::printf("{\"call\": %d, \"system\": %d, \"first\": %s, \"wall_ms\": %.6f, \"event_ms\": %.6f, "
                "\"execute\": %d, \"cg_converged\": %s, \"cg_iterations\": %d, \"cg_error\": %.17g, "
                "\"rel_residual\": %.17g, \"itmax\": %d}\n",
                c, k, c == 0 ? "true" : "false", wall_ms, (double)ev_ms, rc, converged ? "true" : "false", its,
                cg_err, res, c == 0 || itmax <= 0 ? 100 : itmax);
    std::fflush(stdout);
  }
  delete hs;
  return 0;
}
