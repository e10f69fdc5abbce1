// Drop-in C++ API: the public interface of the reference's HykktSolver
// (src/HykktSolver.hpp:17-137) implemented over the hykkt_gb300 C ABI.
// A caller of the reference recompiles against this header and links
// libhykkt_gb300.so; no other change is needed.
#pragma once

#include <cstdint>

#include "MMatrix.hpp"
#include "hykkt_gb300.h"

class HykktSolver {
 public:
  explicit HykktSolver(double gamma);
  ~HykktSolver();
  HykktSolver(const HykktSolver&) = delete;
  HykktSolver& operator=(const HykktSolver&) = delete;

  // Read the eight block files of one KKT system (same nonzero structure on
  // every call after the first).
  void read_matrix_files(char const* const h_file, char const* const ds_file, char const* const jc_file,
                         char const* const jd_file, char const* const rx_file, char const* const rs_file,
                         char const* const ry_file, char const* const ryd_file, int skip_lines);

  // Borrow caller-owned CSR blocks (H full symmetric).
  void set_H(int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
  void set_Ds(int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
  void set_Jc(int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);
  void set_Jd(int* rowptrs, int* colidx, double* vals, int n, int m, int nnz);

  void set_rx(double* vals, int n);
  void set_rs(double* vals, int n);
  void set_ry(double* vals, int n);
  void set_ryd(double* vals, int n);

  void set_x_host(double* vals, int n);
  void set_s_host(double* vals, int n);
  void set_y_host(double* vals, int n);
  void set_yd_host(double* vals, int n);

  void set_gamma(double gamma);

  // Solve; 0 when the relative residual is below 1e-2, 1 otherwise.
  int execute();

  // Additions over the reference API.
  int get_solution(double* x, double* s, double* y, double* yd);
  int get_info(hykkt_info* info);
  hykkt_solver_t handle() const { return h_; }

 private:
  hykkt_solver_t h_;
};
