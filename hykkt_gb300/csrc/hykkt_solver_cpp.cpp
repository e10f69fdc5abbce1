// The drop-in C++ class HykktSolver (include/HykktSolver.hpp) over the C ABI.
// Error behaviour follows the reference: execute() returns 0/1; setters that
// the reference guards with assert() report through stderr instead of aborting.
#include <cstdio>
#include <stdexcept>

#include "HykktSolver.hpp"

namespace {
void report(int rc, const char* what) {
  if (rc != HYKKT_OK) std::fprintf(stderr, "HykktSolver::%s: %s\n", what, hykkt_last_error());
}
}  // namespace

HykktSolver::HykktSolver(double gamma) : h_(hykkt_solver_create(gamma)) {
  if (!h_) throw std::runtime_error("HykktSolver: allocation failed");
}

HykktSolver::~HykktSolver() { hykkt_solver_destroy(h_); }

void HykktSolver::read_matrix_files(char const* const h_file, char const* const ds_file, char const* const jc_file,
                                    char const* const jd_file, char const* const rx_file, char const* const rs_file,
                                    char const* const ry_file, char const* const ryd_file, int skip_lines) {
  report(hykkt_solver_read_matrix_files(h_, h_file, ds_file, jc_file, jd_file, rx_file, rs_file, ry_file, ryd_file,
                                        skip_lines),
         "read_matrix_files");
}

void HykktSolver::set_H(int* r, int* c, double* v, int n, int m, int nnz) { report(hykkt_solver_set_H(h_, r, c, v, n, m, nnz), "set_H"); }
void HykktSolver::set_Ds(int* r, int* c, double* v, int n, int m, int nnz) { report(hykkt_solver_set_Ds(h_, r, c, v, n, m, nnz), "set_Ds"); }
void HykktSolver::set_Jc(int* r, int* c, double* v, int n, int m, int nnz) { report(hykkt_solver_set_Jc(h_, r, c, v, n, m, nnz), "set_Jc"); }
void HykktSolver::set_Jd(int* r, int* c, double* v, int n, int m, int nnz) { report(hykkt_solver_set_Jd(h_, r, c, v, n, m, nnz), "set_Jd"); }

void HykktSolver::set_rx(double* v, int n) { report(hykkt_solver_set_rx(h_, v, n), "set_rx"); }
void HykktSolver::set_rs(double* v, int n) { report(hykkt_solver_set_rs(h_, v, n), "set_rs"); }
void HykktSolver::set_ry(double* v, int n) { report(hykkt_solver_set_ry(h_, v, n), "set_ry"); }
void HykktSolver::set_ryd(double* v, int n) { report(hykkt_solver_set_ryd(h_, v, n), "set_ryd"); }

void HykktSolver::set_x_host(double* v, int n) { report(hykkt_solver_set_x_host(h_, v, n), "set_x_host"); }
void HykktSolver::set_s_host(double* v, int n) { report(hykkt_solver_set_s_host(h_, v, n), "set_s_host"); }
void HykktSolver::set_y_host(double* v, int n) { report(hykkt_solver_set_y_host(h_, v, n), "set_y_host"); }
void HykktSolver::set_yd_host(double* v, int n) { report(hykkt_solver_set_yd_host(h_, v, n), "set_yd_host"); }

void HykktSolver::set_gamma(double gamma) { report(hykkt_solver_set_gamma(h_, gamma), "set_gamma"); }

int HykktSolver::execute() {
  const int rc = hykkt_solver_execute(h_);
  if (rc != 0) std::fprintf(stderr, "HykktSolver::execute: %s\n", hykkt_last_error());
  return rc;
}

int HykktSolver::get_solution(double* x, double* s, double* y, double* yd) {
  return hykkt_solver_get_solution(h_, x, s, y, yd);
}

int HykktSolver::get_info(hykkt_info* info) { return hykkt_solver_get_info(h_, info); }
