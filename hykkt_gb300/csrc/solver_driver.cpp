// solver_driver: the reference's two-system same-sparsity flow
// (examples/cuSolver_driver_solver.cpp:5-141; CTest solver1/solver2):
//
//   solver_driver h1 ds1 jc1 jd1 rx1 rs1 ry1 ryd1 h2 ds2 jc2 jd2 rx2 rs2 ry2 ryd2 skip gamma
//
// System 1 is registered through the pointer API (borrowed buffers), solved,
// then the same buffers are overwritten in place with system 2 and execute()
// runs again on the kept symbolic analysis.  Exit status of the last execute().
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "HykktSolver.hpp"
#include "input_functions.hpp"

namespace {
struct Blocks {
  MMatrix H, Ds, Jc, Jd;
  std::vector<double> rx, rs, ry, ryd;
};
void load(Blocks& b, char** f, int skip) {
  read_mm_file_into_coo(f[0], b.H, skip);
  read_mm_file_into_coo(f[1], b.Ds, skip);
  read_mm_file_into_coo(f[2], b.Jc, skip);
  read_mm_file_into_coo(f[3], b.Jd, skip);
  sym_coo_to_csr(b.H);
  coo_to_csr(b.Ds);
  coo_to_csr(b.Jc);
  coo_to_csr(b.Jd);
  b.rx.assign(b.H.n_, 0.0);
  b.rs.assign(b.Ds.n_, 0.0);
  b.ry.assign(b.Jc.n_, 0.0);
  b.ryd.assign(b.Jd.n_, 0.0);
  read_rhs(f[4], b.rx.data());
  read_rhs(f[5], b.rs.data());
  read_rhs(f[6], b.ry.data());
  read_rhs(f[7], b.ryd.data());
}
}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 19) {
    std::printf("Incorrect number of inputs. Exiting ...\n");
    return -1;
  }
  const int skip = std::atoi(argv[17]);
  const double gamma = std::atof(argv[18]);
  Blocks s1, s2;
  load(s1, argv + 1, skip);
  load(s2, argv + 9, skip);
  std::vector<double> x(s1.H.n_, 0.0), s(s1.Ds.n_, 0.0), y(s1.Jc.n_, 0.0), yd(s1.Jd.n_, 0.0);
  HykktSolver hs(gamma);
  hs.set_H(s1.H.csr_rows, s1.H.csr_cols, s1.H.csr_vals, s1.H.n_, s1.H.m_, s1.H.nnz_);
  hs.set_Ds(s1.Ds.csr_rows, s1.Ds.csr_cols, s1.Ds.csr_vals, s1.Ds.n_, s1.Ds.m_, s1.Ds.nnz_);
  hs.set_Jc(s1.Jc.csr_rows, s1.Jc.csr_cols, s1.Jc.csr_vals, s1.Jc.n_, s1.Jc.m_, s1.Jc.nnz_);
  hs.set_Jd(s1.Jd.csr_rows, s1.Jd.csr_cols, s1.Jd.csr_vals, s1.Jd.n_, s1.Jd.m_, s1.Jd.nnz_);
  hs.set_rx(s1.rx.data(), s1.H.n_);
  hs.set_rs(s1.rs.data(), s1.Ds.n_);
  hs.set_ry(s1.ry.data(), s1.Jc.n_);
  hs.set_ryd(s1.ryd.data(), s1.Jd.n_);
  hs.set_x_host(x.data(), s1.H.n_);
  hs.set_s_host(s.data(), s1.Ds.n_);
  hs.set_y_host(y.data(), s1.Jc.n_);
  hs.set_yd_host(yd.data(), s1.Jd.n_);
  int status = hs.execute();
  hykkt_info info;
  if (hs.get_info(&info) == HYKKT_OK)
    std::printf("system 1: ||Ax-b||/||b|| = %.17g (full %.17g), CG iterations %d\n", info.rel_residual,
                info.rel_residual_full, info.cg_iterations);
  if (status == 1) return 1;
  copy_mmatrix(s2.H, s1.H);
  copy_mmatrix(s2.Ds, s1.Ds);
  copy_mmatrix(s2.Jc, s1.Jc);
  copy_mmatrix(s2.Jd, s1.Jd);
  copy_vector(s2.rx.data(), s1.rx.data(), (int)s1.rx.size());
  copy_vector(s2.rs.data(), s1.rs.data(), (int)s1.rs.size());
  copy_vector(s2.ry.data(), s1.ry.data(), (int)s1.ry.size());
  copy_vector(s2.ryd.data(), s1.ryd.data(), (int)s1.ryd.size());
  status = hs.execute();
  if (hs.get_info(&info) == HYKKT_OK)
    std::printf("system 2: ||Ax-b||/||b|| = %.17g (full %.17g), CG iterations %d\n", info.rel_residual,
                info.rel_residual_full, info.cg_iterations);
  return status;
}
