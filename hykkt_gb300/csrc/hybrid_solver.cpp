// hybrid_solver: command-line drop-in for the reference's hybrid driver
// (examples/cuSolver_driver_hybrid.cpp:24-44; CTest cases hybrid1/hybrid2,
// examples/CMakeLists.txt:114-119):
//
//   hybrid_solver h ds jc jd rx rs ry ryd skip gamma
//
// Reads the eight Matrix-Market blocks (H lower-triangle symmetric, the others
// general; `skip` lines consumed before the sizes are parsed from the last of
// them; right-hand sides skip exactly two lines), solves once and exits 0
// when the relative residual is below 1e-2 (hybrid.cpp:679-685).  Prints the
// residual of the reference's definition and the full 4x4 residual.
#include <cstdio>
#include <cstdlib>

#include "HykktSolver.hpp"

int main(int argc, char* argv[]) {
  if (argc != 11) {
    std::printf("Incorrect number of inputs. Exiting ...\n");
    return -1;
  }
  const int skip_lines = std::atoi(argv[9]);
  const double gamma = std::atof(argv[10]);
  HykktSolver hs(gamma);
  hs.read_matrix_files(argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], skip_lines);
  const int status = hs.execute();
  hykkt_info info;
  if (hs.get_info(&info) == HYKKT_OK) {
    std::printf("CG iterations %d, CG error %.17g\n", info.cg_iterations, info.cg_residual);
    std::printf("||Ax-b||/||b|| = %.17g\n", info.rel_residual);
    std::printf("full 4x4 relative residual = %.17g\n", info.rel_residual_full);
  }
  std::printf(status == 0 ? "Residual test passed\n" : "Residual test failed\n");
  return status;
}
