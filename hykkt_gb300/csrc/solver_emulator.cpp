// solver_emulator: the reference's sequence flow -- one solver object, a
// list of same-sparsity systems read from files and solved in turn, as an
// interior-point method would call it (examples/cuSolver_driver_solver_emulator.cpp:52-99):
//
//   solver_emulator base_dir base_name seq[,seq...] skip gamma
//
// For each sequence id s it reads
//   base_dir/block_{H,Ds,Jc,Jd}_matrix_<base_name>_<s>.mtx
//   base_dir/block_{rx,rs,ry,rd}_rhs_<base_name>_<s>.mtx
// with HykktSolver::read_matrix_files and runs execute(); the first failing
// execute() ends the run with exit status 1.  Additions: per sequence the
// reference's residual, the full 4-block residual, the CG iterations and the
// read / solve wall times.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "HykktSolver.hpp"

namespace {
std::vector<std::string> split(const std::string& s, const std::string& delim) {
  std::vector<std::string> out;
  size_t start = 0, pos;
  while ((pos = s.find(delim, start)) != std::string::npos) {
    out.push_back(s.substr(start, pos - start));
    start = pos + delim.size();
  }
  out.push_back(s.substr(start));
  return out;
}

std::string block_file(const std::string& dir, const char* preamble, const std::string& base, const std::string& seq) {
  return dir + "/" + preamble + "_" + base + "_" + seq + ".mtx";
}

double seconds_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}
}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 6) {
    std::printf("Incorrect number of inputs. Exiting ...\n");
    return -1;
  }
  std::printf("Starting ...\n");
  const std::string dir = argv[1], base = argv[2];
  const std::vector<std::string> seqs = split(argv[3], ",");
  const int skip = std::atoi(argv[4]);
  const double gamma = std::atof(argv[5]);
  HykktSolver hs(gamma);
  for (const std::string& s : seqs) {
    std::printf("Working on Sequence: %s\n\n", s.c_str());
    auto t = std::chrono::steady_clock::now();
    const std::string h = block_file(dir, "block_H_matrix", base, s), ds = block_file(dir, "block_Ds_matrix", base, s),
                      jc = block_file(dir, "block_Jc_matrix", base, s), jd = block_file(dir, "block_Jd_matrix", base, s),
                      rx = block_file(dir, "block_rx_rhs", base, s), rs = block_file(dir, "block_rs_rhs", base, s),
                      ry = block_file(dir, "block_ry_rhs", base, s), ryd = block_file(dir, "block_rd_rhs", base, s);
    hs.read_matrix_files(h.c_str(), ds.c_str(), jc.c_str(), jd.c_str(), rx.c_str(), rs.c_str(), ry.c_str(), ryd.c_str(),
                         skip);
    const double t_read = seconds_since(t);
    t = std::chrono::steady_clock::now();
    const int status = hs.execute();
    const double t_solve = seconds_since(t);
    hykkt_info info;
    if (hs.get_info(&info) == HYKKT_OK)
      std::printf("sequence %s: ||Ax-b||/||b|| = %.17g (full %.17g), CG iterations %d, read %.3f s, solve %.3f s\n",
                  s.c_str(), info.rel_residual, info.rel_residual_full, info.cg_iterations, t_read, t_solve);
    if (status == 1) return 1;
  }
  return 0;
}
