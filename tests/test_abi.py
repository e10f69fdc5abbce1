"""The C-ABI library: it loads, exports every symbol include/*.h declares, and
the drop-in C++ headers compile against it (CPU; no compute calls)."""
import os
import re
import subprocess

import hykkt_gb300 as hk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions():
    txt = open(os.path.join(INC, "hykkt_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b(hykkt_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def exported_functions():
    out = subprocess.run(["nm", "-D", "--defined-only", hk.LIB_PATH], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_loads():
    L = hk.lib()
    assert L.hykkt_version().decode().startswith("hykkt_gb300")


def test_every_declared_symbol_is_exported():
    decl = declared_functions()
    assert len(decl) >= 40
    exp = exported_functions()
    missing = [d for d in decl if d not in exp]
    assert not missing, missing


def test_cpp_dropin_compiles_and_links(tmp_path):
    """A caller of the reference's C++ API builds unchanged against the headers."""
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include "HykktSolver.hpp"
#include "input_functions.hpp"
int main(int argc, char** argv) {
  if (argc < 2) return 0;
  MMatrix h;
  read_mm_file_into_coo(argv[1], h, 2);
  sym_coo_to_csr(h);
  HykktSolver hs(1e4);
  hs.set_H(h.csr_rows, h.csr_cols, h.csr_vals, h.n_, h.m_, h.nnz_);
  hs.set_gamma(1e5);
  return hs.execute();
}
''')
    exe = tmp_path / "caller"
    lib_dir = os.path.dirname(hk.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-I", INC, str(src), "-o", str(exe), "-L", lib_dir, "-lhykkt_gb300",
                    "-Wl,-rpath," + lib_dir], check=True)
    # no arguments: returns before touching the GPU
    assert subprocess.run([str(exe)]).returncode == 0


def test_cli_argument_count():
    r = subprocess.run([os.path.join(hk.BIN_DIR, "hybrid_solver")], capture_output=True, text=True)
    assert r.returncode != 0 and "Incorrect number of inputs" in r.stdout
    r = subprocess.run([os.path.join(hk.BIN_DIR, "solver_driver")], capture_output=True, text=True)
    assert r.returncode != 0 and "Incorrect number of inputs" in r.stdout


def test_index_plus_value_comparator(tmp_path):
    """indexPlusValue_comp orders by idx only, for qsort (the reference's
    input_functions.hpp:10-19 contract: -1, 0, 1)."""
    src = tmp_path / "cmp.cpp"
    src.write_text(r"""
#include <cstdio>
#include <cstdlib>
#include "input_functions.hpp"
int main() {
  indexPlusValue v[6] = {{0.5, 4}, {1.5, -2}, {2.5, 9}, {3.5, 0}, {4.5, 4}, {5.5, 1}};
  indexPlusValue a{1.0, 3}, b{-7.0, 3}, c{0.0, 8};
  if (indexPlusValue_comp(&a, &b) != 0 || indexPlusValue_comp(&a, &c) != -1 || indexPlusValue_comp(&c, &a) != 1) return 2;
  std::qsort(v, 6, sizeof(indexPlusValue), indexPlusValue_comp);
  for (int i = 0; i < 6; ++i) std::printf("%d ", v[i].idx);
  return 0;
}
""")
    exe = tmp_path / "cmp"
    lib_dir = os.path.dirname(hk.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-I", INC, str(src), "-o", str(exe), "-L", lib_dir, "-lhykkt_gb300",
                    "-Wl,-rpath," + lib_dir], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["-2", "0", "1", "4", "4", "9"]
