"""Matrix-Market input with the reference's skip semantics (CPU).

read_mm_file_into_coo consumes `skip` lines and parses the last as the size
line; read_rhs skips exactly two lines (src/input_functions.cpp:16-217).
The drop-in reader (C++ API, exercised through a tiny program) and the
oracle's reader must give identical CSR arrays for both fixture layouts.
"""
import os
import subprocess

import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DUMP = r'''
#include <cstdio>
#include <cstdlib>
#include "input_functions.hpp"
int main(int argc, char** argv) {
  MMatrix a;
  read_mm_file_into_coo(argv[1], a, std::atoi(argv[2]));
  if (std::atoi(argv[3])) sym_coo_to_csr(a); else coo_to_csr(a);
  std::printf("%d %d %d\n", a.n_, a.m_, a.nnz_);
  for (int i = 0; i <= a.n_; ++i) std::printf("%d ", a.csr_rows[i]);
  std::printf("\n");
  for (int i = 0; i < a.nnz_; ++i) std::printf("%d %.17g\n", a.csr_cols[i], a.csr_vals[i]);
  return 0;
}
'''


@pytest.fixture(scope="module")
def dumper(tmp_path_factory):
    d = tmp_path_factory.mktemp("dump")
    src = d / "dump.cpp"
    src.write_text(DUMP)
    exe = d / "dump"
    lib_dir = os.path.dirname(hk.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", lib_dir,
                    "-lhykkt_gb300", "-Wl,-rpath," + lib_dir], check=True)
    return str(exe)


def run_dump(exe, path, skip, sym):
    out = subprocess.run([exe, path, str(skip), str(int(sym))], capture_output=True, text=True, check=True).stdout
    lines = out.splitlines()
    n, m, nnz = (int(t) for t in lines[0].split())
    rp = np.array([int(t) for t in lines[1].split()])
    cols = np.array([int(ln.split()[0]) for ln in lines[2:]])
    vals = np.array([float(ln.split()[1]) for ln in lines[2:]])
    return n, m, nnz, rp, cols, vals


@pytest.mark.parametrize("name", ["a200_AC_10", "a2000_AC_09"])
def test_reader_matches_oracle(name, tmp_path, dumper):
    paths = H.write_fixture_files(name, str(tmp_path))
    skip = H.fixture_skip(name)
    for i, p in enumerate(paths[:4]):
        sym = i == 0
        n, m, nnz, rp, cols, vals = run_dump(dumper, p, skip, sym)
        on, om, r, c, v = O.read_mm(p, skip)
        orp, oci, ov = (O.sym_coo_to_csr(on, r, c, v) if sym else O.coo_to_csr(on, r, c, v))
        assert (n, m) == (on, om)
        assert np.array_equal(rp, orp) and np.array_equal(cols, oci) and np.array_equal(vals, ov)
    z = np.load(os.path.join(H.GOLDEN, name + ".npz"))
    for key, p in zip(("rx", "rs", "ry", "ryd"), paths[4:]):
        assert np.array_equal(O.read_rhs(p, len(z[key])), z[key])


def test_skip_semantics_parse_last_consumed_line(tmp_path, dumper):
    """With skip=3 on a file whose size line is the third line, the size is
    taken from line 3; entries start on line 4."""
    p = tmp_path / "m.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% c\n2 3 2\n1 1 1.5\n2 3 -2\n")
    n, m, nnz, rp, cols, vals = run_dump(dumper, str(p), 3, False)
    assert (n, m, nnz) == (2, 3, 2)
    assert rp.tolist() == [0, 1, 2] and cols.tolist() == [0, 2] and vals.tolist() == [1.5, -2.0]


def test_gridgen_shapes_and_determinism():
    grid = gg.make_grid(500, 0)
    s = gg.make_system(grid, 1, 1e4)
    assert (s.n_x, s.m_c, s.m_d) == (1200, 1000, 1400)
    assert s.Jd.nnz == 5600 and s.H.nnz == 7800
    s2 = gg.make_system(gg.make_grid(500, 0), 1, 1e4)
    assert np.array_equal(s.Jc.vals, s2.Jc.vals) and np.array_equal(s.rx, s2.rx)
    # H symmetric
    Hs = H.to_sp(s.H)
    assert abs(Hs - Hs.T).max() == 0


def test_gridgen_files_roundtrip(tmp_path):
    s = H.small_grid_system(n_bus=30, seed=5)
    names = gg.write_system(str(tmp_path), s)
    n, m, r, c, v = O.read_mm(names["h"], 3)
    rp, ci, vv = O.sym_coo_to_csr(n, r, c, v)
    assert np.array_equal(rp, s.H.rowptr) and np.array_equal(ci, s.H.colidx) and np.array_equal(vv, s.H.vals)
    assert np.array_equal(O.read_rhs(names["rx"], s.n_x), s.rx)


RHS_DUMP = r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "input_functions.hpp"
int main(int argc, char** argv) {
  std::vector<double> v(std::atoi(argv[2]), 0.0);
  read_rhs(argv[1], v.data());
  for (double x : v) std::printf("%.17g\n", x);
  return 0;
}
'''


def test_large_file_parallel_parse_matches_oracle(tmp_path, dumper):
    """A file of several MB is parsed in parallel byte ranges; CRLF line ends,
    blank lines and lines without three numbers are handled like the
    line-by-line reader (skipped), and the entries keep file order."""
    grid = gg.make_grid(10000, 0)
    s = gg.make_system(grid, 1, 1e5, (1e-10, 1e8), (1e-10, 1e8))
    p = tmp_path / "jc.mtx"
    gg.write_mm(str(p), s.Jc)
    lines = p.read_text().split("\n")
    head, body = lines[:3], [ln for ln in lines[3:] if ln]
    rng = np.random.default_rng(0)
    out = []
    for k, ln in enumerate(body):
        out.append(ln + ("\r" if k % 7 == 0 else ""))
        if rng.random() < 0.001:
            out.append("")          # blank line
        if rng.random() < 0.001:
            out.append("   ")       # blanks only
    q = tmp_path / "jc_mixed.mtx"
    q.write_text("\n".join(head + out) + "\n")
    assert q.stat().st_size > 4 << 20
    n, m, nnz, rp, cols, vals = run_dump(dumper, str(q), 3, False)
    on, om, r, c, v = O.read_mm(str(p), 3)
    orp, oci, ov = O.coo_to_csr(on, r, c, v)
    assert (n, m, nnz) == (on, om, len(v))
    assert np.array_equal(rp, orp) and np.array_equal(cols, oci) and np.array_equal(vals, ov)
    # right-hand side reader on the same system's vector
    names = gg.write_system(str(tmp_path / "sys"), s)
    src = tmp_path / "rhs.cpp"
    src.write_text(RHS_DUMP)
    exe = tmp_path / "rhs"
    lib_dir = os.path.dirname(hk.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", lib_dir,
                    "-lhykkt_gb300", "-Wl,-rpath," + lib_dir], check=True)
    got = subprocess.run([str(exe), names["rx"], str(s.n_x)], capture_output=True, text=True, check=True).stdout
    assert np.array_equal(np.array([float(t) for t in got.split()]), s.rx)
