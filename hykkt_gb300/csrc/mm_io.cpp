// MMatrix and the Matrix-Market readers of the drop-in API.  Same file
// semantics as the reference (src/input_functions.cpp:16-217,
// src/MMatrix.cpp:6-149); lines that do not parse are skipped instead of
// re-using the previous line's numbers, and entries beyond the declared nnz
// are rejected.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "MMatrix.hpp"
#include "input_functions.hpp"

MMatrix::MMatrix()
    : coo_rows(nullptr), coo_cols(nullptr), coo_vals(nullptr), csr_rows(nullptr), csr_cols(nullptr),
      csr_vals(nullptr), n_(0), m_(0), nnz_(0), nnz_unpacked_(0), owns_csr_data_(true) {}

MMatrix::MMatrix(int n, int m, int nnz) : MMatrix() { populate(n, m, nnz); }

MMatrix::~MMatrix() {
  delete[] coo_rows;
  delete[] coo_cols;
  delete[] coo_vals;
  if (owns_csr_data_) {
    delete[] csr_rows;
    delete[] csr_cols;
    delete[] csr_vals;
  }
}

void MMatrix::owns_csr_data(bool flag) { owns_csr_data_ = flag; }
bool MMatrix::owns_csr_data() { return owns_csr_data_; }

void MMatrix::populate(int n, int m, int nnz) {
  n_ = n;
  m_ = m;
  nnz_ = nnz;
  coo_rows = new int[nnz];
  coo_cols = new int[nnz];
  coo_vals = new double[nnz];
  csr_rows = new int[n + 1];
  csr_cols = new int[nnz];
  csr_vals = new double[nnz];
}

void MMatrix::print_csr() {
  std::cout << "Printing " << n_ << "x" << m_ << " matrix with " << nnz_ << " nonzeros:\n";
  for (int i = 0; i < nnz_; ++i) {
    if (i < n_ + 1) std::cout << std::setw(10) << csr_rows[i] << " ";
    std::cout << std::setw(10) << csr_cols[i] << " " << std::setw(10) << csr_vals[i] << "\n";
  }
}

void MMatrix::clear() {
  delete[] coo_cols; coo_cols = nullptr;
  delete[] coo_rows; coo_rows = nullptr;
  delete[] coo_vals; coo_vals = nullptr;
  if (owns_csr_data_) {
    delete[] csr_cols; csr_cols = nullptr;
    delete[] csr_rows; csr_rows = nullptr;
    delete[] csr_vals; csr_vals = nullptr;
  }
  n_ = m_ = nnz_ = 0;
}

void copy_mmatrix(const MMatrix& src, MMatrix& dst) {
  if (src.n_ != dst.n_ || src.m_ != dst.m_ || src.nnz_ != dst.nnz_)
    throw std::runtime_error("copy_mmatrix: size mismatch");
  std::copy(src.csr_rows, src.csr_rows + dst.n_ + 1, dst.csr_rows);
  std::copy(src.csr_cols, src.csr_cols + dst.nnz_, dst.csr_cols);
  std::copy(src.csr_vals, src.csr_vals + dst.nnz_, dst.csr_vals);
}

void copy_vector(const double* src, double* dst, int n) { std::copy(src, src + n, dst); }

namespace {
struct File {
  FILE* f;
  explicit File(const char* name) : f(std::fopen(name, "r")) {
    if (!f) throw std::runtime_error(std::string("cannot open ") + name);
  }
  ~File() { std::fclose(f); }
};
// fgets-style line reader without a length limit
bool read_line(FILE* f, std::string& s) {
  s.clear();
  int c;
  while ((c = std::fgetc(f)) != EOF) {
    if (c == '\n') return true;
    s.push_back((char)c);
  }
  return !s.empty();
}
}  // namespace

void read_mm_file_into_coo(const char* matrix_file_name, MMatrix& mat_a, int lines) {
  File file(matrix_file_name);
  std::string line;
  for (int i = 0; i < lines; ++i)
    if (!read_line(file.f, line)) throw std::runtime_error("read_mm_file_into_coo: file shorter than skip");
  // the last line consumed holds the sizes
  if (std::sscanf(line.c_str(), "%d %d %d", &mat_a.n_, &mat_a.m_, &mat_a.nnz_) != 3)
    throw std::runtime_error("read_mm_file_into_coo: size line not found after skipping lines");
  if (mat_a.n_ < 0 || mat_a.m_ < 0 || mat_a.nnz_ < 0) throw std::runtime_error("read_mm_file_into_coo: negative size");
  delete[] mat_a.coo_vals;
  delete[] mat_a.coo_rows;
  delete[] mat_a.coo_cols;
  mat_a.coo_vals = new double[mat_a.nnz_];
  mat_a.coo_rows = new int[mat_a.nnz_];
  mat_a.coo_cols = new int[mat_a.nnz_];
  int i = 0;
  while (read_line(file.f, line)) {
    int r, c;
    double v;
    if (std::sscanf(line.c_str(), "%d %d %lf", &r, &c, &v) != 3) continue;
    if (i >= mat_a.nnz_) throw std::runtime_error("read_mm_file_into_coo: more entries than declared");
    if (r < 1 || r > mat_a.n_ || c < 1 || c > mat_a.m_) throw std::runtime_error("read_mm_file_into_coo: index out of range");
    mat_a.coo_rows[i] = r - 1;
    mat_a.coo_cols[i] = c - 1;
    mat_a.coo_vals[i] = v;
    ++i;
  }
  if (i != mat_a.nnz_) throw std::runtime_error("read_mm_file_into_coo: fewer entries than declared");
}

namespace {
void fill_sorted_csr(int n, const std::vector<int>& counts, const std::vector<int>& rr, const std::vector<int>& cc,
                     const std::vector<double>& vv, int* rows, int* cols, double* vals) {
  rows[0] = 0;
  for (int i = 0; i < n; ++i) rows[i + 1] = rows[i] + counts[i];
  std::vector<int> next(rows, rows + n);
  const size_t nnz = rr.size();
  std::vector<std::pair<int, double>> tmp(nnz);
  for (size_t t = 0; t < nnz; ++t) tmp[next[rr[t]]++] = {cc[t], vv[t]};
  for (int i = 0; i < n; ++i)
    std::stable_sort(tmp.begin() + rows[i], tmp.begin() + rows[i + 1],
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
  for (size_t t = 0; t < nnz; ++t) {
    cols[t] = tmp[t].first;
    vals[t] = tmp[t].second;
  }
}
}  // namespace

void sym_coo_to_csr(MMatrix& mat_a) {
  std::vector<int> counts(mat_a.n_, 0), rr, cc;
  std::vector<double> vv;
  rr.reserve(2 * (size_t)mat_a.nnz_);
  cc.reserve(2 * (size_t)mat_a.nnz_);
  vv.reserve(2 * (size_t)mat_a.nnz_);
  for (int i = 0; i < mat_a.nnz_; ++i) {
    int r = mat_a.coo_rows[i], c = mat_a.coo_cols[i];
    double v = mat_a.coo_vals[i];
    rr.push_back(r); cc.push_back(c); vv.push_back(v); counts[r]++;
    if (r != c) { rr.push_back(c); cc.push_back(r); vv.push_back(v); counts[c]++; }
  }
  mat_a.nnz_unpacked_ = (int)rr.size();
  if (mat_a.owns_csr_data()) {
    delete[] mat_a.csr_vals;
    delete[] mat_a.csr_cols;
    delete[] mat_a.csr_rows;
  }
  mat_a.csr_vals = new double[mat_a.nnz_unpacked_];
  mat_a.csr_cols = new int[mat_a.nnz_unpacked_];
  mat_a.csr_rows = new int[mat_a.n_ + 1];
  fill_sorted_csr(mat_a.n_, counts, rr, cc, vv, mat_a.csr_rows, mat_a.csr_cols, mat_a.csr_vals);
  mat_a.nnz_ = mat_a.nnz_unpacked_;
}

void coo_to_csr(MMatrix& mat_a) {
  std::vector<int> counts(mat_a.n_, 0), rr(mat_a.coo_rows, mat_a.coo_rows + mat_a.nnz_),
      cc(mat_a.coo_cols, mat_a.coo_cols + mat_a.nnz_);
  std::vector<double> vv(mat_a.coo_vals, mat_a.coo_vals + mat_a.nnz_);
  for (int i = 0; i < mat_a.nnz_; ++i) counts[rr[i]]++;
  if (mat_a.owns_csr_data()) {
    delete[] mat_a.csr_vals;
    delete[] mat_a.csr_cols;
    delete[] mat_a.csr_rows;
  }
  mat_a.csr_rows = new int[mat_a.n_ + 1];
  mat_a.csr_vals = new double[std::max(mat_a.nnz_, 1)];
  mat_a.csr_cols = new int[std::max(mat_a.nnz_, 1)];
  fill_sorted_csr(mat_a.n_, counts, rr, cc, vv, mat_a.csr_rows, mat_a.csr_cols, mat_a.csr_vals);
  // the reference also leaves the COO arrays in sorted CSR order (input_functions.cpp:167-173)
  for (int i = 0; i < mat_a.n_; ++i)
    for (int p = mat_a.csr_rows[i]; p < mat_a.csr_rows[i + 1]; ++p) mat_a.coo_rows[p] = i;
  std::copy(mat_a.csr_cols, mat_a.csr_cols + mat_a.nnz_, mat_a.coo_cols);
  std::copy(mat_a.csr_vals, mat_a.csr_vals + mat_a.nnz_, mat_a.coo_vals);
}

void read_rhs(const char* rhs_file_name, double* rhs) {
  File file(rhs_file_name);
  std::string line;
  read_line(file.f, line);
  read_line(file.f, line);
  int i = 0;
  while (read_line(file.f, line)) {
    double v;
    if (std::sscanf(line.c_str(), "%lf", &v) != 1) continue;
    rhs[i++] = v;
  }
}

void read_1idx_perm(const char* rhs_file_name, int* rhs) {
  File file(rhs_file_name);
  std::string line;
  read_line(file.f, line);
  read_line(file.f, line);
  int i = 0;
  while (read_line(file.f, line)) {
    int v;
    if (std::sscanf(line.c_str(), "%d", &v) != 1) continue;
    rhs[i++] = v - 1;
  }
}
