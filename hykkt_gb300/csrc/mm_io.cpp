// MMatrix and the Matrix-Market readers of the drop-in API.  Same file
// semantics as the reference (src/input_functions.cpp:16-217,
// src/MMatrix.cpp:6-149); lines that do not parse are skipped instead of
// re-using the previous line's numbers, and entries beyond the declared nnz
// are rejected.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <thread>
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

namespace {
// The whole file in memory (NUL-terminated, so strtod stops inside it).
std::string slurp(const char* name) {
  File file(name);
  std::string buf;
  char tmp[1 << 16];
  size_t n;
  while ((n = std::fread(tmp, 1, sizeof(tmp), file.f)) > 0) buf.append(tmp, n);
  return buf;
}

bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// a decimal integer as %d reads it (leading blanks, optional sign)
bool parse_int(const char*& p, const char* e, long& out) {
  while (p < e && is_blank(*p)) ++p;
  bool neg = false;
  if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
  if (p >= e || *p < '0' || *p > '9') return false;
  long v = 0;
  while (p < e && *p >= '0' && *p <= '9') {
    v = v * 10 + (*p++ - '0');
    if (v > 2147483647L) return false;
  }
  out = neg ? -v : v;
  return true;
}

// "row col value" at the start of the line [p, e); the value with strtod,
// which rounds exactly as %lf does
bool parse_entry(const char* p, const char* e, long& r, long& c, double& v) {
  if (!parse_int(p, e, r) || !parse_int(p, e, c)) return false;
  while (p < e && is_blank(*p)) ++p;
  if (p >= e) return false;
  char* end = nullptr;
  v = std::strtod(p, &end);
  return end != p && end <= e;
}

struct Entries {
  std::vector<int> r, c;
  std::vector<double> v;
};

// Parses the lines of [b, e) into `out` (lines that do not hold three
// numbers are skipped, as the reference's reader would not use them).
void parse_range(const char* b, const char* e, Entries& out) {
  const char* p = b;
  while (p < e) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', e - p));
    const char* le = nl ? nl : e;
    long r, c;
    double v;
    if (parse_entry(p, le, r, c, v)) {
      out.r.push_back((int)r);
      out.c.push_back((int)c);
      out.v.push_back(v);
    }
    p = nl ? nl + 1 : e;
  }
}
}  // namespace

// Reads the whole file, then parses its entry lines in parallel: the data is
// cut into one byte range per thread at line boundaries and the ranges'
// entries are concatenated in file order (time-to-first-solve of the large
// workloads is dominated by this parse).
void read_mm_file_into_coo(const char* matrix_file_name, MMatrix& mat_a, int lines) {
  const std::string buf = slurp(matrix_file_name);
  const char* p = buf.data();
  const char* end = p + buf.size();
  const char* line = p;
  const char* line_end = p;
  for (int i = 0; i < lines; ++i) {
    if (p >= end) throw std::runtime_error("read_mm_file_into_coo: file shorter than skip");
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', end - p));
    line = p;
    line_end = nl ? nl : end;
    p = nl ? nl + 1 : end;
  }
  // the last line consumed holds the sizes
  const std::string size_line(line, line_end);
  if (std::sscanf(size_line.c_str(), "%d %d %d", &mat_a.n_, &mat_a.m_, &mat_a.nnz_) != 3)
    throw std::runtime_error("read_mm_file_into_coo: size line not found after skipping lines");
  if (mat_a.n_ < 0 || mat_a.m_ < 0 || mat_a.nnz_ < 0) throw std::runtime_error("read_mm_file_into_coo: negative size");
  const size_t bytes = end - p;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int T = (int)std::max<size_t>(1, std::min<size_t>(std::min(hw, 32u), bytes / (1 << 20)));
  std::vector<const char*> cut(T + 1, end);
  cut[0] = p;
  for (int t = 1; t < T; ++t) {
    const char* q = p + bytes * t / T;
    q = std::max(q, cut[t - 1]);
    const char* nl = q < end ? static_cast<const char*>(std::memchr(q, '\n', end - q)) : nullptr;
    cut[t] = nl ? nl + 1 : end;
  }
  std::vector<Entries> parts(T);
  if (T == 1) {
    parse_range(cut[0], cut[1], parts[0]);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) th.emplace_back([&, t] { parse_range(cut[t], cut[t + 1], parts[t]); });
    for (auto& x : th) x.join();
  }
  size_t total = 0;
  for (const Entries& e : parts) total += e.v.size();
  if (total > (size_t)mat_a.nnz_) throw std::runtime_error("read_mm_file_into_coo: more entries than declared");
  if (total != (size_t)mat_a.nnz_) throw std::runtime_error("read_mm_file_into_coo: fewer entries than declared");
  delete[] mat_a.coo_vals;
  delete[] mat_a.coo_rows;
  delete[] mat_a.coo_cols;
  mat_a.coo_vals = new double[mat_a.nnz_];
  mat_a.coo_rows = new int[mat_a.nnz_];
  mat_a.coo_cols = new int[mat_a.nnz_];
  size_t i = 0;
  for (const Entries& e : parts)
    for (size_t k = 0; k < e.v.size(); ++k, ++i) {
      const int r = e.r[k], c = e.c[k];
      if (r < 1 || r > mat_a.n_ || c < 1 || c > mat_a.m_)
        throw std::runtime_error("read_mm_file_into_coo: index out of range");
      mat_a.coo_rows[i] = r - 1;
      mat_a.coo_cols[i] = c - 1;
      mat_a.coo_vals[i] = e.v[k];
    }
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
  // two header lines, then one value per line (lines without a number are
  // skipped); the whole file is read at once
  const std::string buf = slurp(rhs_file_name);
  const char* p = buf.data();
  const char* end = p + buf.size();
  for (int h = 0; h < 2 && p < end; ++h) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', end - p));
    p = nl ? nl + 1 : end;
  }
  int i = 0;
  while (p < end) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', end - p));
    const char* le = nl ? nl : end;
    const char* q = p;
    while (q < le && is_blank(*q)) ++q;
    if (q < le) {
      char* stop = nullptr;
      const double v = std::strtod(q, &stop);
      if (stop != q && stop <= le) rhs[i++] = v;
    }
    p = nl ? nl + 1 : end;
  }
}

int indexPlusValue_comp(const void* a, const void* b) {
  const int ia = static_cast<const indexPlusValue*>(a)->idx, ib = static_cast<const indexPlusValue*>(b)->idx;
  return (ia > ib) - (ia < ib);
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
