// Host matrix container of the drop-in C++ API (same members and methods as
// the reference's MMatrix, src/MMatrix.hpp:3-54): COO arrays filled by the
// Matrix-Market reader, CSR arrays used by HykktSolver.  When owns_csr_data()
// is false the CSR arrays are borrowed from the caller and not freed.
#pragma once

struct MMatrix {
  MMatrix();
  MMatrix(int n, int m, int nnz);
  ~MMatrix();

  void owns_csr_data(bool flag);
  bool owns_csr_data();

  // Allocate COO and CSR arrays for an n x m matrix with nnz entries.
  void populate(int n, int m, int nnz);
  void print_csr();
  void clear();

  int* coo_rows;
  int* coo_cols;
  double* coo_vals;

  int* csr_rows;
  int* csr_cols;
  double* csr_vals;

  int n_;
  int m_;
  int nnz_;
  int nnz_unpacked_;

 private:
  bool owns_csr_data_;
};

// Element-wise copy of the CSR arrays of src into dst (same n, m, nnz);
// used to overwrite a borrowed system in place between execute() calls.
void copy_mmatrix(const MMatrix& src, MMatrix& dst);
void copy_vector(const double* src, double* dst, int n);
