// Matrix-Market readers of the drop-in C++ API, with the reference's exact
// semantics (src/input_functions.hpp, src/input_functions.cpp:16-217):
//   * read_mm_file_into_coo consumes `lines` lines and parses the LAST one of
//     them as "n m nnz"; every following line is "row col value" (1-based).
//   * sym_coo_to_csr expands a lower-triangle (symmetric) COO into a full CSR
//     with sorted columns; coo_to_csr builds a CSR with sorted columns.
//   * read_rhs always skips exactly two header lines, then one value per line.
#pragma once

#include "MMatrix.hpp"

struct indexPlusValue {
  double value;
  int idx;
};

// qsort comparator over indexPlusValue by idx: negative, zero or positive as
// a's idx is below, equal to or above b's (src/input_functions.hpp:10-19).
int indexPlusValue_comp(const void* a, const void* b);

void read_mm_file_into_coo(const char* matrix_file_name, MMatrix& mat_a, int lines);
void sym_coo_to_csr(MMatrix& mat_a);
void coo_to_csr(MMatrix& mat_a);
void read_rhs(const char* rhs_file_name, double* rhs);
void read_1idx_perm(const char* rhs_file_name, int* rhs);
