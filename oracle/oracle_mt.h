/*
 * Multithreaded supernodal Cholesky of the CPU baseline (oracle_mt.c) --
 * TEST AND MEASUREMENT INFRASTRUCTURE ONLY.  Input: the lower triangle of
 * the permuted matrix by rows (row k: columns j <= k) and its elimination
 * tree; the factor is computed and applied in the permuted numbering.
 */
#ifndef HYKKT_ORACLE_MT_H
#define HYKKT_ORACLE_MT_H

#include <stdint.h>

typedef struct sn_chol sn_chol;

/* once per pattern: supernodes, row structures, extend-add and assembly maps */
sn_chol* sn_analyze(int n, const int* lrp, const int* lci, const int* parent, int threads);
void sn_retain(sn_chol* c);
void sn_release(sn_chol* c);
int64_t sn_nnz(const sn_chol* c);
/* numeric factor of the values (in lrp/lci order); *bad_col = first column
 * whose pivot is <= 1e-12, or -1.  The caller frees the returned array. */
double* sn_factor(const sn_chol* c, const double* lvals, int* bad_col);
/* y <- (L L^T)^{-1} y, permuted numbering */
void sn_solve(const sn_chol* c, const double* L, double* y);

#endif
