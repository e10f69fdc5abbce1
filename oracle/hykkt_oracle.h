/*
 * CPU oracle of the HyKKT KKT solve path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm, used by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the
 * checker.  Nothing in the product (hykkt_gb300/, include/) links, loads or
 * calls it.  Each function cites the reference file:line it restates.
 *
 * Parity pins: the permutation-map known-answer test
 * (examples/perm_driver.cpp:15-108), the Ruiz known answers
 * (examples/Ruiz_driver.cpp:145-182), the Cholesky and Schur-CG known
 * answers on the a200 fixtures (examples/cuSolver_driver_cholesky.cpp:66-75,
 * examples/cuSolver_driver_schur_cg.cpp:145-154) and the end-to-end residual
 * tests on a200/a2000 (examples/CMakeLists.txt:22-86).
 */
#ifndef HYKKT_ORACLE_H
#define HYKKT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Threads used by the factorization, the triangular solves and the CG (the
 * CPU baseline's setting; default 1 = the pinned up-looking checker). */
void oracle_set_threads(int threads);
int oracle_get_threads(void);

/* Matrix-Market input (src/input_functions.cpp:16-217) */
int oracle_mm_header(const char* file, int skip, int* n, int* m, int* nnz);
int oracle_mm_read(const char* file, int skip, int* rows, int* cols, double* vals);
int oracle_coo_to_csr(int n, int nnz, const int* rows, const int* cols, const double* vals, int* rp, int* ci,
                      double* v);
int oracle_sym_coo_count(int nnz, const int* rows, const int* cols);
int oracle_sym_coo_to_csr(int n, int nnz, const int* rows, const int* cols, const double* vals, int* rp, int* ci,
                          double* v);
int oracle_read_rhs(const char* file, double* out, int nmax);

/* Permutation maps (src/permcheck.cu:99-195) */
void oracle_reverse_perm(int n, const int* perm, int* rev);
void oracle_vec_map_rc(int n, const int* rows, const int* cols, const int* perm, const int* rev, int* prows,
                       int* pcols, int* map);
void oracle_vec_map_c(int n, const int* rows, const int* cols, const int* rev, int* pcols, int* map);
void oracle_vec_map_r(int n, const int* rows, const int* cols, const int* perm, int* prows, int* pcols, int* map);

/* Ruiz scaling (src/RuizClass.cpp:54-98, src/matrix_vector_ops.cu:146-266) */
void oracle_ruiz_scale(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v,
                       const int* bt_i, const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1,
                       double* rhs2, double* max_d);

/* Sparse Cholesky of an SPD matrix in the given order (lower triangle read),
 * and solve.  Handle-based. */
typedef struct oracle_chol oracle_chol;
oracle_chol* oracle_chol_factor(int n, const int* rp, const int* ci, const double* v, const int* perm, int* status);
void oracle_chol_solve(const oracle_chol* c, const double* b, double* x);
long oracle_chol_nnz(const oracle_chol* c);
void oracle_chol_free(oracle_chol* c);

/* Schur-complement CG (src/SchurComplementConjugateGradient.cpp:89-194) with
 * the factor c; x holds x0 on entry. Returns the iterations. */
int oracle_schur_cg(const oracle_chol* c, int m, int n, const int* jc_rp, const int* jc_ci, const double* jc_v,
                    const double* b, double* x, int itmax, double tol, double* final_err);

/* The full path (HykktSolver::execute, src/HykktSolver.cpp:240-286). */
typedef struct oracle_result oracle_result;
oracle_result* oracle_solve(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                            const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                            const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                            const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                            const int* perm, int itmax, double tol);
/* With the accuracy controls of the GPU path: CG relative tolerance and
 * iterative refinement on the full KKT system with the same factor, whose
 * corrections run CG to refine_rtol (< 0: rtol). */
oracle_result* oracle_solve_ex(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                               const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                               const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                               const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                               const int* perm, int itmax, double tol, double rtol, int refine_max,
                               double refine_target, double refine_rtol);
/* oracle_solve_ex with delta added to the diagonal of Hgamma before the
 * factorization (add_diag, HykktSolver.cpp:392, whose reference value is 0). */
oracle_result* oracle_solve_reg(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                                const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                                const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                                const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                                const int* perm, int itmax, double tol, double rtol, int refine_max,
                                double refine_target, double refine_rtol, double delta);
long oracle_size(const oracle_result* r, const char* name);
int oracle_get(const oracle_result* r, const char* name, void* out, long n);
double oracle_scalar(const oracle_result* r, const char* name);
void oracle_free(oracle_result* r);

#ifdef __cplusplus
}
#endif
#endif
