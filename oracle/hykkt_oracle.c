/*
 * CPU oracle of the HyKKT KKT solve path -- TEST INFRASTRUCTURE ONLY
 * (see hykkt_oracle.h).  Compiled with -ffp-contract=off so that every
 * product and sum is rounded separately; the formation steps (H~, Ruiz,
 * Hgamma, r^x) then match the GPU kernels bit for bit, which use the same
 * operation order with __dmul_rn/__dadd_rn.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include "hykkt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "oracle_mt.h"

#define NEW(T, n) ((T*)calloc((size_t)((n) > 0 ? (n) : 1), sizeof(T)))

/* Threads of the factorization, triangular solves and CG vector work.  1
 * (the default) is the pinned checker: the up-looking factorization and
 * serial loops below.  More threads switch to the supernodal factorization
 * of oracle_mt.c and parallel loops with the same mathematics (the CPU
 * baseline's configuration). */
static int g_threads = 1;
void oracle_set_threads(int threads) { g_threads = threads > 1 ? threads : 1; }
int oracle_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------------ */
/* Matrix-Market input: src/input_functions.cpp:16-52 (read_mm_file_into_coo),
 * :54-119 (sym_coo_to_csr), :121-175 (coo_to_csr), :198-217 (read_rhs)    */
/* ------------------------------------------------------------------------ */
static int read_line(FILE* f, char* buf, int cap) {
  int c, k = 0, any = 0;
  while ((c = fgetc(f)) != EOF) {
    any = 1;
    if (c == '\n') break;
    if (k < cap - 1) buf[k++] = (char)c;
  }
  buf[k] = 0;
  return any;
}

int oracle_mm_header(const char* file, int skip, int* n, int* m, int* nnz) {
  FILE* f = fopen(file, "r");
  char buf[1024];
  if (!f) return -1;
  buf[0] = 0;
  for (int i = 0; i < skip; ++i)
    if (!read_line(f, buf, sizeof buf)) { fclose(f); return -2; }
  int ok = sscanf(buf, "%d %d %d", n, m, nnz) == 3;  /* the last consumed line holds the sizes */
  fclose(f);
  return ok ? 0 : -3;
}

int oracle_mm_read(const char* file, int skip, int* rows, int* cols, double* vals) {
  FILE* f = fopen(file, "r");
  char buf[1024];
  int n, m, nnz, i = 0;
  if (!f) return -1;
  for (int k = 0; k < skip; ++k) read_line(f, buf, sizeof buf);
  if (sscanf(buf, "%d %d %d", &n, &m, &nnz) != 3) { fclose(f); return -3; }
  while (read_line(f, buf, sizeof buf)) {
    int r, c;
    double v;
    if (sscanf(buf, "%d %d %lf", &r, &c, &v) != 3) continue;
    if (i >= nnz) { fclose(f); return -4; }
    rows[i] = r - 1;
    cols[i] = c - 1;
    vals[i] = v;
    ++i;
  }
  fclose(f);
  return i == nnz ? 0 : -5;
}

typedef struct { int idx; double val; int ord; } entry_t;
static int cmp_entry(const void* a, const void* b) {
  const entry_t* x = (const entry_t*)a;
  const entry_t* y = (const entry_t*)b;
  if (x->idx != y->idx) return x->idx < y->idx ? -1 : 1;
  return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

static void csr_from_triplets(int n, int cnt, const int* r, const int* c, const double* v, int* rp, int* ci, double* vv) {
  int* next = NEW(int, n);
  entry_t* tmp = NEW(entry_t, cnt);
  memset(rp, 0, sizeof(int) * (n + 1));
  for (int t = 0; t < cnt; ++t) rp[r[t] + 1]++;
  for (int i = 0; i < n; ++i) rp[i + 1] += rp[i];
  for (int i = 0; i < n; ++i) next[i] = rp[i];
  for (int t = 0; t < cnt; ++t) {
    int q = next[r[t]]++;
    tmp[q].idx = c[t];
    tmp[q].val = v[t];
    tmp[q].ord = t;
  }
  for (int i = 0; i < n; ++i) qsort(tmp + rp[i], rp[i + 1] - rp[i], sizeof(entry_t), cmp_entry);
  for (int t = 0; t < cnt; ++t) { ci[t] = tmp[t].idx; vv[t] = tmp[t].val; }
  free(next);
  free(tmp);
}

int oracle_coo_to_csr(int n, int nnz, const int* rows, const int* cols, const double* vals, int* rp, int* ci, double* v) {
  csr_from_triplets(n, nnz, rows, cols, vals, rp, ci, v);
  return 0;
}

int oracle_sym_coo_count(int nnz, const int* rows, const int* cols) {
  int c = 0;
  for (int i = 0; i < nnz; ++i) c += (rows[i] != cols[i]) ? 2 : 1;
  return c;
}

int oracle_sym_coo_to_csr(int n, int nnz, const int* rows, const int* cols, const double* vals, int* rp, int* ci, double* v) {
  int cnt = oracle_sym_coo_count(nnz, rows, cols);
  int* r = NEW(int, cnt);
  int* c = NEW(int, cnt);
  double* x = NEW(double, cnt);
  int k = 0;
  for (int i = 0; i < nnz; ++i) {
    r[k] = rows[i]; c[k] = cols[i]; x[k] = vals[i]; ++k;
    if (rows[i] != cols[i]) { r[k] = cols[i]; c[k] = rows[i]; x[k] = vals[i]; ++k; }
  }
  csr_from_triplets(n, cnt, r, c, x, rp, ci, v);
  free(r); free(c); free(x);
  return cnt;
}

int oracle_read_rhs(const char* file, double* out, int nmax) {
  FILE* f = fopen(file, "r");
  char buf[1024];
  int i = 0;
  if (!f) return -1;
  read_line(f, buf, sizeof buf);  /* exactly two header lines */
  read_line(f, buf, sizeof buf);
  while (read_line(f, buf, sizeof buf)) {
    double v;
    if (sscanf(buf, "%lf", &v) != 1) continue;
    if (i < nmax) out[i] = v;
    ++i;
  }
  fclose(f);
  return i;
}

/* ------------------------------------------------------------------------ */
/* Permutation maps: src/permcheck.cu:78-97 (insertion_sort), :99-124
 * (make_vec_map_c), :126-132 (reverse_perm), :134-160 (make_vec_map_r),
 * :162-195 (make_vec_map_rc)                                               */
/* ------------------------------------------------------------------------ */
static void insertion_sort2(int len, int* key, int* val) {
  for (int i = 1; i < len; ++i) {
    int k = key[i], v = val[i], j = i - 1;
    while (j >= 0 && key[j] > k) { key[j + 1] = key[j]; val[j + 1] = val[j]; --j; }
    key[j + 1] = k;
    val[j + 1] = v;
  }
}

void oracle_reverse_perm(int n, const int* perm, int* rev) {
  for (int i = 0; i < n; ++i) rev[perm[i]] = i;
}

void oracle_vec_map_c(int n, const int* rows, const int* cols, const int* rev, int* pcols, int* map) {
  for (int i = 0; i < n; ++i) {
    int s = rows[i], len = rows[i + 1] - s;
    for (int j = 0; j < len; ++j) { map[s + j] = s + j; pcols[s + j] = rev[cols[s + j]]; }
    insertion_sort2(len, pcols + s, map + s);
  }
}

void oracle_vec_map_r(int n, const int* rows, const int* cols, const int* perm, int* prows, int* pcols, int* map) {
  int count = 0;
  prows[0] = 0;
  for (int i = 0; i < n; ++i) {
    int idx = perm[i], s = rows[idx], len = rows[idx + 1] - s;
    prows[i + 1] = prows[i] + len;
    for (int j = 0; j < len; ++j) { map[count + j] = s + j; pcols[count + j] = cols[s + j]; }
    count += len;
  }
}

void oracle_vec_map_rc(int n, const int* rows, const int* cols, const int* perm, const int* rev, int* prows, int* pcols,
                       int* map) {
  int count = 0;
  prows[0] = 0;
  for (int i = 0; i < n; ++i) {
    int idx = perm[i], s = rows[idx], len = rows[idx + 1] - s;
    prows[i + 1] = prows[i] + len;
    for (int j = 0; j < len; ++j) { map[count + j] = s + j; pcols[count + j] = rev[cols[s + j]]; }
    insertion_sort2(len, pcols + count, map + count);
    count += len;
  }
}

/* ------------------------------------------------------------------------ */
/* Ruiz: RuizClass::ruiz_scale (RuizClass.cpp:54-88) = reset_scaling (max_d =
 * 1, :95-98) then `its` x [adapt_row_max (matrix_vector_ops.cu:218-266);
 * adapt_diag_scale (:146-186)].                                             */
/* ------------------------------------------------------------------------ */
void oracle_ruiz_scale(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v,
                       const int* bt_i, const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1,
                       double* rhs2, double* max_d) {
  double* scale = NEW(double, n + m);
  for (int i = 0; i < n + m; ++i) max_d[i] = 1.0;
  for (int it = 0; it < its; ++it) {
    for (int i = 0; i < n + m; ++i) {  /* adapt_row_max */
      double max_l = 0, max_u = 0, e;
      if (i < n) {
        for (int j = a_i[i]; j < a_i[i + 1]; ++j) { e = fabs(a_v[j]); if (e > max_l) max_l = e; }
        for (int j = bt_i[i]; j < bt_i[i + 1]; ++j) { e = fabs(bt_v[j]); if (e > max_u) max_u = e; }
        scale[i] = (max_l > max_u) ? 1.0 / sqrt(max_l) : 1.0 / sqrt(max_u);
      } else {
        for (int j = b_i[i - n]; j < b_i[i - n + 1]; ++j) { e = fabs(b_v[j]); if (e > max_l) max_l = e; }
        scale[i] = 1.0 / sqrt(max_l);
      }
    }
    for (int i = 0; i < n + m; ++i) {  /* adapt_diag_scale */
      if (i < n) {
        for (int j = a_i[i]; j < a_i[i + 1]; ++j) a_v[j] *= scale[i] * scale[a_j[j]];
        rhs1[i] *= scale[i];
        max_d[i] *= scale[i];
        for (int j = bt_i[i]; j < bt_i[i + 1]; ++j) bt_v[j] *= scale[i] * scale[n + bt_j[j]];
      } else {
        for (int j = b_i[i - n]; j < b_i[i - n + 1]; ++j) b_v[j] *= scale[i] * scale[b_j[j]];
        rhs2[i - n] *= scale[i];
        max_d[i] *= scale[i];
      }
    }
  }
  free(scale);
}

/* ------------------------------------------------------------------------ */
/* Sparse Cholesky (replaces cusolverSpDcsrchol*, CholeskyClass.cpp:31-101).
 * Up-looking: row k of L from a sparse triangular solve over the row
 * subtree of the elimination tree (Davis, "Direct Methods for Sparse Linear
 * Systems", SIAM 2006, ch. 4).  Reads the lower triangle of P A P^T.        */
/* ------------------------------------------------------------------------ */
struct oracle_chol {
  int n;
  int* perm;    /* perm[new] = old */
  int* rev;
  int* parent;  /* etree of P A P^T */
  int* cp;      /* L by columns, diagonal first, rows ascending */
  int* ri;
  double* lv;
  sn_chol* sn;  /* multithreaded supernodal factor (oracle_set_threads > 1), else NULL */
  double* snL;
  int threads;
};

/* lower triangle of P A P^T by rows: for permuted row k, the permuted
 * columns j <= k (upper entries of A are ignored) */
static void permuted_lower_rows(int n, const int* rp, const int* ci, const double* v, const int* rev, int** orp,
                                int** oci, double** ov) {
  int* cnt = NEW(int, n + 1);
  for (int i = 0; i < n; ++i)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      int j = ci[p];
      if (j > i) continue;
      int a = rev[i], b = rev[j];
      int row = a > b ? a : b;
      cnt[row + 1]++;
    }
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  int* nx = NEW(int, n);
  for (int i = 0; i < n; ++i) nx[i] = cnt[i];
  int* c = NEW(int, cnt[n]);
  double* x = NEW(double, cnt[n]);
  for (int i = 0; i < n; ++i)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      int j = ci[p];
      if (j > i) continue;
      int a = rev[i], b = rev[j];
      int row = a > b ? a : b, col = a > b ? b : a;
      int q = nx[row]++;
      c[q] = col;
      x[q] = v[p];
    }
  free(nx);
  *orp = cnt;
  *oci = c;
  *ov = x;
}

static void etree_rows(int n, const int* lrp, const int* lci, int* parent) {
  int* anc = NEW(int, n);
  for (int k = 0; k < n; ++k) {
    parent[k] = -1;
    anc[k] = -1;
    for (int p = lrp[k]; p < lrp[k + 1]; ++p) {
      int i = lci[p];
      while (i != -1 && i < k) {
        int nxt = anc[i];
        anc[i] = k;
        if (nxt == -1) parent[i] = k;
        i = nxt;
      }
    }
  }
  free(anc);
}

/* row subtree of row k: columns j < k with L(k,j) != 0, in topological
 * order in s[top..n-1] */
static int ereach(int k, const int* lrp, const int* lci, const int* parent, int* s, int* w, int n) {
  int top = n;
  w[k] = k;
  for (int p = lrp[k]; p < lrp[k + 1]; ++p) {
    int i = lci[p];
    if (i >= k) continue;
    int len = 0;
    for (; w[i] != k; i = parent[i]) {
      s[len++] = i;
      w[i] = k;
    }
    while (len > 0) s[--top] = s[--len];
  }
  return top;
}

/* the supernodal analysis of the last pattern (and ordering) factorized
 * with threads, reused while the lower pattern is the same: the analysis is
 * once-per-pattern work, as in the reference's first execute() */
static struct {
  pthread_mutex_t mu;
  uint64_t key;
  int threads;
  sn_chol* sym;
} g_sn_cache = {PTHREAD_MUTEX_INITIALIZER, 0, 0, NULL};

static uint64_t pattern_key(int n, const int* lrp, const int* lci) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)n;
  for (int i = 0; i <= n; ++i) h = (h ^ (uint64_t)(uint32_t)lrp[i]) * 1099511628211ull;
  for (int p = 0; p < lrp[n]; ++p) h = (h ^ (uint64_t)(uint32_t)lci[p]) * 1099511628211ull;
  return h;
}

static sn_chol* cached_analysis(int n, const int* lrp, const int* lci, const int* parent, int threads) {
  const uint64_t key = pattern_key(n, lrp, lci);
  pthread_mutex_lock(&g_sn_cache.mu);
  if (!g_sn_cache.sym || g_sn_cache.key != key || g_sn_cache.threads != threads) {
    if (g_sn_cache.sym) sn_release(g_sn_cache.sym);
    g_sn_cache.sym = sn_analyze(n, lrp, lci, parent, threads);
    g_sn_cache.key = key;
    g_sn_cache.threads = threads;
  }
  sn_chol* s = g_sn_cache.sym;
  sn_retain(s);
  pthread_mutex_unlock(&g_sn_cache.mu);
  return s;
}

oracle_chol* oracle_chol_factor(int n, const int* rp, const int* ci, const double* v, const int* perm, int* status) {
  oracle_chol* c = (oracle_chol*)calloc(1, sizeof(oracle_chol));
  c->n = n;
  c->perm = NEW(int, n);
  c->rev = NEW(int, n);
  for (int i = 0; i < n; ++i) c->perm[i] = perm ? perm[i] : i;
  oracle_reverse_perm(n, c->perm, c->rev);
  int *lrp, *lci;
  double* lvv;
  permuted_lower_rows(n, rp, ci, v, c->rev, &lrp, &lci, &lvv);
  c->parent = NEW(int, n);
  etree_rows(n, lrp, lci, c->parent);
  if (g_threads > 1) {
    c->threads = g_threads;
    c->sn = cached_analysis(n, lrp, lci, c->parent, g_threads);
    int bad = -1;
    c->snL = sn_factor(c->sn, lvv, &bad);
    *status = bad;
    c->cp = NEW(int, n + 1);  /* no flat factor in this mode */
    free(lrp); free(lci); free(lvv);
    return c;
  }
  int* s = NEW(int, n);
  int* w = NEW(int, n);
  int* cnt = NEW(int, n);
  for (int k = 0; k < n; ++k) w[k] = -1;
  for (int k = 0; k < n; ++k) {
    cnt[k]++;
    int top = ereach(k, lrp, lci, c->parent, s, w, n);
    for (int t = top; t < n; ++t) cnt[s[t]]++;
  }
  c->cp = NEW(int, n + 1);
  for (int k = 0; k < n; ++k) c->cp[k + 1] = c->cp[k] + cnt[k];
  long nnz = c->cp[n];
  c->ri = NEW(int, nnz);
  c->lv = NEW(double, nnz);
  int* fill = NEW(int, n);  /* next free slot per column */
  double* x = NEW(double, n);
  for (int k = 0; k < n; ++k) w[k] = -1;
  *status = -1;
  for (int k = 0; k < n; ++k) {
    int top = ereach(k, lrp, lci, c->parent, s, w, n);
    x[k] = 0;
    for (int p = lrp[k]; p < lrp[k + 1]; ++p) x[lci[p]] += lvv[p];
    double d = x[k];
    x[k] = 0;
    for (int t = top; t < n; ++t) {
      int j = s[t];
      double lkj = x[j] / c->lv[c->cp[j]];
      x[j] = 0;
      for (int p = c->cp[j] + 1; p < c->cp[j] + fill[j]; ++p) x[c->ri[p]] -= c->lv[p] * lkj;
      d -= lkj * lkj;
      int q = c->cp[j] + fill[j]++;
      c->ri[q] = k;
      c->lv[q] = lkj;
    }
    if (!(d > 1e-24) && *status < 0) *status = k;  /* pivot sqrt(d) <= 1e-12 */
    int q = c->cp[k] + fill[k]++;
    c->ri[q] = k;
    c->lv[q] = sqrt(d);
  }
  free(fill); free(x); free(s); free(w); free(cnt); free(lrp); free(lci); free(lvv);
  return c;
}

long oracle_chol_nnz(const oracle_chol* c) { return c->sn ? (long)sn_nnz(c->sn) : c->cp[c->n]; }

/* x = A^{-1} b in the original numbering */
void oracle_chol_solve(const oracle_chol* c, const double* b, double* x) {
  int n = c->n;
  double* y = NEW(double, n);
  for (int i = 0; i < n; ++i) y[i] = b[c->perm[i]];
  if (c->sn) {
    sn_solve(c->sn, c->snL, y);
    for (int i = 0; i < n; ++i) x[c->perm[i]] = y[i];
    free(y);
    return;
  }
  for (int j = 0; j < n; ++j) {  /* L y = b */
    y[j] /= c->lv[c->cp[j]];
    for (int p = c->cp[j] + 1; p < c->cp[j + 1]; ++p) y[c->ri[p]] -= c->lv[p] * y[j];
  }
  for (int j = n - 1; j >= 0; --j) {  /* L^T x = y */
    double t = y[j];
    for (int p = c->cp[j] + 1; p < c->cp[j + 1]; ++p) t -= c->lv[p] * y[c->ri[p]];
    y[j] = t / c->lv[c->cp[j]];
  }
  for (int i = 0; i < n; ++i) x[c->perm[i]] = y[i];
  free(y);
}

void oracle_chol_free(oracle_chol* c) {
  if (!c) return;
  free(c->perm); free(c->rev); free(c->parent); free(c->cp); free(c->ri); free(c->lv);
  free(c->snL);
  sn_release(c->sn);
  free(c);
}

/* ------------------------------------------------------------------------ */
/* Schur-complement CG: SchurComplementConjugateGradient::setup + solve
 * (SchurComplementConjugateGradient.cpp:89-194), S = Jc A^{-1} Jc^T.       */
/* ------------------------------------------------------------------------ */
static double dot(int n, const double* a, const double* b) {
  double s = 0;
  if (g_threads > 1) {
    /* fixed chunks, partial sums added in chunk order: repeatable */
    enum { CH = 64 };
    double part[CH];
    const int per = (n + CH - 1) / CH;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < CH; ++t) {
      double q = 0;
      const int e = (t + 1) * per < n ? (t + 1) * per : n;
      for (int i = t * per; i < e; ++i) q += a[i] * b[i];
      part[t] = q;
    }
    for (int t = 0; t < CH; ++t) s += part[t];
    return s;
  }
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
static void spmv(int m, const int* rp, const int* ci, const double* v, const double* x, double* y) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
  for (int k = 0; k < m; ++k) {
    double s = 0;
    for (int p = rp[k]; p < rp[k + 1]; ++p) s += v[p] * x[ci[p]];
    y[k] = s;
  }
}
static void spmv_t(int m, int n, const int* rp, const int* ci, const double* v, const double* x, double* y) {
  for (int i = 0; i < n; ++i) y[i] = 0;
  for (int k = 0; k < m; ++k)
    for (int p = rp[k]; p < rp[k + 1]; ++p) y[ci[p]] += v[p] * x[k];
}

/* Jc^T x as rows of the transpose (each output summed over k ascending,
 * the order of spmv_t); threads when set */
typedef struct { const int *rp, *ci; const double* v; } csr_view;
static void spmv_tt(const csr_view* T, int m, int n, const int* rp, const int* ci, const double* v, const double* x,
                    double* y) {
  if (!T || g_threads <= 1) {
    spmv_t(m, n, rp, ci, v, x, y);
    return;
  }
  spmv(n, T->rp, T->ci, T->v, x, y);
}

static int schur_cg_rel(const oracle_chol* c, int m, int n, const int* jc_rp, const int* jc_ci, const double* jc_v,
                        const csr_view* jct, const double* b, double* x, int itmax, double tol, double rtol,
                        double* final_err);

int oracle_schur_cg(const oracle_chol* c, int m, int n, const int* jc_rp, const int* jc_ci, const double* jc_v,
                    const double* b, double* x, int itmax, double tol, double* final_err) {
  return schur_cg_rel(c, m, n, jc_rp, jc_ci, jc_v, NULL, b, x, itmax, tol, 0.0, final_err);
}

/* Stops when sqrt(r.r) < rtol * ||r0|| (rtol > 0), else when sqrt(r.r) < tol,
 * the reference's absolute test (SchurCG.cpp:156). */
static int schur_cg_rel(const oracle_chol* c, int m, int n, const int* jc_rp, const int* jc_ci, const double* jc_v,
                        const csr_view* jct, const double* b, double* x, int itmax, double tol, double rtol,
                        double* final_err) {
  double* yv = NEW(double, n);
  double* z = NEW(double, n);
  double* r = NEW(double, m);
  double* w = NEW(double, m);
  double* p = NEW(double, m);
  double* s = NEW(double, m);
  double* t = NEW(double, m);
  for (int k = 0; k < m; ++k) { r[k] = b[k]; w[k] = b[k]; p[k] = b[k]; s[k] = b[k]; }
  double beta = 0, gam, gam1 = 0, delta, alpha;
  spmv_tt(jct, m, n, jc_rp, jc_ci, jc_v, x, yv);  /* y = Jc^T x0 */
  oracle_chol_solve(c, yv, z);
  spmv(m, jc_rp, jc_ci, jc_v, z, t);
  for (int k = 0; k < m; ++k) r[k] -= t[k];  /* r = b - S x0 */
  gam = dot(m, r, r);
  const double thr = rtol > 0.0 ? rtol * sqrt(gam) : tol;
  spmv_tt(jct, m, n, jc_rp, jc_ci, jc_v, r, yv);
  oracle_chol_solve(c, yv, z);
  spmv(m, jc_rp, jc_ci, jc_v, z, w);  /* w = S r */
  delta = dot(m, w, r);
  alpha = gam / delta;
  int i;
  for (i = 0; i < itmax; ++i) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int k = 0; k < m; ++k) {
      p[k] = beta * p[k] + r[k];
      s[k] = beta * s[k] + w[k];
      x[k] += alpha * p[k];
      r[k] -= alpha * s[k];
    }
    gam1 = dot(m, r, r);
    if (sqrt(gam1) < thr) break;
    spmv_tt(jct, m, n, jc_rp, jc_ci, jc_v, r, yv);
    oracle_chol_solve(c, yv, z);
    spmv(m, jc_rp, jc_ci, jc_v, z, w);
    delta = dot(m, w, r);
    beta = gam1 / gam;
    gam = gam1;
    alpha = gam / (delta - beta * gam / alpha);
  }
  if (final_err) *final_err = sqrt(gam1);
  free(yv); free(z); free(r); free(w); free(p); free(s); free(t);
  return i < itmax ? i + 1 : itmax;
}

/* ------------------------------------------------------------------------ */
/* The full path                                                            */
/* ------------------------------------------------------------------------ */
struct oracle_result {
  int n_x, m_c, m_d;
  int *ht_rp, *ht_ci, *hg_rp, *hg_ci, *parent, *L_cp, *L_ri, *perm;
  double *ht_v0, *ht_v, *jc_s, *ry_s, *rxt, *max_d, *hg_v, *rhat, *rxp, *hrxp, *schur, *L_v;
  double *x, *s, *y, *yd;
  long nnz_ht, nnz_hg, nnz_L;
  double rel_res_ref, rel_res_full, cg_err, cg_iters, pivot_col;
  double rel_res_first, cg_iters_total, refine_steps;
  double t_setup, t_cg;  /* seconds: everything before the first CG; all CG iterations */
};

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* sorted union of row i of base and of B^T B (k ascending), with the
 * values base + sum_k (B[k,i]*B[k,j]) * wk[k] (wk NULL: weight 1), and then
 * scaled: out = base + g * acc. */
static void product_union(int n, const int* brp, const int* bci, const double* bv, int mb, const int* Brp,
                          const int* Bci, const double* Bv, const int* BTrp, const int* BTci, const double* BTv,
                          const double* wk, double g, int use_g, int** orp, int** oci, double** ov) {
  (void)mb;
  int* mark = NEW(int, n);
  int* list = NEW(int, n);
  double* base = NEW(double, n);
  double* acc = NEW(double, n);
  for (int j = 0; j < n; ++j) mark[j] = -1;
  int cap = brp[n] + 16;
  int* rp = NEW(int, n + 1);
  int* ci = NEW(int, cap);
  double* v = NEW(double, cap);
  int nnz = 0;
  for (int i = 0; i < n; ++i) {
    int len = 0;
    for (int p = brp[i]; p < brp[i + 1]; ++p) {
      int j = bci[p];
      if (mark[j] != i) { mark[j] = i; list[len++] = j; base[j] = 0; acc[j] = 0; }
      base[j] = bv[p];
    }
    if (BTrp)
      for (int q = BTrp[i]; q < BTrp[i + 1]; ++q) {
        int k = BTci[q];
        double bki = BTv[q];
        for (int p = Brp[k]; p < Brp[k + 1]; ++p) {
          int j = Bci[p];
          if (mark[j] != i) { mark[j] = i; list[len++] = j; base[j] = 0; acc[j] = 0; }
          double term = bki * Bv[p];
          if (wk) term = term * wk[k];
          acc[j] = acc[j] + term;
        }
      }
    /* sort the row's columns */
    for (int a = 1; a < len; ++a) {
      int key = list[a], b = a - 1;
      while (b >= 0 && list[b] > key) { list[b + 1] = list[b]; --b; }
      list[b + 1] = key;
    }
    if (nnz + len > cap) {
      cap = 2 * (nnz + len);
      ci = (int*)realloc(ci, sizeof(int) * cap);
      v = (double*)realloc(v, sizeof(double) * cap);
    }
    for (int a = 0; a < len; ++a) {
      int j = list[a];
      ci[nnz] = j;
      v[nnz] = use_g ? base[j] + g * acc[j] : base[j] + acc[j];
      ++nnz;
    }
    rp[i + 1] = nnz;
  }
  free(mark); free(list); free(base); free(acc);
  *orp = rp;
  *oci = ci;
  *ov = v;
}

static void transpose_vals(int m, int n, const int* rp, const int* ci, const double* v, int** trp, int** tci,
                           double** tv) {
  int nnz = rp[m];
  int* r = NEW(int, n + 1);
  int* c = NEW(int, nnz);
  double* x = NEW(double, nnz);
  for (int p = 0; p < nnz; ++p) r[ci[p] + 1]++;
  for (int j = 0; j < n; ++j) r[j + 1] += r[j];
  int* nx = NEW(int, n);
  for (int j = 0; j < n; ++j) nx[j] = r[j];
  for (int k = 0; k < m; ++k)
    for (int p = rp[k]; p < rp[k + 1]; ++p) {
      int q = nx[ci[p]]++;
      c[q] = k;
      x[q] = v[p];
    }
  free(nx);
  *trp = r;
  *tci = c;
  *tv = x;
}

static double* dup(const double* a, long n) {
  double* b = NEW(double, n);
  if (a) memcpy(b, a, sizeof(double) * (n > 0 ? n : 0));
  return b;
}

/* The 4x4 KKT system in the original numbering, for residuals. */
typedef struct {
  int n, m_c, m_d, jd_flag;
  const int *h_rp, *h_ci;
  const double *h_v, *ds_v;
  const int *jc_rp, *jc_ci;
  const double* jc_v;
  const int *jd_rp, *jd_ci;
  const double* jd_v;
  const double *rx, *rs, *ry, *ryd;
} kkt_t;

/* residual blocks e = b - K z and the relative norms of rows {1,3} (the
 * reference's check_error, HykktSolver.cpp:846-930) and of all four rows */
/* (s, c) += a*b with the product's error (fma) and the sum's error (two-sum)
 * carried in c: the residual is accumulated as in twice the working
 * precision (Ogita, Rump, Oishi, SIAM J. Sci. Comput. 26, 2005), so that
 * refinement is not stopped by cancellation among large terms.  Compiled
 * with -ffp-contract=off, so a*b below is the rounded product. */
static inline void acc2(double* s, double* c, double a, double b) {
  const double p = a * b;
  const double pe = fma(a, b, -p);
  const double t = *s + p;
  const double z = t - *s;
  const double e = (*s - (t - z)) + (p - z);
  *s = t;
  *c += e + pe;
}

/* 4-block residual of the KKT system (the reference checks rows 1 and 3,
 * HykktSolver.cpp:845-930; the full check adds rows 2 and 4). */
static void kkt_residual(const kkt_t* K, const double* x, const double* s, const double* y, const double* yd,
                         double* e1, double* e2, double* e3, double* e4, double* rel_ref, double* rel_full) {
  double nb = 0, r1 = 0, r2 = 0, r3 = 0, r4 = 0;
  for (int i = 0; i < K->n; ++i) nb += K->rx[i] * K->rx[i];
  for (int k = 0; k < K->m_d; ++k) nb += K->rs[k] * K->rs[k] + K->ryd[k] * K->ryd[k];
  for (int k = 0; k < K->m_c; ++k) nb += K->ry[k] * K->ry[k];
  double* c1 = (double*)calloc(K->n > 0 ? K->n : 1, sizeof(double));
  for (int i = 0; i < K->n; ++i) {
    e1[i] = K->rx[i];
    for (int p = K->h_rp[i]; p < K->h_rp[i + 1]; ++p) acc2(&e1[i], &c1[i], -K->h_v[p], x[K->h_ci[p]]);
  }
  if (K->jd_flag)
    for (int k = 0; k < K->m_d; ++k)
      for (int p = K->jd_rp[k]; p < K->jd_rp[k + 1]; ++p) acc2(&e1[K->jd_ci[p]], &c1[K->jd_ci[p]], -K->jd_v[p], yd[k]);
  for (int k = 0; k < K->m_c; ++k)
    for (int p = K->jc_rp[k]; p < K->jc_rp[k + 1]; ++p) acc2(&e1[K->jc_ci[p]], &c1[K->jc_ci[p]], -K->jc_v[p], y[k]);
  for (int i = 0; i < K->n; ++i) {
    e1[i] += c1[i];
    r1 += e1[i] * e1[i];
  }
  free(c1);
  for (int k = 0; k < K->m_c; ++k) {
    double sv = K->ry[k], c = 0;
    for (int p = K->jc_rp[k]; p < K->jc_rp[k + 1]; ++p) acc2(&sv, &c, -K->jc_v[p], x[K->jc_ci[p]]);
    e3[k] = sv + c;
    r3 += e3[k] * e3[k];
  }
  for (int k = 0; k < K->m_d; ++k) {
    double s2 = K->rs[k], c2 = 0;
    acc2(&s2, &c2, -K->ds_v[k], s[k]);
    acc2(&s2, &c2, yd[k], 1.0);
    e2[k] = s2 + c2;
    double s4 = K->ryd[k], c4 = 0;
    if (K->jd_flag)
      for (int p = K->jd_rp[k]; p < K->jd_rp[k + 1]; ++p) acc2(&s4, &c4, -K->jd_v[p], x[K->jd_ci[p]]);
    acc2(&s4, &c4, s[k], 1.0);
    e4[k] = s4 + c4;
    r2 += e2[k] * e2[k];
    r4 += e4[k] * e4[k];
  }
  *rel_ref = sqrt(r1 + r3) / sqrt(nb);
  *rel_full = sqrt(r1 + r2 + r3 + r4) / sqrt(nb);
}

oracle_result* oracle_solve(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                            const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                            const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                            const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                            const int* perm, int itmax, double tol) {
  return oracle_solve_ex(n_x, m_c, m_d, h_rp, h_ci, h_v, ds_v, jc_rp, jc_ci, jc_v, jd_rp, jd_ci, jd_v, nnz_jd, rx, rs,
                         ry, ryd, y0, gamma, perm, itmax, tol, 0.0, 0, 0.0, -1.0);
}

oracle_result* oracle_solve_ex(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                               const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                               const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                               const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                               const int* perm, int itmax, double tol, double rtol, int refine_max,
                               double refine_target, double refine_rtol) {
  return oracle_solve_reg(n_x, m_c, m_d, h_rp, h_ci, h_v, ds_v, jc_rp, jc_ci, jc_v, jd_rp, jd_ci, jd_v, nnz_jd, rx, rs,
                          ry, ryd, y0, gamma, perm, itmax, tol, rtol, refine_max, refine_target, refine_rtol, 0.0);
}

oracle_result* oracle_solve_reg(int n_x, int m_c, int m_d, const int* h_rp, const int* h_ci, const double* h_v,
                                const double* ds_v, const int* jc_rp, const int* jc_ci, const double* jc_v,
                                const int* jd_rp, const int* jd_ci, const double* jd_v, int nnz_jd, const double* rx,
                                const double* rs, const double* ry, const double* ryd, const double* y0, double gamma,
                                const int* perm, int itmax, double tol, double rtol, int refine_max,
                                double refine_target, double refine_rtol, double delta) {
  oracle_result* R = (oracle_result*)calloc(1, sizeof(oracle_result));
  if (refine_rtol < 0) refine_rtol = rtol;
  const double t0 = now_s();
  const int n = n_x;
  R->n_x = n_x;
  R->m_c = m_c;
  R->m_d = m_d;
  const int jd_flag = nnz_jd > 0;
  /* --- compute_spgemm_htil (HykktSolver.cpp:289-337) --- */
  int *jdt_rp = NULL, *jdt_ci = NULL;
  double* jdt_v = NULL;
  R->rxt = NEW(double, n);
  if (jd_flag) {
    transpose_vals(m_d, n, jd_rp, jd_ci, jd_v, &jdt_rp, &jdt_ci, &jdt_v);
    double* ryd_s = NEW(double, m_d);
    for (int k = 0; k < m_d; ++k) ryd_s[k] = ryd[k] * ds_v[k] + rs[k];  /* row_scale then add_vecs */
    for (int i = 0; i < n; ++i) {
      double acc = 0;
      for (int q = jdt_rp[i]; q < jdt_rp[i + 1]; ++q) acc = acc + jdt_v[q] * ryd_s[jdt_ci[q]];
      R->rxt[i] = rx[i] + acc;
    }
    free(ryd_s);
    product_union(n, h_rp, h_ci, h_v, m_d, jd_rp, jd_ci, jd_v, jdt_rp, jdt_ci, jdt_v, ds_v, 0, 0, &R->ht_rp,
                  &R->ht_ci, &R->ht_v);
  } else {
    for (int i = 0; i < n; ++i) R->rxt[i] = rx[i];
    product_union(n, h_rp, h_ci, h_v, 0, NULL, NULL, NULL, NULL, NULL, NULL, NULL, 0, 0, &R->ht_rp, &R->ht_ci,
                  &R->ht_v);
  }
  R->nnz_ht = R->ht_rp[n];
  R->ht_v0 = dup(R->ht_v, R->nnz_ht);
  /* --- compute_ruiz_scaling (HykktSolver.cpp:340-349) on [H~ Jc^T; Jc 0] --- */
  const int nnz_jc = jc_rp[m_c];
  R->jc_s = dup(jc_v, nnz_jc);
  R->ry_s = dup(ry, m_c);
  R->max_d = NEW(double, n + m_c);
  int *jct_rp, *jct_ci;
  double* jct_v;
  transpose_vals(m_c, n, jc_rp, jc_ci, R->jc_s, &jct_rp, &jct_ci, &jct_v);
  oracle_ruiz_scale(2, n, m_c, R->ht_v, R->ht_rp, R->ht_ci, jct_v, jct_rp, jct_ci, R->jc_s, jc_rp, jc_ci, R->rxt,
                    R->ry_s, R->max_d);
  /* --- compute_spgemm_hgamma (HykktSolver.cpp:370-383) --- */
  product_union(n, R->ht_rp, R->ht_ci, R->ht_v, m_c, jc_rp, jc_ci, R->jc_s, jct_rp, jct_ci, jct_v, NULL, gamma, 1,
                &R->hg_rp, &R->hg_ci, &R->hg_v);
  R->nnz_hg = R->hg_rp[n];
  R->rhat = NEW(double, n);
  for (int i = 0; i < n; ++i) {
    double acc = 0;
    for (int q = jct_rp[i]; q < jct_rp[i + 1]; ++q) acc = acc + jct_v[q] * R->ry_s[jct_ci[q]];
    R->rhat[i] = R->rxt[i] + gamma * acc;
  }
  /* --- setup_permutation / apply_permutation (HykktSolver.cpp:386-395, 760-798) --- */
  R->perm = NEW(int, n);
  for (int i = 0; i < n; ++i) R->perm[i] = perm ? perm[i] : i;
  int* rev = NEW(int, n);
  oracle_reverse_perm(n, R->perm, rev);
  R->rxp = NEW(double, n);
  for (int i = 0; i < n; ++i) R->rxp[i] = R->rhat[R->perm[i]];
  /* --- add_diag (HykktSolver.cpp:392; matrix_vector_ops.cu:344-358): delta
   *     added to the diagonal entries present in the pattern, none inserted
   *     (the reference passes 0; delta != 0 is the regularized H_delta) --- */
  if (delta != 0.0)
    for (int i = 0; i < n; ++i)
      for (int q = R->hg_rp[i]; q < R->hg_rp[i + 1]; ++q)
        if (R->hg_ci[q] == i) {
          R->hg_v[q] += delta;
          break;
        }
  /* --- compute_hgamma_factorization (HykktSolver.cpp:398-401) --- */
  int st;
  oracle_chol* C = oracle_chol_factor(n, R->hg_rp, R->hg_ci, R->hg_v, R->perm, &st);
  R->pivot_col = st;
  R->parent = NEW(int, n);
  memcpy(R->parent, C->parent, sizeof(int) * n);
  R->nnz_L = C->sn ? 0 : C->cp[n];  /* the flat factor exists in the one-thread mode only */
  R->L_cp = NEW(int, n + 1);
  memcpy(R->L_cp, C->cp, sizeof(int) * (n + 1));
  R->L_ri = NEW(int, R->nnz_L);
  if (R->nnz_L) memcpy(R->L_ri, C->ri, sizeof(int) * R->nnz_L);
  R->L_v = dup(C->lv, R->nnz_L);
  /* --- setup_conjugate_gradient (HykktSolver.cpp:814-843): hrxp = Hg_p^{-1} rxp,
   *     schur = Jc_p hrxp - ry.  Done in the original numbering. --- */
  double* rhs_o = NEW(double, n);
  double* sol_o = NEW(double, n);
  memcpy(rhs_o, R->rhat, sizeof(double) * n);
  oracle_chol_solve(C, rhs_o, sol_o);
  R->hrxp = NEW(double, n);
  for (int i = 0; i < n; ++i) R->hrxp[i] = sol_o[R->perm[i]];
  R->schur = NEW(double, m_c);
  spmv(m_c, jc_rp, jc_ci, R->jc_s, sol_o, R->schur);
  for (int k = 0; k < m_c; ++k) R->schur[k] = R->schur[k] - R->ry_s[k];
  /* --- compute_conjugate_gradient (HykktSolver.cpp:404-407) --- */
  R->y = NEW(double, m_c);
  for (int k = 0; k < m_c; ++k) R->y[k] = y0 ? y0[k] : 0.0;
  double err = 0;
  const double t1 = now_s();
  R->t_setup = t1 - t0;
  const csr_view jct_view = {jct_rp, jct_ci, jct_v};
  int its = m_c > 0 ? schur_cg_rel(C, m_c, n, jc_rp, jc_ci, R->jc_s, &jct_view, R->schur, R->y, itmax, tol, rtol, &err)
                    : 0;
  R->t_cg = now_s() - t1;
  R->cg_iters = its;
  R->cg_err = err;
  /* --- recover_solution (HykktSolver.cpp:410-457) --- */
  double* t = NEW(double, n);
  spmv_t(m_c, n, jc_rp, jc_ci, R->jc_s, R->y, t);
  for (int i = 0; i < n; ++i) rhs_o[i] = R->rhat[i] - t[i];
  R->x = NEW(double, n);
  oracle_chol_solve(C, rhs_o, R->x);
  for (int i = 0; i < n; ++i) R->x[i] *= R->max_d[i];
  for (int k = 0; k < m_c; ++k) R->y[k] *= R->max_d[n + k];
  R->s = NEW(double, m_d);
  R->yd = NEW(double, m_d);
  for (int k = 0; k < m_d; ++k) {
    double jx = 0;
    if (jd_flag)
      for (int p = jd_rp[k]; p < jd_rp[k + 1]; ++p) jx += jd_v[p] * R->x[jd_ci[p]];
    R->s[k] = jd_flag ? jx - ryd[k] : -ryd[k];
    R->yd[k] = R->s[k] * ds_v[k] - rs[k];
  }
  /* --- check_error (HykktSolver.cpp:846-930) and the two rows it assumes 0 --- */
  kkt_t K = {n, m_c, m_d, jd_flag, h_rp, h_ci, h_v, ds_v, jc_rp, jc_ci, jc_v, jd_rp, jd_ci, jd_v, rx, rs, ry, ryd};
  double* e1 = NEW(double, n);
  double* e2 = NEW(double, m_d);
  double* e3 = NEW(double, m_c);
  double* e4 = NEW(double, m_d);
  kkt_residual(&K, R->x, R->s, R->y, R->yd, e1, e2, e3, e4, &R->rel_res_ref, &R->rel_res_full);
  R->rel_res_first = R->rel_res_full;
  /* --- iterative refinement on the full KKT system (an addition; the
   *     reference stops here): correction with the residual as right-hand
   *     side through the same scaling, factor and CG --- */
  double* dx = NEW(double, n);
  double* dy = NEW(double, m_c);
  double* rxc = NEW(double, n);
  double* ryc = NEW(double, m_c);
  int total_its = its;
  R->refine_steps = 0;
  double res_prev = R->rel_res_full;
  /* continue while above the target and the last step at least halved the
   * residual (the GPU path's rule) */
  for (int step = 0; step < refine_max && R->rel_res_full > refine_target &&
                     (step == 0 || R->rel_res_full < 0.5 * res_prev);
       ++step) {
    res_prev = R->rel_res_full;
    for (int i = 0; i < n; ++i) {
      double acc = 0;
      if (jd_flag)
        for (int q = jdt_rp[i]; q < jdt_rp[i + 1]; ++q) acc += jdt_v[q] * (e4[jdt_ci[q]] * ds_v[jdt_ci[q]] + e2[jdt_ci[q]]);
      rxc[i] = (e1[i] + acc) * R->max_d[i];
    }
    for (int k = 0; k < m_c; ++k) ryc[k] = e3[k] * R->max_d[n + k];
    for (int i = 0; i < n; ++i) {
      double acc = 0;
      for (int q = jct_rp[i]; q < jct_rp[i + 1]; ++q) acc += jct_v[q] * ryc[jct_ci[q]];
      rhs_o[i] = rxc[i] + gamma * acc;
    }
    oracle_chol_solve(C, rhs_o, sol_o);
    double* sc = NEW(double, m_c);
    spmv(m_c, jc_rp, jc_ci, R->jc_s, sol_o, sc);
    for (int k = 0; k < m_c; ++k) { sc[k] -= ryc[k]; dy[k] = 0.0; }
    double cerr = 0;
    const double t2 = now_s();
    total_its += m_c > 0 ? schur_cg_rel(C, m_c, n, jc_rp, jc_ci, R->jc_s, &jct_view, sc, dy, itmax, tol, refine_rtol,
                                        &cerr)
                         : 0;
    R->t_cg += now_s() - t2;
    free(sc);
    spmv_t(m_c, n, jc_rp, jc_ci, R->jc_s, dy, t);
    for (int i = 0; i < n; ++i) t[i] = rhs_o[i] - t[i];
    oracle_chol_solve(C, t, dx);
    for (int i = 0; i < n; ++i) R->x[i] += dx[i] * R->max_d[i];
    for (int k = 0; k < m_c; ++k) R->y[k] += dy[k] * R->max_d[n + k];
    for (int k = 0; k < m_d; ++k) {
      double jx = 0;
      if (jd_flag)
        for (int p = jd_rp[k]; p < jd_rp[k + 1]; ++p) jx += jd_v[p] * (dx[jd_ci[p]] * R->max_d[jd_ci[p]]);
      const double dsk = jd_flag ? jx - e4[k] : -e4[k];
      R->s[k] += dsk;
      R->yd[k] += dsk * ds_v[k] - e2[k];
    }
    kkt_residual(&K, R->x, R->s, R->y, R->yd, e1, e2, e3, e4, &R->rel_res_ref, &R->rel_res_full);
    R->refine_steps += 1;
  }
  R->cg_iters_total = total_its;
  free(e1); free(e2); free(e3); free(e4); free(dx); free(dy); free(rxc); free(ryc);
  free(t); free(rhs_o); free(sol_o); free(rev);
  free(jct_rp); free(jct_ci); free(jct_v);
  if (jd_flag) { free(jdt_rp); free(jdt_ci); free(jdt_v); }
  oracle_chol_free(C);
  return R;
}

typedef struct { const char* name; int is_int; } field_t;

static const void* field(const oracle_result* R, const char* name, long* n, int* is_int) {
  const int nx = R->n_x;
  *is_int = 0;
#define F(NAME, PTR, LEN, INT) if (!strcmp(name, NAME)) { *n = (LEN); *is_int = (INT); return (PTR); }
  F("ht_rp", R->ht_rp, nx + 1, 1)
  F("ht_ci", R->ht_ci, R->nnz_ht, 1)
  F("ht_v0", R->ht_v0, R->nnz_ht, 0)
  F("ht_v", R->ht_v, R->nnz_ht, 0)
  F("jc_s", R->jc_s, -1, 0)
  F("ry_s", R->ry_s, R->m_c, 0)
  F("rxt", R->rxt, nx, 0)
  F("max_d", R->max_d, nx + R->m_c, 0)
  F("hg_rp", R->hg_rp, nx + 1, 1)
  F("hg_ci", R->hg_ci, R->nnz_hg, 1)
  F("hg_v", R->hg_v, R->nnz_hg, 0)
  F("rhat", R->rhat, nx, 0)
  F("rxp", R->rxp, nx, 0)
  F("hrxp", R->hrxp, nx, 0)
  F("schur", R->schur, R->m_c, 0)
  F("parent", R->parent, nx, 1)
  F("L_cp", R->L_cp, nx + 1, 1)
  F("L_ri", R->L_ri, R->nnz_L, 1)
  F("L_v", R->L_v, R->nnz_L, 0)
  F("perm", R->perm, nx, 1)
  F("x", R->x, nx, 0)
  F("s", R->s, R->m_d, 0)
  F("y", R->y, R->m_c, 0)
  F("yd", R->yd, R->m_d, 0)
#undef F
  *n = -2;
  return NULL;
}

long oracle_size(const oracle_result* R, const char* name) {
  long n;
  int it;
  field(R, name, &n, &it);
  return n;
}

int oracle_get(const oracle_result* R, const char* name, void* out, long n) {
  long len;
  int it;
  const void* p = field(R, name, &len, &it);
  if (!p) return -1;
  if (len >= 0 && n > len) return -2;
  memcpy(out, p, (size_t)n * (it ? sizeof(int) : sizeof(double)));
  return 0;
}

double oracle_scalar(const oracle_result* R, const char* name) {
  if (!strcmp(name, "rel_res_ref")) return R->rel_res_ref;
  if (!strcmp(name, "rel_res_full")) return R->rel_res_full;
  if (!strcmp(name, "cg_err")) return R->cg_err;
  if (!strcmp(name, "cg_iters")) return R->cg_iters;
  if (!strcmp(name, "pivot_col")) return R->pivot_col;
  if (!strcmp(name, "nnz_L")) return (double)R->nnz_L;
  if (!strcmp(name, "rel_res_first")) return R->rel_res_first;
  if (!strcmp(name, "cg_iters_total")) return R->cg_iters_total;
  if (!strcmp(name, "refine_steps")) return R->refine_steps;
  if (!strcmp(name, "t_setup")) return R->t_setup;
  if (!strcmp(name, "t_cg")) return R->t_cg;
  return NAN;
}

void oracle_free(oracle_result* R) {
  if (!R) return;
  free(R->ht_rp); free(R->ht_ci); free(R->hg_rp); free(R->hg_ci); free(R->parent); free(R->L_cp); free(R->L_ri);
  free(R->perm); free(R->ht_v0); free(R->ht_v); free(R->jc_s); free(R->ry_s); free(R->rxt); free(R->max_d);
  free(R->hg_v); free(R->rhat); free(R->rxp); free(R->hrxp); free(R->schur); free(R->L_v);
  free(R->x); free(R->s); free(R->y); free(R->yd);
  free(R);
}
