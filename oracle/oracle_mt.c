/*
 * Multithreaded supernodal Cholesky for the CPU baseline -- TEST AND
 * MEASUREMENT INFRASTRUCTURE ONLY.
 *
 * The oracle's default factorization (hykkt_oracle.c, up-looking, one
 * thread) is the checker; this file gives the CPU baseline a solve that uses
 * every host core, with the same mathematics: the Cholesky factor of the
 * permuted H_gamma (CholeskyClass::numerical_factorization,
 * CholeskyClass.cpp:71-90, pivot test 1e-12) and the two triangular solves
 * (CholeskyClass::solve, CholeskyClass.cpp:93-101).  The reference calls
 * cuSOLVER for both; its internal method is not public, so this is a
 * textbook multifrontal method (Duff and Reid 1983; Liu 1992):
 *   - analysis (once per pattern): column counts from the row-subtree
 *     walks, fundamental supernodes, each supernode's row structure, the
 *     extend-add positions of every child in its parent, the assembly map;
 *   - numeric: supernodes by tree level; fronts of a level with at most
 *     SMALL_FRONT rows are factorized one per thread in per-thread
 *     workspaces, larger fronts one at a time in one reused workspace, with
 *     their assembly, extend-add and blocked dense kernels spread over the
 *     threads;
 *   - solves: forward by levels with per-supernode update vectors (no two
 *     threads write one entry), backward by levels top-down; supernodes
 *     holding more than PAR_SOLVE entries are split over the threads.
 * Every sum is taken in a fixed order for a fixed thread count, so a solve
 * is repeatable.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_mt.h"

#define NEWZ(T, n) ((T*)calloc((size_t)((n) > 0 ? (n) : 1), sizeof(T)))
#define SMALL_FRONT 384  /* fronts up to this many rows: one thread each */
#define NB 64            /* panel width of the blocked partial Cholesky */
#define TB 128           /* tile size of the trailing update / solve blocks */
#define PAR_SOLVE (1 << 18)  /* solve a supernode with all threads above this many stored entries */

struct sn_chol {
  int n, nsn, threads;
  int *sn_first;     /* nsn+1: columns of supernode J are sn_first[J] .. sn_first[J+1]-1 */
  int *sn_of;        /* n: supernode of each column */
  int *sn_parent;    /* nsn: -1 at roots */
  int *ch_p, *ch;    /* children of each supernode, ascending */
  int *ip, *post;    /* n: the postorder numbering of the caller's column j is ip[j]; post = its inverse */
  int refs;          /* owners of this analysis (sn_retain / sn_release) */
  int64_t *rows_p;   /* nsn+1: rows of J (its columns first, ascending) */
  int *rows;
  int64_t *rel_p;    /* nsn+1: positions of J's below rows inside its parent's rows */
  int *rel;
  int *lvl_p, *lvl;  /* supernodes grouped by tree level (leaves first) */
  int nlvl;
  int64_t *a_p;      /* nsn+1: original lower entries assembled into J */
  int *a_row, *a_col;  /* front-local row position, local column */
  int64_t *a_src;    /* index into the lower-rows value array */
  int64_t *L_off;    /* nsn+1: factor block of J (nr x nc, column-major) */
  int64_t *u_off;    /* nsn+1: forward update vector of J (nr - nc) */
};

static inline int nr_of(const sn_chol* c, int J) { return (int)(c->rows_p[J + 1] - c->rows_p[J]); }
static inline int nc_of(const sn_chol* c, int J) { return c->sn_first[J + 1] - c->sn_first[J]; }

/* ------------------------------------------------------------------------ */
/* analysis                                                                  */
/* ------------------------------------------------------------------------ */
/* nonzero pattern of row k of L (columns < k), by the row subtree of the
 * elimination tree (Davis 2006, sec. 4.1); returns the start in s[] */
static int row_reach(int k, const int* lrp, const int* lci, const int* parent, int* s, int* w, int n) {
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

/* relaxed amalgamation: may a child of nc_c columns (stored entries st_c,
 * zeros z_c) merge into its parent (nc_p, nr_p, st_p, z_p)?  Thresholds as
 * in common supernodal codes: always up to 4 columns, then a shrinking
 * fraction of explicit zeros as the merged supernode widens */
static int may_merge(int64_t nc_c, int64_t st_c, int64_t z_c, int64_t nc_p, int64_t nr_p, int64_t st_p, int64_t z_p,
                     int64_t* st_new, int64_t* z_new) {
  const int64_t nc = nc_c + nc_p, nr = nc_c + nr_p;
  const int64_t st = nc * nr - nc * (nc - 1) / 2;
  const int64_t z = st - (st_c - z_c) - (st_p - z_p);
  *st_new = st;
  *z_new = z;
  const double frac = st > 0 ? (double)z / (double)st : 0.0;
  if (nc <= 4) return 1;
  if (nc <= 16) return frac < 0.8;
  if (nc <= 48) return frac < 0.1;
  return frac < 0.05;
}

sn_chol* sn_analyze(int n, const int* lrp0, const int* lci0, const int* parent0, int threads) {
  sn_chol* c = (sn_chol*)calloc(1, sizeof(sn_chol));
  c->n = n;
  c->threads = threads > 0 ? threads : 1;
  /* postorder of the elimination tree (children ascending): every subtree
   * becomes a contiguous range of columns, so a supernode's last child sits
   * right before it and can merge.  Structure is preserved (an entry
   * L(k, j) has k an ancestor of j, which stays after j). */
  int* post = c->post = NEWZ(int, n);  /* post[new] = old */
  c->ip = NEWZ(int, n);      /* ip[old] = new */
  {
    int *head = NEWZ(int, n), *next = NEWZ(int, n), *stack = NEWZ(int, n);
    for (int j = 0; j < n; ++j) head[j] = -1;
    for (int j = n - 1; j >= 0; --j)
      if (parent0[j] >= 0) {
        next[j] = head[parent0[j]];
        head[parent0[j]] = j;
      }
    int k = 0;
    for (int r = 0; r < n; ++r) {
      if (parent0[r] >= 0) continue;
      int top = 0;
      stack[top++] = r;
      while (top > 0) {
        const int j = stack[top - 1];
        const int ch = head[j];
        if (ch < 0) {
          --top;
          post[k++] = j;
        } else {
          head[j] = next[ch];
          stack[top++] = ch;
        }
      }
    }
    for (int j = 0; j < n; ++j) c->ip[post[j]] = j;
    free(head); free(next); free(stack);
  }
  /* lower rows and etree in the postordered numbering; the value array
   * stays in the caller's order (src[] maps the entries) */
  int* parent = NEWZ(int, n);
  for (int j = 0; j < n; ++j) parent[c->ip[j]] = parent0[j] >= 0 ? c->ip[parent0[j]] : -1;
  int* lrp = NEWZ(int, n + 1);
  int* lci = NEWZ(int, lrp0[n]);
  int64_t* lsrc = NEWZ(int64_t, lrp0[n]);
  for (int k = 0; k < n; ++k) lrp[c->ip[k] + 1] = lrp0[k + 1] - lrp0[k];
  for (int k = 0; k < n; ++k) lrp[k + 1] += lrp[k];
  for (int k = 0; k < n; ++k) {
    int q = lrp[c->ip[k]];
    for (int p = lrp0[k]; p < lrp0[k + 1]; ++p, ++q) {
      lci[q] = c->ip[lci0[p]];
      lsrc[q] = p;
    }
  }
  int* s = NEWZ(int, n);
  int* w = NEWZ(int, n);
  int* cnt = NEWZ(int, n);
  for (int k = 0; k < n; ++k) w[k] = -1;
  for (int k = 0; k < n; ++k) {
    cnt[k]++;
    int top = row_reach(k, lrp, lci, parent, s, w, n);
    for (int t = top; t < n; ++t) cnt[s[t]]++;
  }
  /* fundamental supernodes: j joins j-1's supernode when j is j-1's parent,
   * its only child, and L(:, j-1) = {j-1} + L(:, j) */
  int* nchild = NEWZ(int, n);
  for (int j = 0; j < n; ++j)
    if (parent[j] >= 0) nchild[parent[j]]++;
  int* fsn_first = NEWZ(int, n + 1);
  int* fsn_of = NEWZ(int, n);
  int nf = 0;
  for (int j = 0; j < n; ++j) {
    const int join = j > 0 && parent[j - 1] == j && nchild[j] == 1 && cnt[j - 1] == cnt[j] + 1;
    if (!join) fsn_first[nf++] = j;
    fsn_of[j] = nf - 1;
  }
  fsn_first[nf] = n;
  /* relaxed amalgamation, bottom-up: a supernode absorbs the child that
   * ends right before its first column when may_merge() allows */
  int* grp_first = NEWZ(int, nf);  /* first column of the merged group ending at fundamental supernode F */
  int64_t* st = NEWZ(int64_t, nf);
  int64_t* zz = NEWZ(int64_t, nf);
  int* absorbed = NEWZ(int, nf);
  for (int F = 0; F < nf; ++F) {
    const int64_t ncF = fsn_first[F + 1] - fsn_first[F], nrF = cnt[fsn_first[F]];
    grp_first[F] = fsn_first[F];
    st[F] = ncF * nrF - ncF * (ncF - 1) / 2;
    zz[F] = 0;
    if (F == 0) continue;
    const int C = fsn_of[grp_first[F] - 1];  /* the group ending right before F */
    const int lastC = fsn_first[C + 1] - 1;
    if (parent[lastC] < fsn_first[F] || parent[lastC] >= fsn_first[F + 1]) continue;  /* not F's child */
    const int64_t ncC = fsn_first[C + 1] - grp_first[C];
    int64_t st_new, z_new;
    if (may_merge(ncC, st[C], zz[C], ncF, nrF, st[F], zz[F], &st_new, &z_new)) {
      grp_first[F] = grp_first[C];
      st[F] = st_new;
      zz[F] = z_new;
      absorbed[C] = 1;
    }
  }
  int nsn = 0;
  for (int F = 0; F < nf; ++F) nsn += !absorbed[F];
  c->nsn = nsn;
  c->sn_first = NEWZ(int, nsn + 1);
  c->sn_of = NEWZ(int, n);
  int* top_f = NEWZ(int, nsn);  /* the fundamental supernode holding each final supernode's last column */
  {
    int J = 0;
    for (int F = 0; F < nf; ++F)
      if (!absorbed[F]) {
        c->sn_first[J] = grp_first[F];
        top_f[J] = F;
        for (int j = grp_first[F]; j < fsn_first[F + 1]; ++j) c->sn_of[j] = J;
        ++J;
      }
    c->sn_first[nsn] = n;
  }
  c->sn_parent = NEWZ(int, nsn);
  for (int J = 0; J < nsn; ++J) {
    const int last = c->sn_first[J + 1] - 1;
    c->sn_parent[J] = parent[last] >= 0 ? c->sn_of[parent[last]] : -1;
  }
  c->ch_p = NEWZ(int, nsn + 1);
  c->ch = NEWZ(int, nsn);
  for (int J = 0; J < nsn; ++J)
    if (c->sn_parent[J] >= 0) c->ch_p[c->sn_parent[J] + 1]++;
  for (int J = 0; J < nsn; ++J) c->ch_p[J + 1] += c->ch_p[J];
  {
    int* at = NEWZ(int, nsn);
    for (int J = 0; J < nsn; ++J)
      if (c->sn_parent[J] >= 0) c->ch[c->ch_p[c->sn_parent[J]] + at[c->sn_parent[J]]++] = J;
    free(at);
  }
  /* rows of the top fundamental supernode F = {first column of F} + {k :
   * first column of F in the row pattern of k}; a final supernode's rows are
   * its own columns followed by F's rows beyond its last column */
  int64_t* frows_p = NEWZ(int64_t, nf + 1);
  for (int F = 0; F < nf; ++F) frows_p[F + 1] = frows_p[F] + cnt[fsn_first[F]];
  int* frows = NEWZ(int, frows_p[nf]);
  int64_t* fill = NEWZ(int64_t, nf);
  for (int F = 0; F < nf; ++F) {
    frows[frows_p[F]] = fsn_first[F];
    fill[F] = 1;
  }
  for (int k = 0; k < n; ++k) w[k] = -1;
  for (int k = 0; k < n; ++k) {
    int top = row_reach(k, lrp, lci, parent, s, w, n);
    for (int t = top; t < n; ++t) {
      const int j = s[t];
      const int F = fsn_of[j];
      if (fsn_first[F] == j && !absorbed[F]) frows[frows_p[F] + fill[F]++] = k;  /* ascending in k */
    }
  }
  c->rows_p = NEWZ(int64_t, nsn + 1);
  for (int J = 0; J < nsn; ++J) {
    const int F = top_f[J];
    const int ncJ = c->sn_first[J + 1] - c->sn_first[J];
    const int ncF = fsn_first[F + 1] - fsn_first[F];
    c->rows_p[J + 1] = c->rows_p[J] + ncJ + (cnt[fsn_first[F]] - ncF);
  }
  c->rows = NEWZ(int, c->rows_p[nsn]);
  for (int J = 0; J < nsn; ++J) {
    const int F = top_f[J];
    const int ncJ = c->sn_first[J + 1] - c->sn_first[J];
    const int ncF = fsn_first[F + 1] - fsn_first[F];
    int* r = c->rows + c->rows_p[J];
    for (int a = 0; a < ncJ; ++a) r[a] = c->sn_first[J] + a;
    memcpy(r + ncJ, frows + frows_p[F] + ncF, sizeof(int) * (size_t)(cnt[fsn_first[F]] - ncF));
  }
  free(fsn_first); free(fsn_of); free(grp_first); free(st); free(zz); free(absorbed); free(top_f);
  free(frows_p); free(frows); free(fill);
  /* extend-add positions of each supernode's below rows in its parent */
  c->rel_p = NEWZ(int64_t, nsn + 1);
  for (int J = 0; J < nsn; ++J) c->rel_p[J + 1] = c->rel_p[J] + (nr_of(c, J) - nc_of(c, J));
  c->rel = NEWZ(int, c->rel_p[nsn]);
  for (int J = 0; J < nsn; ++J) {
    const int P = c->sn_parent[J];
    if (P < 0) continue;
    const int* rj = c->rows + c->rows_p[J] + nc_of(c, J);
    const int* rp = c->rows + c->rows_p[P];
    const int m = nr_of(c, J) - nc_of(c, J), np = nr_of(c, P);
    int q = 0;
    for (int a = 0; a < m; ++a) {
      while (q < np && rp[q] < rj[a]) ++q;
      c->rel[c->rel_p[J] + a] = q;  /* the parent's rows contain every below row of a child */
    }
  }
  /* tree levels (a supernode's level is above all of its children's) */
  int* lev = NEWZ(int, nsn);
  int nlvl = 0;
  for (int J = 0; J < nsn; ++J) {  /* children have smaller indices */
    const int P = c->sn_parent[J];
    if (P >= 0 && lev[P] < lev[J] + 1) lev[P] = lev[J] + 1;
    if (lev[J] + 1 > nlvl) nlvl = lev[J] + 1;
  }
  c->nlvl = nlvl;
  c->lvl_p = NEWZ(int, nlvl + 1);
  c->lvl = NEWZ(int, nsn);
  for (int J = 0; J < nsn; ++J) c->lvl_p[lev[J] + 1]++;
  for (int l = 0; l < nlvl; ++l) c->lvl_p[l + 1] += c->lvl_p[l];
  int* pos = NEWZ(int, nlvl);
  for (int J = 0; J < nsn; ++J) c->lvl[c->lvl_p[lev[J]] + pos[lev[J]]++] = J;
  /* assembly map: entry (k, j) of the lower rows (j <= k) goes to front
   * position (row of k in sn(j), column j - first); its value is entry
   * lsrc of the caller's array */
  c->a_p = NEWZ(int64_t, nsn + 1);
  for (int k = 0; k < n; ++k)
    for (int p = lrp[k]; p < lrp[k + 1]; ++p) c->a_p[c->sn_of[lci[p]] + 1]++;
  for (int J = 0; J < nsn; ++J) c->a_p[J + 1] += c->a_p[J];
  const int64_t na = c->a_p[nsn];
  c->a_row = NEWZ(int, na);
  c->a_col = NEWZ(int, na);
  c->a_src = NEWZ(int64_t, na);
  int64_t* ap = NEWZ(int64_t, nsn);
  for (int J = 0; J < nsn; ++J) ap[J] = c->a_p[J];
  int* loc = NEWZ(int, n);
  for (int k = 0; k < n; ++k)
    for (int p = lrp[k]; p < lrp[k + 1]; ++p) {
      const int J = c->sn_of[lci[p]];
      const int64_t q = ap[J]++;
      c->a_row[q] = k;  /* global row, resolved below */
      c->a_col[q] = lci[p] - c->sn_first[J];
      c->a_src[q] = lsrc[p];
    }
  for (int J = 0; J < nsn; ++J) {
    const int* r = c->rows + c->rows_p[J];
    for (int a = 0; a < nr_of(c, J); ++a) loc[r[a]] = a;
    for (int64_t q = c->a_p[J]; q < c->a_p[J + 1]; ++q) c->a_row[q] = loc[c->a_row[q]];
  }
  c->L_off = NEWZ(int64_t, nsn + 1);
  c->u_off = NEWZ(int64_t, nsn + 1);
  for (int J = 0; J < nsn; ++J) {
    c->L_off[J + 1] = c->L_off[J] + (int64_t)nr_of(c, J) * nc_of(c, J);
    c->u_off[J + 1] = c->u_off[J] + (nr_of(c, J) - nc_of(c, J));
  }
  c->refs = 1;
  free(s); free(w); free(cnt); free(nchild); free(lev); free(pos); free(ap); free(loc);
  free(parent); free(lrp); free(lci); free(lsrc);
  return c;
}

int64_t sn_nnz(const sn_chol* c) { return c->L_off[c->nsn]; }

/* ------------------------------------------------------------------------ */
/* dense kernels (column-major, lower triangle)                             */
/* ------------------------------------------------------------------------ */
/* C(i0:i1, j0:j1) -= A(i0:i1, 0:kb) * A(j0:j1, 0:kb)^T with A(i, k) = a[i + k*ld] */
static void tile_update(double* C, int ld, const double* a, int kb, int i0, int i1, int j0, int j1) {
  int j = j0;
  for (; j + 4 <= j1; j += 4) {
    int i = i0;
    for (; i + 8 <= i1; i += 8) {
      double acc[4][8];
      for (int x = 0; x < 4; ++x)
        for (int y = 0; y < 8; ++y) acc[x][y] = 0.0;
      for (int k = 0; k < kb; ++k) {
        const double* ak = a + (int64_t)k * ld;
        const double b0 = ak[j], b1 = ak[j + 1], b2 = ak[j + 2], b3 = ak[j + 3];
        for (int y = 0; y < 8; ++y) {
          const double av = ak[i + y];
          acc[0][y] += av * b0;
          acc[1][y] += av * b1;
          acc[2][y] += av * b2;
          acc[3][y] += av * b3;
        }
      }
      for (int x = 0; x < 4; ++x)
        for (int y = 0; y < 8; ++y) C[(i + y) + (int64_t)(j + x) * ld] -= acc[x][y];
    }
    for (; i < i1; ++i)
      for (int x = 0; x < 4; ++x) {
        double t = 0.0;
        for (int k = 0; k < kb; ++k) t += a[i + (int64_t)k * ld] * a[j + x + (int64_t)k * ld];
        C[i + (int64_t)(j + x) * ld] -= t;
      }
  }
  for (; j < j1; ++j)
    for (int i = i0; i < i1; ++i) {
      double t = 0.0;
      for (int k = 0; k < kb; ++k) t += a[i + (int64_t)k * ld] * a[j + (int64_t)k * ld];
      C[i + (int64_t)j * ld] -= t;
    }
}

/* unblocked Cholesky of the kb x kb block at F (ld); returns the first bad
 * column or -1 (pivot sqrt(d) <= 1e-12, CholeskyClass.cpp:87-89) */
static int potf2(double* F, int ld, int kb) {
  int bad = -1;
  for (int k = 0; k < kb; ++k) {
    double d = F[k + (int64_t)k * ld];
    if (!(d > 1e-24) && bad < 0) bad = k;
    d = sqrt(d > 0 ? d : 0.0);
    F[k + (int64_t)k * ld] = d;
    const double inv = d > 0 ? 1.0 / d : 0.0;
    for (int i = k + 1; i < kb; ++i) F[i + (int64_t)k * ld] *= inv;
    for (int j = k + 1; j < kb; ++j) {
      const double ljk = F[j + (int64_t)k * ld];
      for (int i = j; i < kb; ++i) F[i + (int64_t)j * ld] -= F[i + (int64_t)k * ld] * ljk;
    }
  }
  return bad;
}

/* rows r0..r1 of the panel below the diagonal block: A21 <- A21 L11^{-T} */
static void trsm_rows(double* F, int ld, int k0, int kb, int r0, int r1) {
  const double* L11 = F + k0 + (int64_t)k0 * ld;
  for (int k = 0; k < kb; ++k) {
    double* ck = F + (int64_t)(k0 + k) * ld;
    for (int m = 0; m < k; ++m) {
      const double lkm = L11[k + (int64_t)m * ld];
      const double* cm = F + (int64_t)(k0 + m) * ld;
      for (int i = r0; i < r1; ++i) ck[i] -= cm[i] * lkm;
    }
    const double d = L11[k + (int64_t)k * ld];
    const double inv = d > 0 ? 1.0 / d : 0.0;
    for (int i = r0; i < r1; ++i) ck[i] *= inv;
  }
}

/* partial Cholesky of the first nc columns of the nr x nr front F (ld = nr),
 * the trailing block becomes the update matrix; par: spread over threads */
static int front_factor(double* F, int nr, int nc, int par, int threads) {
  const int ld = nr;
  int bad = -1;
  for (int k0 = 0; k0 < nc; k0 += NB) {
    const int kb = nc - k0 < NB ? nc - k0 : NB;
    const int b = potf2(F + k0 + (int64_t)k0 * ld, ld, kb);
    if (b >= 0 && bad < 0) bad = k0 + b;
    const int r0 = k0 + kb;
    if (r0 >= nr) break;
    const int nrb = (nr - r0 + TB - 1) / TB;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) if (par)
    for (int t = 0; t < nrb; ++t) {
      const int a = r0 + t * TB, e = a + TB < nr ? a + TB : nr;
      trsm_rows(F, ld, k0, kb, a, e);
    }
    /* lower tiles (ti >= tj) of the trailing matrix */
    const long ntile = (long)nrb * (nrb + 1) / 2;
    const double* panel = F + (int64_t)k0 * ld;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) if (par)
    for (long t = 0; t < ntile; ++t) {
      /* t -> (ti, tj), tj <= ti, row-major over the lower triangle of tiles */
      int ti = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) / 2.0);
      while ((long)ti * (ti + 1) / 2 > t) --ti;
      while ((long)(ti + 1) * (ti + 2) / 2 <= t) ++ti;
      const int tj = (int)(t - (long)ti * (ti + 1) / 2);
      const int i0 = r0 + ti * TB, i1 = i0 + TB < nr ? i0 + TB : nr;
      const int j0 = r0 + tj * TB, j1 = j0 + TB < nr ? j0 + TB : nr;
      tile_update(F, ld, panel, kb, i0, i1, j0, j1);
    }
  }
  return bad;
}

/* ------------------------------------------------------------------------ */
/* numeric factorization                                                    */
/* ------------------------------------------------------------------------ */
/* assemble A's entries and the children's update matrices into the front F
 * (nr x nr, ld nr; its lower part zero on entry); par: spread over threads */
static void assemble(const sn_chol* c, int J, const double* lvals, double** U, double* F, int par, int T) {
  const int nr = nr_of(c, J);
  for (int64_t e = c->a_p[J]; e < c->a_p[J + 1]; ++e) F[c->a_row[e] + (int64_t)c->a_col[e] * nr] += lvals[c->a_src[e]];
  /* children in index order: a fixed summation order for every entry */
  for (int ci = c->ch_p[J]; ci < c->ch_p[J + 1]; ++ci) {
    const int C = c->ch[ci];
    if (!U[C]) continue;
    const int m = nr_of(c, C) - nc_of(c, C);
    const int* rel = c->rel + c->rel_p[C];
    const double* u = U[C];
#pragma omp parallel for schedule(dynamic, 16) num_threads(T) if (par)
    for (int b = 0; b < m; ++b) {
      double* Fb = F + (int64_t)rel[b] * nr;
      const double* ub = u + (int64_t)b * m;
      for (int a = b; a < m; ++a) Fb[rel[a]] += ub[a];
    }
    free(U[C]);
    U[C] = NULL;
  }
}

/* after the partial factorization: J's factor block to Lv, its update
 * matrix (lower m x m) to a new array for the parent */
static double* extract(const sn_chol* c, int J, const double* F, double* Lv, int par, int T) {
  const int nr = nr_of(c, J), nc = nc_of(c, J), m = nr - nc;
#pragma omp parallel for schedule(static) num_threads(T) if (par)
  for (int k = 0; k < nc; ++k) memcpy(Lv + c->L_off[J] + (int64_t)k * nr, F + (int64_t)k * nr, sizeof(double) * nr);
  if (m <= 0 || c->sn_parent[J] < 0) return NULL;
  double* u = (double*)malloc(sizeof(double) * (size_t)m * m);
#pragma omp parallel for schedule(dynamic, 16) num_threads(T) if (par)
  for (int b = 0; b < m; ++b)
    memcpy(u + (int64_t)b * m + b, F + (nc + b) + (int64_t)(nc + b) * nr, sizeof(double) * (m - b));
  return u;
}

/* zero the lower part of an nr x nr front */
static void zero_lower(double* F, int nr, int par, int T) {
#pragma omp parallel for schedule(static) num_threads(T) if (par)
  for (int b = 0; b < nr; ++b) memset(F + (int64_t)b * nr + b, 0, sizeof(double) * (nr - b));
}

double* sn_factor(const sn_chol* c, const double* lvals, int* bad_col) {
  const int T = c->threads;
  double* Lv = (double*)malloc(sizeof(double) * (size_t)(c->L_off[c->nsn] > 0 ? c->L_off[c->nsn] : 1));
  double** U = (double**)calloc((size_t)c->nsn, sizeof(double*));  /* update matrices awaiting the parent */
  int maxbig = 0;
  for (int J = 0; J < c->nsn; ++J)
    if (nr_of(c, J) > SMALL_FRONT && nr_of(c, J) > maxbig) maxbig = nr_of(c, J);
  /* one workspace for the large fronts (factorized one at a time), one
   * small-front workspace per thread: no allocation per front */
  double* Wbig = maxbig ? (double*)malloc(sizeof(double) * (size_t)maxbig * maxbig) : NULL;
  double* Wsmall = (double*)malloc(sizeof(double) * (size_t)T * SMALL_FRONT * SMALL_FRONT);
  int bad = INT32_MAX;
  for (int l = 0; l < c->nlvl; ++l) {
    const int lo = c->lvl_p[l], hi = c->lvl_p[l + 1];
    int bad_small = INT32_MAX;
#pragma omp parallel for schedule(dynamic, 1) num_threads(T) reduction(min : bad_small)
    for (int q = lo; q < hi; ++q) {
      const int J = c->lvl[q];
      const int nr = nr_of(c, J), nc = nc_of(c, J);
      if (nr > SMALL_FRONT) continue;
      double* F = Wsmall + (size_t)omp_get_thread_num() * SMALL_FRONT * SMALL_FRONT;
      zero_lower(F, nr, 0, 1);
      assemble(c, J, lvals, U, F, 0, 1);
      const int b = front_factor(F, nr, nc, 0, 1);
      if (b >= 0 && c->sn_first[J] + b < bad_small) bad_small = c->sn_first[J] + b;
      U[J] = extract(c, J, F, Lv, 0, 1);
    }
    if (bad_small < bad) bad = bad_small;
    for (int q = lo; q < hi; ++q) {
      const int J = c->lvl[q];
      const int nr = nr_of(c, J), nc = nc_of(c, J);
      if (nr <= SMALL_FRONT) continue;
      zero_lower(Wbig, nr, 1, T);
      assemble(c, J, lvals, U, Wbig, 1, T);
      const int b = front_factor(Wbig, nr, nc, 1, T);
      if (b >= 0 && c->sn_first[J] + b < bad) bad = c->sn_first[J] + b;
      U[J] = extract(c, J, Wbig, Lv, 1, T);
    }
  }
  for (int J = 0; J < c->nsn; ++J) free(U[J]);
  free(U);
  free(Wbig);
  free(Wsmall);
  /* the first failed pivot in the postordered elimination, in the caller's numbering */
  *bad_col = bad == INT32_MAX ? -1 : c->post[bad];
  return Lv;
}

/* ------------------------------------------------------------------------ */
/* solves: y (permuted numbering) is overwritten by (L L^T)^{-1} y          */
/* ------------------------------------------------------------------------ */
/* x(0:nc) <- L11^{-1} x for the nc x nc lower block at L (ld) */
static void trsv_lower(const double* L, int ld, int nc, double* x) {
  for (int k = 0; k < nc; ++k) {
    const double xk = x[k] / L[k + (int64_t)k * ld];
    x[k] = xk;
    const double* lk = L + (int64_t)k * ld;
    for (int i = k + 1; i < nc; ++i) x[i] -= lk[i] * xk;
  }
}
/* x(0:nc) <- L11^{-T} x */
static void trsv_lower_t(const double* L, int ld, int nc, double* x) {
  for (int k = nc - 1; k >= 0; --k) {
    const double* lk = L + (int64_t)k * ld;
    double t = x[k];
    for (int i = k + 1; i < nc; ++i) t -= lk[i] * x[i];
    x[k] = t / L[k + (int64_t)k * ld];
  }
}

/* forward step of supernode J: v holds b(cols) then 0 (below); children's
 * update vectors are subtracted; x(cols) and J's own update vector result */
static void fwd_node(const sn_chol* c, const double* Lv, int J, double* y, double* uvec, double* v, int par) {
  const int nr = nr_of(c, J), nc = nc_of(c, J), f = c->sn_first[J];
  const int T = c->threads;
  for (int a = 0; a < nc; ++a) v[a] = y[f + a];
  for (int a = nc; a < nr; ++a) v[a] = 0.0;
  for (int ci = c->ch_p[J]; ci < c->ch_p[J + 1]; ++ci) {
    const int C = c->ch[ci];
    const int m = nr_of(c, C) - nc_of(c, C);
    const int* rel = c->rel + c->rel_p[C];
    const double* uc = uvec + c->u_off[C];
    for (int a = 0; a < m; ++a) v[rel[a]] -= uc[a];
  }
  const double* L = Lv + c->L_off[J];
  if (!par) {
    trsv_lower(L, nr, nc, v);
    for (int k = 0; k < nc; ++k) {
      const double xk = v[k];
      const double* lk = L + (int64_t)k * nr;
      for (int i = nc; i < nr; ++i) v[i] -= lk[i] * xk;
    }
  } else {
    for (int k0 = 0; k0 < nc; k0 += TB) {
      const int kb = nc - k0 < TB ? nc - k0 : TB;
      trsv_lower(L + k0 + (int64_t)k0 * nr, nr, kb, v + k0);
      const int r0 = k0 + kb, nrb = (nr - r0 + TB - 1) / TB;
#pragma omp parallel for schedule(static) num_threads(T)
      for (int t = 0; t < nrb; ++t) {
        const int a = r0 + t * TB, e = a + TB < nr ? a + TB : nr;
        for (int k = 0; k < kb; ++k) {
          const double xk = v[k0 + k];
          const double* lk = L + (int64_t)(k0 + k) * nr;
          for (int i = a; i < e; ++i) v[i] -= lk[i] * xk;
        }
      }
    }
  }
  for (int a = 0; a < nc; ++a) y[f + a] = v[a];
  double* u = uvec + c->u_off[J];
  for (int a = nc; a < nr; ++a) u[a - nc] = -v[a];
}

/* backward step: y(cols) <- L11^{-T} (y(cols) - L21^T y(below rows)) */
static void bwd_node(const sn_chol* c, const double* Lv, int J, double* y, double* v, double* part, int par) {
  const int nr = nr_of(c, J), nc = nc_of(c, J), f = c->sn_first[J];
  const int T = c->threads;
  const int* rows = c->rows + c->rows_p[J];
  const double* L = Lv + c->L_off[J];
  for (int a = 0; a < nr; ++a) v[a] = y[rows[a]];
  if (!par) {
    for (int k = 0; k < nc; ++k) {
      const double* lk = L + (int64_t)k * nr;
      double t = 0.0;
      for (int i = nc; i < nr; ++i) t += lk[i] * v[i];
      v[k] -= t;
    }
    trsv_lower_t(L, nr, nc, v);
  } else {
    const int nkb = (nc + TB - 1) / TB;
    for (int kbi = nkb - 1; kbi >= 0; --kbi) {
      const int k0 = kbi * TB, kb = nc - k0 < TB ? nc - k0 : TB;
      const int r0 = k0 + kb, nrb = (nr - r0 + TB - 1) / TB;
      /* per row block partial dot products, summed in block order */
#pragma omp parallel for schedule(static) num_threads(T)
      for (int t = 0; t < nrb; ++t) {
        const int a = r0 + t * TB, e = a + TB < nr ? a + TB : nr;
        for (int k = 0; k < kb; ++k) {
          const double* lk = L + (int64_t)(k0 + k) * nr;
          double s = 0.0;
          for (int i = a; i < e; ++i) s += lk[i] * v[i];
          part[(int64_t)t * TB + k] = s;
        }
      }
      for (int k = 0; k < kb; ++k) {
        double s = 0.0;
        for (int t = 0; t < nrb; ++t) s += part[(int64_t)t * TB + k];
        v[k0 + k] -= s;
      }
      trsv_lower_t(L + k0 + (int64_t)k0 * nr, nr, kb, v + k0);
    }
  }
  for (int a = 0; a < nc; ++a) y[f + a] = v[a];
}

static int big_solve(const sn_chol* c, int J) { return (int64_t)nr_of(c, J) * nc_of(c, J) > PAR_SOLVE; }

void sn_solve(const sn_chol* c, const double* Lv, double* y0) {
  const int T = c->threads;
  double* y = NEWZ(double, c->n);
  for (int i = 0; i < c->n; ++i) y[c->ip[i]] = y0[i];
  double* uvec = NEWZ(double, c->u_off[c->nsn]);
  int maxr = 1;
  for (int J = 0; J < c->nsn; ++J) maxr = nr_of(c, J) > maxr ? nr_of(c, J) : maxr;
  double* part = NEWZ(double, (int64_t)((maxr + TB - 1) / TB) * TB);
  for (int l = 0; l < c->nlvl; ++l) {
    const int lo = c->lvl_p[l], hi = c->lvl_p[l + 1];
#pragma omp parallel num_threads(T)
    {
      double* v = NEWZ(double, maxr);
#pragma omp for schedule(dynamic, 4)
      for (int q = lo; q < hi; ++q)
        if (!big_solve(c, c->lvl[q])) fwd_node(c, Lv, c->lvl[q], y, uvec, v, 0);
      free(v);
    }
    double* v = NEWZ(double, maxr);
    for (int q = lo; q < hi; ++q)
      if (big_solve(c, c->lvl[q])) fwd_node(c, Lv, c->lvl[q], y, uvec, v, 1);
    free(v);
  }
  for (int l = c->nlvl - 1; l >= 0; --l) {
    const int lo = c->lvl_p[l], hi = c->lvl_p[l + 1];
    double* v = NEWZ(double, maxr);
    for (int q = lo; q < hi; ++q)
      if (big_solve(c, c->lvl[q])) bwd_node(c, Lv, c->lvl[q], y, v, part, 1);
    free(v);
#pragma omp parallel num_threads(T)
    {
      double* w = NEWZ(double, maxr);
#pragma omp for schedule(dynamic, 4)
      for (int q = lo; q < hi; ++q)
        if (!big_solve(c, c->lvl[q])) bwd_node(c, Lv, c->lvl[q], y, w, NULL, 0);
      free(w);
    }
  }
  for (int i = 0; i < c->n; ++i) y0[i] = y[c->ip[i]];
  free(y);
  free(uvec);
  free(part);
}

void sn_retain(sn_chol* c) {
#pragma omp atomic
  c->refs++;
}

void sn_release(sn_chol* c) {
  if (!c) return;
  int left;
#pragma omp atomic capture
  left = --c->refs;
  if (left > 0) return;
  free(c->sn_first); free(c->sn_of); free(c->sn_parent); free(c->ch_p); free(c->ch); free(c->ip); free(c->post); free(c->rows_p);
  free(c->rows); free(c->rel_p); free(c->rel); free(c->lvl_p); free(c->lvl); free(c->a_p); free(c->a_row);
  free(c->a_col); free(c->a_src); free(c->L_off); free(c->u_off);
  free(c);
}
