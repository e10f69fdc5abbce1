// Per-sparsity symbolic analysis (host).  See symbolic.hpp for what the
// reference does at the same points.
#include "symbolic.hpp"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>

namespace hykkt {

Transposed transpose_pattern(const CsrPattern& a) {
  // Counting sort by column; rows are visited in increasing order so the
  // entries of each transposed row come out sorted by original row.
  Transposed t;
  t.pat.n = a.m;
  t.pat.m = a.n;
  const int nnz = a.nnz();
  t.pat.rp.assign(a.m + 1, 0);
  t.pat.ci.resize(nnz);
  t.src.resize(nnz);
  for (int p = 0; p < nnz; ++p) t.pat.rp[a.ci[p] + 1]++;
  for (int j = 0; j < a.m; ++j) t.pat.rp[j + 1] += t.pat.rp[j];
  std::vector<int> next(t.pat.rp.begin(), t.pat.rp.end() - 1);
  for (int i = 0; i < a.n; ++i)
    for (int p = a.rp[i]; p < a.rp[i + 1]; ++p) {
      int q = next[a.ci[p]]++;
      t.pat.ci[q] = i;
      t.src[q] = p;
    }
  return t;
}

static void check_csr(const CsrPattern& a, const char* name) {
  if ((int)a.rp.size() != a.n + 1) throw std::runtime_error(std::string(name) + ": bad row pointer length");
  if (a.rp[0] != 0) throw std::runtime_error(std::string(name) + ": row pointer must start at 0");
  for (int i = 0; i < a.n; ++i) {
    if (a.rp[i + 1] < a.rp[i]) throw std::runtime_error(std::string(name) + ": row pointers not monotone");
    for (int p = a.rp[i]; p < a.rp[i + 1]; ++p) {
      if (a.ci[p] < 0 || a.ci[p] >= a.m) throw std::runtime_error(std::string(name) + ": column index out of range");
      if (p > a.rp[i] && a.ci[p] <= a.ci[p - 1])
        throw std::runtime_error(std::string(name) + ": columns not sorted/unique within a row");
    }
  }
}

namespace {

// Union of the pattern of row i of a base matrix and of B^T B restricted to
// row i, where B is given by its rows (brp/bci) and its transpose (btrp/btci/
// btsrc).  Produces the sorted union, the base source slot per entry, and the
// product contributions (a = index of B[k,i], b = index of B[k,j], k)
// ascending in k for every entry.
struct ProductUnion {
  CsrPattern pat;
  std::vector<int> base_src;
  std::vector<int> cp;
  std::vector<int> ca, cb, ck;
};

ProductUnion product_union(const CsrPattern& base, const CsrPattern& B, const Transposed& BT) {
  const int n = base.n;
  ProductUnion u;
  u.pat.n = n;
  u.pat.m = base.m;
  u.pat.rp.assign(n + 1, 0);
  std::vector<int> mark(n, -1), slot(n, -1);
  std::vector<int> cols;
  struct Tr { int j, a, b, k; };
  std::vector<Tr> tr;
  u.cp.push_back(0);
  for (int i = 0; i < n; ++i) {
    cols.clear();
    tr.clear();
    for (int p = base.rp[i]; p < base.rp[i + 1]; ++p) {
      int j = base.ci[p];
      if (mark[j] != i) { mark[j] = i; cols.push_back(j); }
    }
    if (!B.rp.empty()) {
      for (int q = BT.pat.rp[i]; q < BT.pat.rp[i + 1]; ++q) {
        int k = BT.pat.ci[q];
        int a = BT.src[q];
        for (int p = B.rp[k]; p < B.rp[k + 1]; ++p) {
          int j = B.ci[p];
          if (mark[j] != i) { mark[j] = i; cols.push_back(j); }
          tr.push_back({j, a, p, k});
        }
      }
    }
    std::sort(cols.begin(), cols.end());
    int base_slot0 = (int)u.pat.ci.size();
    for (size_t t = 0; t < cols.size(); ++t) slot[cols[t]] = base_slot0 + (int)t;
    for (int j : cols) { u.pat.ci.push_back(j); u.base_src.push_back(-1); }
    for (int p = base.rp[i]; p < base.rp[i + 1]; ++p) u.base_src[slot[base.ci[p]]] = p;
    // contributions grouped by slot, k order preserved (BT row is sorted by k)
    std::stable_sort(tr.begin(), tr.end(), [](const Tr& x, const Tr& y) { return x.j < y.j; });
    size_t t = 0;
    for (size_t c = 0; c < cols.size(); ++c) {
      int j = cols[c];
      while (t < tr.size() && tr[t].j == j) {
        u.ca.push_back(tr[t].a);
        u.cb.push_back(tr[t].b);
        u.ck.push_back(tr[t].k);
        ++t;
      }
      u.cp.push_back((int)u.ca.size());
    }
    u.pat.rp[i + 1] = (int)u.pat.ci.size();
  }
  return u;
}

}  // namespace

Symbolic build_symbolic(const CsrPattern& H, const CsrPattern& Ds, const CsrPattern& Jc,
                        const CsrPattern& Jd, const SymbolicOptions& opt, const int* user_perm) {
  Symbolic S;
  // phase timings on stderr when HYKKT_SYMBOLIC_TIMING is set
  const bool timing = std::getenv("HYKKT_SYMBOLIC_TIMING") != nullptr;
  auto t_last = std::chrono::steady_clock::now();
  const char* cur = "checks";
  auto phase = [&](const char* next) {
    if (timing) {
      const auto now = std::chrono::steady_clock::now();
      std::fprintf(stderr, "symbolic %-10s %.3f s\n", cur, std::chrono::duration<double>(now - t_last).count());
      t_last = now;
    }
    cur = next;
  };
  check_csr(H, "H");
  check_csr(Jc, "Jc");
  if (Jd.n > 0 || Jd.nnz() > 0) check_csr(Jd, "Jd");
  if (Ds.n > 0) check_csr(Ds, "Ds");
  if (H.n != H.m) throw std::runtime_error("H must be square");
  if (Jc.m != H.n) throw std::runtime_error("Jc must have n_x columns");
  if (Jd.nnz() > 0 && Jd.m != H.n) throw std::runtime_error("Jd must have n_x columns");
  S.n_x = H.n;
  S.m_c = Jc.n;
  S.m_d = Jd.n;
  S.nnz_h = H.nnz();
  S.nnz_jc = Jc.nnz();
  S.nnz_jd = Jd.nnz();
  S.nnz_ds = Ds.nnz();
  S.jd_flag = S.nnz_jd > 0;
  S.H = H;
  S.Jc = Jc;
  S.Jd = Jd;
  S.Ds = Ds;
  if (S.jd_flag) {
    // Ds is used as a diagonal in row order (row_scale reads ds[i] for row i,
    // src/matrix_vector_ops.cu:490-509)
    if (Ds.nnz() != S.m_d) throw std::runtime_error("Ds must hold one diagonal entry per Jd row");
  }
  S.JcT = transpose_pattern(Jc);
  if (S.jd_flag) S.JdT = transpose_pattern(Jd);
  const int n = S.n_x;

  phase("htilde");
  // ---- H~ = H + Jd^T Ds Jd ------------------------------------------------
  {
    CsrPattern emptyB;
    ProductUnion u = S.jd_flag ? product_union(H, Jd, S.JdT) : product_union(H, emptyB, S.JdT);
    S.Ht = std::move(u.pat);
    S.ht_hsrc = std::move(u.base_src);
    S.ht_cp = std::move(u.cp);
    S.ht_ca = std::move(u.ca);
    S.ht_cb = std::move(u.cb);
    S.ht_ck = std::move(u.ck);
  }
  phase("hgamma");
  // ---- Hgamma = H~ + gamma Jc^T Jc (full pattern, contributions kept) -----
  ProductUnion hg = product_union(S.Ht, Jc, S.JcT);
  S.Hg = hg.pat;

  phase("ordering");
  // ---- ordering -------------------------------------------------------------
  S.perm.resize(n);
  if (user_perm) {
    std::vector<char> seen(n, 0);
    for (int i = 0; i < n; ++i) {
      if (user_perm[i] < 0 || user_perm[i] >= n || seen[user_perm[i]])
        throw std::runtime_error("user permutation is not a permutation");
      seen[user_perm[i]] = 1;
      S.perm[i] = user_perm[i];
    }
    S.ordering_used = -1;
    S.ordering_note = "user";
  } else if (opt.ordering == ORDER_IDENTITY) {
    std::iota(S.perm.begin(), S.perm.end(), 0);
    S.ordering_used = ORDER_IDENTITY;
    S.ordering_note = "identity";
  } else {
    bool ok = false;
    if (opt.ordering == ORDER_AUTO || opt.ordering == ORDER_REFERENCE) {
      ok = order_reference_symamd(S.Hg, S.perm, S.ordering_note);
      if (ok) S.ordering_used = ORDER_REFERENCE;
      if (!ok && opt.ordering == ORDER_REFERENCE)
        throw std::runtime_error("reference ordering unavailable: " + S.ordering_note);
    }
    if (!ok) {
      order_builtin_amd(S.Hg, S.perm);
      S.ordering_used = ORDER_BUILTIN;
      if (S.ordering_note.empty()) S.ordering_note = "builtin";
      else S.ordering_note = "builtin (" + S.ordering_note + ")";
    }
  }
  S.rev_perm.assign(n, 0);
  for (int i = 0; i < n; ++i) S.rev_perm[S.perm[i]] = i;

  phase("lower");
  // ---- permuted lower triangle (CSC by permuted column) ---------------------
  const int nnz_hg = S.Hg.nnz();
  std::vector<int> lo_slot;  // Hg slot of each lower entry, grouped by column
  {
    std::vector<int> cnt(n + 1, 0);
    for (int i = 0; i < n; ++i)
      for (int p = S.Hg.rp[i]; p < S.Hg.rp[i + 1]; ++p) {
        int pi = S.rev_perm[i], pj = S.rev_perm[S.Hg.ci[p]];
        if (pi >= pj) cnt[pj + 1]++;
      }
    for (int j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
    S.lp_cp = cnt;
    const int nlo = cnt[n];
    S.lp_row.resize(nlo);
    lo_slot.resize(nlo);
    std::vector<int> next(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < n; ++i)
      for (int p = S.Hg.rp[i]; p < S.Hg.rp[i + 1]; ++p) {
        int pi = S.rev_perm[i], pj = S.rev_perm[S.Hg.ci[p]];
        if (pi >= pj) {
          int q = next[pj]++;
          S.lp_row[q] = pi;
          lo_slot[q] = p;
        }
      }
    // sort rows within each column
    std::vector<std::pair<int, int>> tmp;
    for (int j = 0; j < n; ++j) {
      tmp.clear();
      for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q) tmp.push_back({S.lp_row[q], lo_slot[q]});
      std::sort(tmp.begin(), tmp.end());
      for (int q = S.lp_cp[j], t = 0; q < S.lp_cp[j + 1]; ++q, ++t) {
        S.lp_row[q] = tmp[t].first;
        lo_slot[q] = tmp[t].second;
      }
    }
    S.lp_htsrc.resize(nlo);
    S.lp_ccp.assign(nlo + 1, 0);
    for (int q = 0; q < nlo; ++q) {
      int s = lo_slot[q];
      S.lp_htsrc[q] = hg.base_src[s];
      S.lp_ccp[q + 1] = S.lp_ccp[q] + (hg.cp[s + 1] - hg.cp[s]);
    }
    S.lp_ca.resize(S.lp_ccp[nlo]);
    S.lp_cb.resize(S.lp_ccp[nlo]);
    for (int q = 0; q < nlo; ++q) {
      int s = lo_slot[q];
      for (int t = hg.cp[s], o = S.lp_ccp[q]; t < hg.cp[s + 1]; ++t, ++o) {
        S.lp_ca[o] = hg.ca[t];
        S.lp_cb[o] = hg.cb[t];
      }
    }
  }
  (void)nnz_hg;

  // lower rows (strictly below the diagonal) of the permuted matrix
  std::vector<int> lr_rp(n + 1, 0), lr_ci;
  for (int j = 0; j < n; ++j)
    for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q)
      if (S.lp_row[q] > j) lr_rp[S.lp_row[q] + 1]++;
  for (int i = 0; i < n; ++i) lr_rp[i + 1] += lr_rp[i];
  lr_ci.resize(lr_rp[n]);
  {
    std::vector<int> next(lr_rp.begin(), lr_rp.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q)
        if (S.lp_row[q] > j) lr_ci[next[S.lp_row[q]]++] = j;
  }

  phase("etree");
  // ---- elimination tree (Liu, path compression) -----------------------------
  S.parent.assign(n, -1);
  {
    std::vector<int> anc(n, -1);
    for (int k = 0; k < n; ++k)
      for (int p = lr_rp[k]; p < lr_rp[k + 1]; ++p) {
        int i = lr_ci[p];
        while (i != -1 && i < k) {
          int nxt = anc[i];
          anc[i] = k;
          if (nxt == -1) S.parent[i] = k;
          i = nxt;
        }
      }
  }
  phase("colcounts");
  // ---- column counts by row-subtree traversal ------------------------------
  S.colcount.assign(n, 1);
  {
    std::vector<int> mark(n, -1);
    for (int k = 0; k < n; ++k) {
      mark[k] = k;
      for (int p = lr_rp[k]; p < lr_rp[k + 1]; ++p) {
        int j = lr_ci[p];
        while (j != -1 && mark[j] != k) {
          S.colcount[j]++;
          mark[j] = k;
          j = S.parent[j];
        }
      }
    }
  }
  S.nnz_L = 0;
  S.factor_flops = 0;
  for (int j = 0; j < n; ++j) {
    S.nnz_L += S.colcount[j];
    S.factor_flops += (double)S.colcount[j] * (double)S.colcount[j];
  }

  phase("supernodes");
  // ---- fundamental supernodes ----------------------------------------------
  std::vector<int> nchild(n, 0);
  for (int j = 0; j < n; ++j)
    if (S.parent[j] >= 0) nchild[S.parent[j]]++;
  std::vector<int> fs_first;
  for (int j = 0; j < n; ++j) {
    bool join = j > 0 && S.parent[j - 1] == j && S.colcount[j - 1] == S.colcount[j] + 1 && nchild[j] == 1;
    if (!join) fs_first.push_back(j);
  }
  fs_first.push_back(n);
  const int nfs = (int)fs_first.size() - 1;
  std::vector<int> fs_of(n);
  for (int J = 0; J < nfs; ++J)
    for (int c = fs_first[J]; c < fs_first[J + 1]; ++c) fs_of[c] = J;

  // ---- relaxed amalgamation: merge a supernode into its parent when the two
  // are contiguous and the merged front carries few explicit zeros ----------
  std::vector<int> grp(nfs);
  std::iota(grp.begin(), grp.end(), 0);  // representative = group's topmost fundamental supernode
  std::vector<int> g_first(nfs), g_ncols(nfs), g_nrows(nfs);
  std::vector<double> g_zeros(nfs, 0.0);
  for (int J = 0; J < nfs; ++J) {
    g_first[J] = fs_first[J];
    g_ncols[J] = fs_first[J + 1] - fs_first[J];
    g_nrows[J] = S.colcount[fs_first[J]];
  }
  std::vector<int> group_of(nfs);
  std::iota(group_of.begin(), group_of.end(), 0);
  auto find = [&](int x) {
    while (group_of[x] != x) { group_of[x] = group_of[group_of[x]]; x = group_of[x]; }
    return x;
  };
  if (opt.relax) {
    for (int J = 0; J < nfs; ++J) {
      int g = find(J);
      int last = fs_first[J + 1] - 1;  // J is the top of its group (groups grow upwards)
      int pc = S.parent[last];
      if (pc < 0) continue;
      int P = fs_of[pc];
      int gp = find(P);
      if (pc != last + 1 || g_first[gp] != pc) continue;  // not contiguous
      int ncols_m = g_ncols[g] + g_ncols[gp];
      int nrows_m = g_ncols[g] + g_nrows[gp];
      int r_g = g_nrows[g] - g_ncols[g];
      double extra = (double)g_ncols[g] * (double)(g_nrows[gp] - r_g);
      double zeros = g_zeros[g] + g_zeros[gp] + extra;
      double stored = 0;
      for (int c = 0; c < ncols_m; ++c) stored += nrows_m - c;
      double zf = zeros / stored;
      bool merge = ncols_m <= 4 || (ncols_m <= 16 && zf <= 0.8) || (ncols_m <= 48 && zf <= 0.1) ||
                   zf <= 0.05;
      if (!merge) continue;
      group_of[gp] = g;  // g becomes representative of the merged group
      g_ncols[g] = ncols_m;
      g_nrows[g] = nrows_m;
      g_zeros[g] = zeros;
      // g_first[g] unchanged (lower columns)
    }
  }
  // final supernodes: groups in column order
  S.sn_first.clear();
  for (int J = 0; J < nfs; ++J) {
    int g = find(J);
    if (g == J) S.sn_first.push_back(fs_first[J]);
  }
  S.sn_first.push_back(n);
  S.nsn = (int)S.sn_first.size() - 1;
  const int nsn = S.nsn;
  S.sn_of.resize(n);
  for (int J = 0; J < nsn; ++J)
    for (int c = S.sn_first[J]; c < S.sn_first[J + 1]; ++c) S.sn_of[c] = J;

  phase("rows");
  // ---- rows(J) = cols(J) U struct(L(:, last(J))) ------------------------------
  {
    std::vector<int> is_last(n, -1);
    for (int J = 0; J < nsn; ++J) is_last[S.sn_first[J + 1] - 1] = J;
    std::vector<std::vector<int>> rstruct(nsn);
    std::vector<int> mark(n, -1);
    for (int k = 0; k < n; ++k) {
      mark[k] = k;
      for (int p = lr_rp[k]; p < lr_rp[k + 1]; ++p) {
        int j = lr_ci[p];
        while (j != -1 && mark[j] != k) {
          if (is_last[j] >= 0) rstruct[is_last[j]].push_back(k);
          mark[j] = k;
          j = S.parent[j];
        }
      }
    }
    S.sn_rp.assign(nsn + 1, 0);
    S.sn_nrows.resize(nsn);
    for (int J = 0; J < nsn; ++J) {
      S.sn_nrows[J] = (S.sn_first[J + 1] - S.sn_first[J]) + (int)rstruct[J].size();
      S.sn_rp[J + 1] = S.sn_rp[J] + S.sn_nrows[J];
    }
    S.sn_rows.resize(S.sn_rp[nsn]);
    for (int J = 0; J < nsn; ++J) {
      int o = S.sn_rp[J];
      for (int c = S.sn_first[J]; c < S.sn_first[J + 1]; ++c) S.sn_rows[o++] = c;
      for (int r : rstruct[J]) S.sn_rows[o++] = r;
    }
  }
  // supernodal tree
  S.sn_parent.assign(nsn, -1);
  for (int J = 0; J < nsn; ++J) {
    int last = S.sn_first[J + 1] - 1;
    if (S.parent[last] >= 0) S.sn_parent[J] = S.sn_of[S.parent[last]];
  }
  S.sn_child_rp.assign(nsn + 1, 0);
  for (int J = 0; J < nsn; ++J)
    if (S.sn_parent[J] >= 0) S.sn_child_rp[S.sn_parent[J] + 1]++;
  for (int J = 0; J < nsn; ++J) S.sn_child_rp[J + 1] += S.sn_child_rp[J];
  S.sn_children.resize(S.sn_child_rp[nsn]);
  {
    std::vector<int> next(S.sn_child_rp.begin(), S.sn_child_rp.end() - 1);
    for (int J = 0; J < nsn; ++J)
      if (S.sn_parent[J] >= 0) S.sn_children[next[S.sn_parent[J]]++] = J;
  }
  // relative maps R_J -> positions in rows(P)
  S.sn_relp.assign(nsn + 1, 0);
  for (int J = 0; J < nsn; ++J) {
    int ncols = S.sn_first[J + 1] - S.sn_first[J];
    S.sn_relp[J + 1] = S.sn_relp[J] + (S.sn_nrows[J] - ncols);
  }
  S.sn_rel.resize(S.sn_relp[nsn]);
  for (int J = 0; J < nsn; ++J) {
    int P = S.sn_parent[J];
    int ncols = S.sn_first[J + 1] - S.sn_first[J];
    int nR = S.sn_nrows[J] - ncols;
    if (nR == 0) continue;
    if (P < 0) throw std::runtime_error("symbolic: root supernode with rows below the diagonal");
    const int* pr = &S.sn_rows[S.sn_rp[P]];
    int pn = S.sn_nrows[P];
    int t = 0;
    for (int r = 0; r < nR; ++r) {
      int row = S.sn_rows[S.sn_rp[J] + ncols + r];
      while (t < pn && pr[t] < row) ++t;
      if (t == pn || pr[t] != row) throw std::runtime_error("symbolic: child rows not contained in parent rows");
      S.sn_rel[S.sn_relp[J] + r] = t;
    }
  }
  // levels
  S.sn_level.assign(nsn, 0);
  for (int J = 0; J < nsn; ++J)
    if (S.sn_parent[J] >= 0) S.sn_level[S.sn_parent[J]] = std::max(S.sn_level[S.sn_parent[J]], S.sn_level[J] + 1);
  S.nlevels = 0;
  for (int J = 0; J < nsn; ++J) S.nlevels = std::max(S.nlevels, S.sn_level[J] + 1);
  S.flevels.assign(S.nlevels, FactorLevel());
  for (int J = 0; J < nsn; ++J) {
    FactorLevel& L = S.flevels[S.sn_level[J]];
    int ncols = S.sn_first[J + 1] - S.sn_first[J];
    if (S.sn_nrows[J] <= opt.small_front_max) L.small.push_back(J);
    else {
      L.large.push_back(J);
      L.max_panels = std::max(L.max_panels, (ncols + opt.panel - 1) / opt.panel);
    }
  }
  // front arena
  S.sn_off.resize(nsn + 1);
  S.sn_off[0] = 0;
  S.L_stored = 0;
  for (int J = 0; J < nsn; ++J) {
    int64_t nj = S.sn_nrows[J];
    S.sn_off[J + 1] = S.sn_off[J] + nj * nj;
    S.L_stored += nj * (int64_t)(S.sn_first[J + 1] - S.sn_first[J]);
  }
  S.front_arena = S.sn_off[nsn];

  // local row of every lower entry inside its column's front
  {
    const int nlo = S.lp_cp[n];
    S.lp_lrow.resize(nlo);
    for (int j = 0; j < n; ++j) {
      int J = S.sn_of[j];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      int nr = S.sn_nrows[J];
      int t = 0;
      for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q) {
        int row = S.lp_row[q];
        while (t < nr && rows[t] < row) ++t;
        if (t == nr || rows[t] != row) throw std::runtime_error("symbolic: entry outside its supernode structure");
        S.lp_lrow[q] = t;
      }
    }
  }

  phase("items");
  // ---- triangular-solve items ----------------------------------------------
  {
    S.sq_sn.clear(); S.sq_c0.clear(); S.sq_c1.clear(); S.sq_level.clear();
    std::vector<int> last_item(nsn, -1);
    for (int J = 0; J < nsn; ++J) {
      int ncols = S.sn_first[J + 1] - S.sn_first[J];
      int lvl0 = 0;
      for (int c = S.sn_child_rp[J]; c < S.sn_child_rp[J + 1]; ++c)
        lvl0 = std::max(lvl0, S.sq_level[last_item[S.sn_children[c]]] + 1);
      int prev = -1;
      for (int c0 = 0; c0 < ncols; c0 += opt.solve_piece) {
        int c1 = std::min(ncols, c0 + opt.solve_piece);
        int lv = prev < 0 ? lvl0 : S.sq_level[prev] + 1;
        S.sq_sn.push_back(J);
        S.sq_c0.push_back(c0);
        S.sq_c1.push_back(c1);
        S.sq_level.push_back(lv);
        prev = (int)S.sq_sn.size() - 1;
      }
      last_item[J] = prev;
    }
    S.nsq = (int)S.sq_sn.size();
    S.nsq_levels = 0;
    for (int q = 0; q < S.nsq; ++q) S.nsq_levels = std::max(S.nsq_levels, S.sq_level[q] + 1);
    S.sq_level_rp.assign(S.nsq_levels + 1, 0);
    for (int q = 0; q < S.nsq; ++q) S.sq_level_rp[S.sq_level[q] + 1]++;
    for (int l = 0; l < S.nsq_levels; ++l) S.sq_level_rp[l + 1] += S.sq_level_rp[l];
    S.sq_level_items.resize(S.nsq);
    {
      std::vector<int> next(S.sq_level_rp.begin(), S.sq_level_rp.end() - 1);
      for (int q = 0; q < S.nsq; ++q) S.sq_level_items[next[S.sq_level[q]]++] = q;
    }
    S.sq_uoff.resize(S.nsq + 1);
    S.sq_uoff[0] = 0;
    for (int q = 0; q < S.nsq; ++q) {
      int J = S.sq_sn[q];
      S.sq_uoff[q + 1] = S.sq_uoff[q] + (S.sn_nrows[J] - S.sq_c1[q]);
    }
    S.u_arena = S.sq_uoff[S.nsq];
    // gather lists
    S.g_rp.assign(n + 1, 0);
    for (int q = 0; q < S.nsq; ++q) {
      int J = S.sq_sn[q];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      for (int t = S.sq_c1[q]; t < S.sn_nrows[J]; ++t) S.g_rp[rows[t] + 1]++;
    }
    for (int i = 0; i < n; ++i) S.g_rp[i + 1] += S.g_rp[i];
    S.g_pos.resize(S.g_rp[n]);
    std::vector<int> next(S.g_rp.begin(), S.g_rp.end() - 1);
    for (int q = 0; q < S.nsq; ++q) {
      int J = S.sq_sn[q];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      for (int t = S.sq_c1[q]; t < S.sn_nrows[J]; ++t)
        S.g_pos[next[rows[t]]++] = S.sq_uoff[q] + (t - S.sq_c1[q]);
    }
  }

  phase("schedule");
  build_solve_schedule(S, opt.chunk_fma, opt.unit_cols, opt.warp_subtree);

  phase("jc");
  // ---- permuted Jc structures for the Schur CG -------------------------------
  S.jcp_ci.resize(S.nnz_jc);
  for (int p = 0; p < S.nnz_jc; ++p) S.jcp_ci[p] = S.rev_perm[Jc.ci[p]];
  S.jctp_rp.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    int o = S.perm[i];
    S.jctp_rp[i + 1] = S.jctp_rp[i] + (S.JcT.pat.rp[o + 1] - S.JcT.pat.rp[o]);
  }
  S.jctp_ci.resize(S.nnz_jc);
  S.jctp_src.resize(S.nnz_jc);
  for (int i = 0; i < n; ++i) {
    int o = S.perm[i];
    int d = S.jctp_rp[i];
    for (int p = S.JcT.pat.rp[o]; p < S.JcT.pat.rp[o + 1]; ++p, ++d) {
      S.jctp_ci[d] = S.JcT.pat.ci[p];
      S.jctp_src[d] = S.JcT.src[p];
    }
  }
  phase("");
  return S;
}

namespace {
// a row panel unit of a staged item: its columns and its task argument
struct Unit {
  int cols, arg;
};
// units of equal width keep their order: the widest units are claimed first
// and the short ones fill the end of the stage (longest-processing-time order)
std::vector<Unit> largest_first(std::vector<Unit> u) {
  std::stable_sort(u.begin(), u.end(), [](const Unit& a, const Unit& b) { return a.cols > b.cols; });
  return u;
}
}  // namespace

void build_solve_schedule(Symbolic& S, int chunk_fma, int unit_cols, int warp_subtree) {
  if (unit_cols < 64 || unit_cols > kMaxUnitCols) throw std::invalid_argument("solve unit columns outside [64, 2048]");
  if (warp_subtree > kMaxSubtree) throw std::invalid_argument("warp subtree size above 64");
  S.unit_cols = unit_cols;
  const int nsq = S.nsq;
  std::vector<int> item_of_col(S.n_x);
  for (int q = 0; q < nsq; ++q)
    for (int c = S.sq_c0[q]; c < S.sq_c1[q]; ++c) item_of_col[S.sn_first[S.sq_sn[q]] + c] = q;
  S.sq_mode.assign(nsq, 0);
  S.sq_rows_x.assign(nsq, 0);
  S.sq_doff.assign(nsq + 1, 0);
  S.ch0.assign(nsq, 0);
  S.nch.assign(nsq, 0);
  S.ch_row0.clear();
  S.ch_rows.clear();
  S.ch_item.clear();
  S.ch_poff.clear();
  int64_t poff = 0;
  for (int q = 0; q < nsq; ++q) {
    const int J = S.sq_sn[q];
    const int ncols = S.sq_c1[q] - S.sq_c0[q];
    const int nrow = S.sn_nrows[J] - S.sq_c0[q];
    const int nR = nrow - ncols;
    int mode = ITEM_STAGED;
    if (nrow <= kWarpItemRows) mode = ITEM_WARP;
    else if (nrow <= kSmallItemRows && ncols <= 64) mode = ITEM_FUSED;
    else if (ncols <= 64) mode = ITEM_HEAD;
    S.sq_mode[q] = mode;
    S.sq_doff[q + 1] = S.sq_doff[q] + (int64_t)ncols * ncols;
    // rows per product task: a power of two in 16..256 giving about
    // chunk_fma multiply-adds per task.  FP64 runs at ~2 multiply-adds per
    // clock per SM, so a 4k task is ~1 us of one SM: small tasks spread an
    // item's rows over many SMs, which shortens the dependency chain, and
    // their blocks fit the task's shared memory (staged while waiting).
    int rows = 256;
    while (rows > 16 && (int64_t)rows * ncols > chunk_fma) rows >>= 1;
    S.sq_rows_x[q] = rows;
    S.ch0[q] = (int)S.ch_row0.size();
    if (nR > 0) {
      const bool panelized = mode == ITEM_STAGED && ncols > unit_cols;
      const int step = (mode == ITEM_WARP || mode == ITEM_FUSED) ? nR : panelized ? unit_cols : rows;  // one chunk for one-task items
      for (int r = 0; r < nR; r += step) {
        S.ch_row0.push_back(r);
        S.ch_rows.push_back(std::min(step, nR - r));
        S.ch_item.push_back(q);
        S.ch_poff.push_back(poff);
        poff += ncols;
      }
    }
    S.nch[q] = (int)S.ch_row0.size() - S.ch0[q];
  }
  S.dinv_arena = S.sq_doff[nsq];
  S.part_arena = poff;
  S.sq_l21f.assign(nsq, -1);
  S.sq_l21b.assign(nsq, -1);
  S.l21f_arena = S.l21b_arena = 0;
  S.bd_need.assign(nsq, 0);
  for (int q = 0; q < nsq; ++q) {
    const int nc = S.sq_c1[q] - S.sq_c0[q], nR = S.sn_nrows[S.sq_sn[q]] - S.sq_c1[q];
    S.bd_need[q] = S.nch[q];
    if (S.sq_mode[q] != ITEM_STAGED || nc <= unit_cols || nR <= 0) continue;
    if (S.sq_rows_x[q] != 16) throw std::runtime_error("panelized item: 16 rows per forward task expected");
    S.sq_l21f[q] = S.l21f_arena;
    S.l21f_arena += (int64_t)((nR + 15) / 16) * 16 * nc;
    S.sq_l21b[q] = S.l21b_arena;
    S.l21b_arena += (int64_t)((nc + 15) / 16) * 16 * nR;
    S.bd_need[q] = S.nch[q] * ((nc + 15) / 16);
  }
  S.sq_xpoff.assign(nsq, -1);
  S.sq_pcoff.assign(nsq, -1);
  S.sq_ppoff.assign(nsq, -1);
  S.xpanel_arena = 0;
  S.npanels = 0;
  S.ppart_arena = 0;
  for (int q = 0; q < nsq; ++q) {
    if (S.sq_mode[q] != ITEM_STAGED) continue;
    const int nc = S.sq_c1[q] - S.sq_c0[q], RT = S.sq_rows_x[q];
    const int np = (nc + RT - 1) / RT;
    S.sq_xpoff[q] = S.xpanel_arena;
    S.xpanel_arena += xpanel_total(RT, nc);
    S.sq_pcoff[q] = S.npanels;
    S.npanels += np;
    S.sq_ppoff[q] = S.ppart_arena;
    S.ppart_arena += (int64_t)np * ((nc + unit_cols - 1) / unit_cols) * RT;
  }
  for (int q = 0; q < nsq; ++q)
    if (S.sq_c1[q] - S.sq_c0[q] >= (1 << kUnitShift)) throw std::runtime_error("solve item too wide");
  if ((int64_t)S.ch_row0.size() >= (1 << kUnitShift)) throw std::runtime_error("too many solve chunks");
  const int nch = (int)S.ch_row0.size();
  // chunk -> distinct items owning its rows (rows ascending, so items ascending)
  S.ct_rp.assign(nch + 1, 0);
  S.ct_item.clear();
  S.diag_need.assign(nsq, 0);
  for (int c = 0; c < nch; ++c) {
    const int q = S.ch_item[c], J = S.sq_sn[q];
    const int* rows = &S.sn_rows[S.sn_rp[J]];
    const int lo = S.sq_c1[q] + S.ch_row0[c], hi = lo + S.ch_rows[c];
    int last = -1;
    for (int lr = lo; lr < hi; ++lr) {
      const int it = item_of_col[rows[lr]];
      if (it != last) {
        S.ct_item.push_back(it);
        S.diag_need[it]++;
        last = it;
      }
    }
    S.ct_rp[c + 1] = (int)S.ct_item.size();
  }
  // item -> chunks with rows in its columns
  S.ic_rp.assign(nsq + 1, 0);
  S.ic_chunk.assign(S.ct_item.size(), 0);
  for (int it : S.ct_item) S.ic_rp[it + 1]++;
  for (int q = 0; q < nsq; ++q) S.ic_rp[q + 1] += S.ic_rp[q];
  {
    std::vector<int> nx(S.ic_rp.begin(), S.ic_rp.end() - 1);
    for (int c = 0; c < nch; ++c)
      for (int p = S.ct_rp[c]; p < S.ct_rp[c + 1]; ++p) S.ic_chunk[nx[S.ct_item[p]]++] = c;
  }
  // forward look-ahead: parents, parent rows, child dot lists, forward
  // chunks and gather lists without the parent rows
  S.sq_parent.assign(nsq, -1);
  S.sq_rpar.assign(nsq, 0);
  S.nchild.assign(nsq, 0);
  S.fch0.assign(nsq, 0);
  S.nfch.assign(nsq, 0);
  S.fch_row0.clear();
  S.fch_rows.clear();
  for (int q = 0; q < nsq; ++q) {
    const int J = S.sq_sn[q];
    const int* rows = &S.sn_rows[S.sn_rp[J]];
    const int c1 = S.sq_c1[q], nJ = S.sn_nrows[J];
    const int nR = nJ - c1;
    int rp = 0;
    // head items only: their parent rows would otherwise take a separate
    // row-chunk task (warp, fused and staged items keep computing them)
    if (nR > 0 && S.sq_mode[q] == ITEM_HEAD) {
      const int p = item_of_col[rows[c1]];
      S.sq_parent[q] = p;
      S.nchild[p]++;
      while (rp < nR && item_of_col[rows[c1 + rp]] == p) ++rp;
    }
    S.sq_rpar[q] = rp;
    S.fch0[q] = (int)S.fch_row0.size();
    const int mode = S.sq_mode[q];
    const int step = (mode == ITEM_WARP || mode == ITEM_FUSED) ? std::max(nR - rp, 1) : S.sq_rows_x[q];
    for (int r = rp; r < nR; r += step) {
      S.fch_row0.push_back(r);
      S.fch_rows.push_back(std::min(step, nR - r));
    }
    S.nfch[q] = (int)S.fch_row0.size() - S.fch0[q];
  }
  {
    // column units of the forward chunks of wide items
    const int nf = (int)S.fch_row0.size();
    S.fch_slot.assign(nf, -1);
    S.fslot_arena = 0;
    for (int q = 0; q < nsq; ++q) {
      const int nc = S.sq_c1[q] - S.sq_c0[q];
      if (S.sq_mode[q] != ITEM_STAGED || nc <= unit_cols) continue;
      const int nu = (nc + unit_cols - 1) / unit_cols;
      for (int c = S.fch0[q]; c < S.fch0[q] + S.nfch[q]; ++c) {
        S.fch_slot[c] = S.fslot_arena;
        S.fslot_arena += (int64_t)nu * S.sq_rows_x[q];
      }
    }
  }
  {
    const int nf = (int)S.fch_row0.size();
    S.fct_rp.assign(nf + 1, 0);
    S.fct_item.clear();
    S.fdiag_need.assign(nsq, 0);
    for (int q = 0; q < nsq; ++q) {
      const int J = S.sq_sn[q];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      for (int c = S.fch0[q]; c < S.fch0[q] + S.nfch[q]; ++c) {
        const int lo = S.sq_c1[q] + S.fch_row0[c], hi = lo + S.fch_rows[c];
        int last = -1;
        for (int lr = lo; lr < hi; ++lr) {
          const int it = item_of_col[rows[lr]];
          if (it != last) {
            S.fct_item.push_back(it);
            S.fdiag_need[it]++;
            last = it;
          }
        }
        S.fct_rp[c + 1] = (int)S.fct_item.size();
      }
    }
    // child dot lists (children in item order) and gather lists (forward chunk rows)
    const int n = S.n_x;
    S.cd_rp.assign(n + 1, 0);
    S.g_rp.assign(n + 1, 0);
    for (int q = 0; q < nsq; ++q) {
      const int J = S.sq_sn[q];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      const int c1 = S.sq_c1[q], nJ = S.sn_nrows[J];
      for (int t = c1; t < nJ; ++t) {
        if (t - c1 < S.sq_rpar[q]) S.cd_rp[rows[t] + 1]++;
        else S.g_rp[rows[t] + 1]++;
      }
    }
    for (int i = 0; i < n; ++i) {
      S.cd_rp[i + 1] += S.cd_rp[i];
      S.g_rp[i + 1] += S.g_rp[i];
    }
    S.cd_item.assign(S.cd_rp[n], 0);
    S.cd_lr.assign(S.cd_rp[n], 0);
    S.cd_loff.assign(S.cd_rp[n], 0);
    S.cd_ld.assign(S.cd_rp[n], 0);
    S.cd_nc.assign(S.cd_rp[n], 0);
    S.cd_x.assign(S.cd_rp[n], 0);
    S.g_pos.assign(S.g_rp[n], 0);
    std::vector<int> nxc(S.cd_rp.begin(), S.cd_rp.end() - 1), nxg(S.g_rp.begin(), S.g_rp.end() - 1);
    for (int q = 0; q < nsq; ++q) {
      const int J = S.sq_sn[q];
      const int* rows = &S.sn_rows[S.sn_rp[J]];
      const int c1 = S.sq_c1[q], nJ = S.sn_nrows[J];
      for (int t = c1; t < nJ; ++t) {
        if (t - c1 < S.sq_rpar[q]) {
          const int e = nxc[rows[t]]++;
          S.cd_item[e] = q;
          S.cd_lr[e] = t;
          S.cd_ld[e] = nJ;
          S.cd_nc[e] = c1 - S.sq_c0[q];
          S.cd_x[e] = S.sn_first[J] + S.sq_c0[q];
          S.cd_loff[e] = (int64_t)S.sq_c0[q] * nJ + t;  // front-relative; the engine adds the front offset
        } else {
          S.g_pos[nxg[rows[t]]++] = S.sq_uoff[q] + (t - c1);
        }
      }
    }
  }

  // warp subtrees: an item is eligible when it is a warp item and all its
  // children (items whose first row below lies in its columns) are eligible;
  // eligible subtrees of 2..warp_subtree items become one task each (a larger
  // subtree is split into its children's subtrees, its root left alone)
  std::vector<int> in_sub(nsq, 0);
  S.sg_rp.assign(1, 0);
  S.sg_item.clear();
  S.sg_lvl.clear();
  {
    std::vector<int> ipar(nsq, -1);
    std::vector<std::vector<int>> kids(nsq);
    for (int q = 0; q < nsq; ++q) {
      const int J = S.sq_sn[q];
      if (S.sq_c1[q] < S.sn_nrows[J]) {
        ipar[q] = item_of_col[S.sn_rows[S.sn_rp[J] + S.sq_c1[q]]];
        kids[ipar[q]].push_back(q);
      }
    }
    std::vector<char> elig(nsq, 0);
    std::vector<int> size(nsq, 0);
    for (int l = 0; l < S.nsq_levels; ++l)
      for (int t = S.sq_level_rp[l]; t < S.sq_level_rp[l + 1]; ++t) {
        const int q = S.sq_level_items[t];
        if (S.sq_mode[q] != ITEM_WARP) continue;
        bool ok = true;
        int sz = 1;
        for (int c : kids[q]) {
          ok = ok && elig[c];
          sz += size[c];
        }
        elig[q] = ok;
        size[q] = ok ? sz : 0;
      }
    // tops of the eligible subtrees, then depth first into the children of
    // every top too large to be one task (an explicit stack: a chain of warp
    // items can be as long as the matrix)
    std::vector<int> todo, stack, members;
    for (int q = nsq - 1; q >= 0; --q)
      if (elig[q] && (ipar[q] < 0 || !elig[ipar[q]])) todo.push_back(q);
    while (!todo.empty()) {
      const int q = todo.back();
      todo.pop_back();
      if (size[q] > std::max(warp_subtree, 1)) {
        for (auto c = kids[q].rbegin(); c != kids[q].rend(); ++c) todo.push_back(*c);
        continue;
      }
      if (size[q] < 2) continue;
      members.clear();
      stack.assign(1, q);
      while (!stack.empty()) {
        const int v = stack.back();
        stack.pop_back();
        members.push_back(v);
        for (int c : kids[v]) stack.push_back(c);
      }
      std::stable_sort(members.begin(), members.end(), [&](int a, int b) { return S.sq_level[a] < S.sq_level[b]; });
      for (int v : members) {
        S.sg_item.push_back(v);
        S.sg_lvl.push_back(S.sq_level[v]);
        in_sub[v] = 1;
      }
      S.sg_rp.push_back((int)S.sg_item.size());
    }
  }

  // warp items grouped by level, up to kWarpsPerTask per group
  S.wg_rp.assign(1, 0);
  S.wg_item.clear();
  std::vector<int> level_wg0(S.nsq_levels + 1, 0);
  for (int l = 0; l < S.nsq_levels; ++l) {
    level_wg0[l] = (int)S.wg_rp.size() - 1;
    int in_group = 0;
    for (int t = S.sq_level_rp[l]; t < S.sq_level_rp[l + 1]; ++t) {
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] != ITEM_WARP || in_sub[q]) continue;
      S.wg_item.push_back(q);
      if (++in_group == kWarpsPerTask) {
        S.wg_rp.push_back((int)S.wg_item.size());
        in_group = 0;
      }
    }
    if (in_group) S.wg_rp.push_back((int)S.wg_item.size());
  }
  level_wg0[S.nsq_levels] = (int)S.wg_rp.size() - 1;
  // task queues in topological order: within a level, every stage of all
  // items of the level before the next stage
  S.tf_kind.clear(); S.tf_item.clear(); S.tf_arg.clear();
  S.tb_kind.clear(); S.tb_item.clear(); S.tb_arg.clear();
  auto pushf = [&](int k, int q, int a) { S.tf_kind.push_back(k); S.tf_item.push_back(q); S.tf_arg.push_back(a); };
  auto pushb = [&](int k, int q, int a) { S.tb_kind.push_back(k); S.tb_item.push_back(q); S.tb_arg.push_back(a); };
  auto ncols_of = [&](int q) { return S.sq_c1[q] - S.sq_c0[q]; };
  const int nsub = (int)S.sg_rp.size() - 1;
  // forward: warp subtrees depend on nothing outside themselves, so they
  // open the queue, the deepest (longest sequential chain) first
  {
    std::vector<int> order(nsub);
    for (int g = 0; g < nsub; ++g) order[g] = g;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return S.sg_lvl[S.sg_rp[a + 1] - 1] > S.sg_lvl[S.sg_rp[b + 1] - 1]; });
    for (int g : order) pushf(T_WSUB, S.sg_item[S.sg_rp[g + 1] - 1], g);
  }
  for (int l = 0; l < S.nsq_levels; ++l) {
    const int t0 = S.sq_level_rp[l], t1 = S.sq_level_rp[l + 1];
    for (int g = level_wg0[l]; g < level_wg0[l + 1]; ++g) pushf(T_WARP, S.wg_item[S.wg_rp[g]], g);
    for (int t = t0; t < t1; ++t) {
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] == ITEM_FUSED) pushf(T_FUSED, q, 0);
      else if (S.sq_mode[q] == ITEM_HEAD) pushf(T_HEAD, q, 0);
      else if (S.sq_mode[q] == ITEM_STAGED)
        for (int c = 0; c < ncols_of(q); c += kColChunk) pushf(T_GATHER, q, c);
    }
    for (int t = t0; t < t1; ++t) {  // row panel units, largest first
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] != ITEM_STAGED) continue;
      const int nc = ncols_of(q), RT = S.sq_rows_x[q];
      std::vector<Unit> units;
      for (int b = (nc - 1) / RT; b >= 0; --b) {
        const int K = std::min(nc, (b + 1) * RT);
        for (int u = 0; u * unit_cols < K; ++u) units.push_back({std::min(unit_cols, K - u * unit_cols), b | (u << kUnitShift)});
      }
      for (const Unit& u : largest_first(units)) pushf(T_INV, q, u.arg);
    }
    for (int t = t0; t < t1; ++t) {
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] == ITEM_HEAD || S.sq_mode[q] == ITEM_STAGED) {
        const int nu = S.fch0[q] < (int)S.fch_slot.size() && S.nfch[q] > 0 && S.fch_slot[S.fch0[q]] >= 0
                           ? (ncols_of(q) + unit_cols - 1) / unit_cols
                           : 1;
        for (int c = S.fch0[q]; c < S.fch0[q] + S.nfch[q]; ++c)
          for (int u = 0; u < nu; ++u) pushf(T_L21, q, c | (u << kUnitShift));
      }
    }
  }
  for (int l = S.nsq_levels - 1; l >= 0; --l) {
    const int t0 = S.sq_level_rp[l], t1 = S.sq_level_rp[l + 1];
    // backward: a warp subtree at its root's level (it waits on the root's rows)
    for (int g = 0; g < nsub; ++g)
      if (S.sg_lvl[S.sg_rp[g + 1] - 1] == l) pushb(T_WSUB, S.sg_item[S.sg_rp[g + 1] - 1], g);
    for (int g = level_wg0[l]; g < level_wg0[l + 1]; ++g) pushb(T_WARP, S.wg_item[S.wg_rp[g]], g);
    for (int t = t0; t < t1; ++t) {
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] == ITEM_FUSED) pushb(T_FUSED, q, 0);
      else if (S.sq_mode[q] != ITEM_WARP) {
        const int npan = S.sq_l21b[q] >= 0 ? (ncols_of(q) + 15) / 16 : 1;  // panelized: one task per 16 columns
        for (int c = S.ch0[q]; c < S.ch0[q] + S.nch[q]; ++c)
          for (int b = 0; b < npan; ++b) pushb(T_L21T, q, c | (b << kUnitShift));
      }
    }
    for (int t = t0; t < t1; ++t) {
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] == ITEM_HEAD) pushb(T_TAIL, q, 0);
      else if (S.sq_mode[q] == ITEM_STAGED && S.nch[q] > 0)  // without rows below: y' = x, kept by the forward INV
        for (int c = 0; c < ncols_of(q); c += kColChunk) pushb(T_REDUCE, q, c);
    }
    for (int t = t0; t < t1; ++t) {  // row panel units of X^T, largest first
      const int q = S.sq_level_items[t];
      if (S.sq_mode[q] != ITEM_STAGED) continue;
      const int nc = ncols_of(q), RT = S.sq_rows_x[q];
      std::vector<Unit> units;
      for (int b = 0; b * RT < nc; ++b) {
        const int K = nc - b * RT;
        for (int u = 0; u * unit_cols < K; ++u) units.push_back({std::min(unit_cols, K - u * unit_cols), b | (u << kUnitShift)});
      }
      for (const Unit& u : largest_first(units)) pushb(T_INVT, q, u.arg);
    }
  }
}

void structural_L(const Symbolic& S, std::vector<int>& cp, std::vector<int>& ri) {
  const int n = S.n_x;
  cp.assign(n + 1, 0);
  for (int j = 0; j < n; ++j) cp[j + 1] = cp[j] + S.colcount[j];
  ri.resize(cp[n]);
  std::vector<int> next(cp.begin(), cp.end() - 1);
  for (int j = 0; j < n; ++j) ri[next[j]++] = j;  // diagonal first (smallest row)
  // lower rows of the permuted matrix
  std::vector<int> lr_rp(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q)
      if (S.lp_row[q] > j) lr_rp[S.lp_row[q] + 1]++;
  for (int i = 0; i < n; ++i) lr_rp[i + 1] += lr_rp[i];
  std::vector<int> lr_ci(lr_rp[n]);
  {
    std::vector<int> nx(lr_rp.begin(), lr_rp.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int q = S.lp_cp[j]; q < S.lp_cp[j + 1]; ++q)
        if (S.lp_row[q] > j) lr_ci[nx[S.lp_row[q]]++] = j;
  }
  std::vector<int> mark(n, -1);
  for (int k = 0; k < n; ++k) {
    mark[k] = k;
    for (int p = lr_rp[k]; p < lr_rp[k + 1]; ++p) {
      int j = lr_ci[p];
      while (j != -1 && mark[j] != k) {
        ri[next[j]++] = k;
        mark[j] = k;
        j = S.parent[j];
      }
    }
  }
}

}  // namespace hykkt
