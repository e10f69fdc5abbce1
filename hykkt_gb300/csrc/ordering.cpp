// Fill-reducing orderings of the Hgamma pattern.
//
// * order_reference_symamd: the reference's own ordering call,
//   cusolverSpXcsrsymamdHost on the full symmetric Hgamma pattern with a
//   general zero-based descriptor (src/PermClass.cpp:88-95).  Loaded with
//   dlopen so the library has no link-time dependency on cuSOLVER; it needs a
//   GPU context (cusolverSpCreate fails without one), so on a machine without
//   a GPU the builtin ordering is used instead and the plan reports it.
// * order_builtin_amd: an approximate-minimum-degree ordering on the quotient
//   graph (Amestoy, Davis & Duff, "An approximate minimum degree ordering
//   algorithm", SIAM J. Matrix Anal. Appl. 17(4), 1996), written from the
//   paper: element absorption and the approximate external degree bound
//   d_i = min(n-k, d_i + |Lp\i|, |A_i\i| + |Lp\i| + sum_{e in E_i\p} |Le\Lp|).
//   No supervariable detection.  It is the fallback when the reference routine
//   is unavailable and is flagged "not reference-exact".
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <numeric>
#include <vector>

#include "symbolic.hpp"

namespace hykkt {

namespace {
typedef int (*fn_create_t)(void**);
typedef int (*fn_destroy_t)(void*);
typedef int (*fn_symamd_t)(void*, int, int, void*, const int*, const int*, int*);
typedef int (*fn_descr_create_t)(void**);
typedef int (*fn_descr_destroy_t)(void*);
}  // namespace

bool order_reference_symamd(const CsrPattern& A, std::vector<int>& perm, std::string& note) {
  void* hs = dlopen("libcusolver.so.12", RTLD_NOW | RTLD_LOCAL);
  if (!hs) hs = dlopen("libcusolver.so", RTLD_NOW | RTLD_LOCAL);
  void* hp = dlopen("libcusparse.so.12", RTLD_NOW | RTLD_LOCAL);
  if (!hp) hp = dlopen("libcusparse.so", RTLD_NOW | RTLD_LOCAL);
  if (!hs || !hp) {
    note = "cuSOLVER/cuSPARSE not loadable";
    return false;
  }
  auto create = (fn_create_t)dlsym(hs, "cusolverSpCreate");
  auto destroy = (fn_destroy_t)dlsym(hs, "cusolverSpDestroy");
  auto symamd = (fn_symamd_t)dlsym(hs, "cusolverSpXcsrsymamdHost");
  auto dcreate = (fn_descr_create_t)dlsym(hp, "cusparseCreateMatDescr");
  auto ddestroy = (fn_descr_destroy_t)dlsym(hp, "cusparseDestroyMatDescr");
  if (!create || !destroy || !symamd || !dcreate || !ddestroy) {
    note = "cuSOLVER symamd symbol missing";
    return false;
  }
  void* handle = nullptr;
  void* descr = nullptr;
  {
    // handle set-up touches the device: not while another thread captures
    std::lock_guard<std::mutex> lk(cuda_setup_mutex());
    if (create(&handle) != 0) {
      note = "cusolverSpCreate failed (no GPU context)";
      return false;
    }
    if (dcreate(&descr) != 0) {
      destroy(handle);
      note = "cusparseCreateMatDescr failed";
      return false;
    }
  }
  perm.assign(A.n, 0);
  int st = symamd(handle, A.n, A.nnz(), descr, A.rp.data(), A.ci.data(), perm.data());
  {
    std::lock_guard<std::mutex> lk(cuda_setup_mutex());
    ddestroy(descr);
    destroy(handle);
  }
  if (st != 0) {
    note = "cusolverSpXcsrsymamdHost failed";
    return false;
  }
  note = "reference symamd (cusolverSpXcsrsymamdHost)";
  return true;
}

void order_builtin_amd(const CsrPattern& A, std::vector<int>& perm) {
  const int n = A.n;
  perm.assign(n, 0);
  if (n == 0) return;
  std::vector<std::vector<int>> Av(n), Ev(n), Le(n);  // variable adjacency, element lists, element members
  for (int i = 0; i < n; ++i)
    for (int p = A.rp[i]; p < A.rp[i + 1]; ++p) {
      int j = A.ci[p];
      if (j != i) { Av[i].push_back(j); }
    }
  // symmetrise (input is expected symmetric; be safe)
  {
    std::vector<std::vector<int>> B(n);
    for (int i = 0; i < n; ++i)
      for (int j : Av[i]) { B[i].push_back(j); B[j].push_back(i); }
    for (int i = 0; i < n; ++i) {
      std::sort(B[i].begin(), B[i].end());
      B[i].erase(std::unique(B[i].begin(), B[i].end()), B[i].end());
      Av[i].swap(B[i]);
    }
  }
  std::vector<int> deg(n), state(n, 0);  // state: 0 variable, 1 element (eliminated), 2 absorbed element
  for (int i = 0; i < n; ++i) deg[i] = (int)Av[i].size();
  // bucket queue
  std::vector<int> head(n + 1, -1), nxt(n, -1), prv(n, -1);
  auto ins = [&](int i) {
    int d = std::min(deg[i], n);
    nxt[i] = head[d];
    prv[i] = -1;
    if (head[d] >= 0) prv[head[d]] = i;
    head[d] = i;
  };
  auto rem = [&](int i) {
    int d = std::min(deg[i], n);
    if (prv[i] >= 0) nxt[prv[i]] = nxt[i];
    else head[d] = nxt[i];
    if (nxt[i] >= 0) prv[nxt[i]] = prv[i];
  };
  for (int i = n - 1; i >= 0; --i) ins(i);
  std::vector<int> mark(n, -1), w(n, -1), wstamp(n, -1);
  int mind = 0;
  std::vector<int> Lp;
  for (int k = 0; k < n; ++k) {
    while (mind <= n && head[mind] < 0) ++mind;
    int p = head[mind];  // deterministic: most recently inserted of minimum degree
    rem(p);
    perm[k] = p;
    // Lp = (A_p U (U_{e in E_p} L_e)) \ {p}, uneliminated only
    Lp.clear();
    mark[p] = k;
    for (int j : Av[p]) if (state[j] == 0 && mark[j] != k) { mark[j] = k; Lp.push_back(j); }
    for (int e : Ev[p]) {
      if (state[e] != 1) continue;
      for (int j : Le[e]) if (state[j] == 0 && mark[j] != k) { mark[j] = k; Lp.push_back(j); }
      state[e] = 2;  // absorbed into p
      std::vector<int>().swap(Le[e]);
    }
    state[p] = 1;
    std::vector<int>().swap(Av[p]);
    std::vector<int>().swap(Ev[p]);
    Le[p] = Lp;
    // update lists of i in Lp
    for (int i : Lp) {
      // drop absorbed elements, add p
      auto& E = Ev[i];
      size_t o = 0;
      for (size_t t = 0; t < E.size(); ++t) if (state[E[t]] == 1 && E[t] != p) E[o++] = E[t];
      E.resize(o);
      E.push_back(p);
      // prune variables covered by Lp (and p itself)
      auto& V = Av[i];
      o = 0;
      for (size_t t = 0; t < V.size(); ++t) {
        int j = V[t];
        if (state[j] == 0 && mark[j] != k) V[o++] = j;
      }
      V.resize(o);
    }
    // |Le \ Lp| for elements adjacent to Lp.  Every member of a live
    // element is a variable (eliminating a member absorbs the element), so
    // |Le| is the list's length.
    for (int i : Lp)
      for (int e : Ev[i]) {
        if (e == p) continue;
        if (wstamp[e] != k) {
          wstamp[e] = k;
          w[e] = (int)Le[e].size();
        }
        w[e] -= 1;
      }
    const int lp = (int)Lp.size();
    const int remaining = n - k - 1;
    for (int i : Lp) {
      rem(i);
      long ext = (long)Av[i].size() + (lp - 1);
      for (int e : Ev[i]) if (e != p) ext += std::max(w[e], 0);
      long d = std::min<long>({(long)remaining - 1 < 0 ? 0 : remaining - 1, (long)deg[i] + lp - 1, ext});
      deg[i] = (int)std::max<long>(d, 0);
      ins(i);
      if (deg[i] < mind) mind = deg[i];
    }
  }
}

}  // namespace hykkt
