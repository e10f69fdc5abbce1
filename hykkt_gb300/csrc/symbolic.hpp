// Per-sparsity symbolic plan of the HyKKT KKT solve path.
//
// The reference recomputes structure through cuSPARSE on the first execute()
// and keeps it for later calls with the same sparsity (src/HykktSolver.cpp:254-279):
//   * H~ = H + Jd^T Ds Jd  pattern        (SpgemmClass, src/HykktSolver.cpp:685-697)
//   * Hgamma = H~ + gamma Jc^T Jc pattern (src/HykktSolver.cpp:352-367)
//   * symamd ordering + permutation maps  (src/HykktSolver.cpp:760-798)
//   * Cholesky analysis                   (src/CholeskyClass.cpp:31-58)
// Everything here is integer work done once per pattern on the host; the
// numeric phase (per system) only reads the arrays built here.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

namespace hykkt {

struct CsrPattern {
  int n = 0, m = 0;
  std::vector<int> rp;  // n+1
  std::vector<int> ci;  // nnz
  int nnz() const { return rp.empty() ? 0 : rp[n]; }
};

// Transpose of a CSR pattern: rows of the transpose are the columns of A,
// entries inside a row are in increasing original-row order (the order
// cusparseCsr2cscEx2 produces, src/cusparse_utils.cpp:49-98).  src[p] is the
// index of the entry in A's value array.
struct Transposed {
  CsrPattern pat;
  std::vector<int> src;
};
Transposed transpose_pattern(const CsrPattern& a);

enum Ordering : int {
  ORDER_AUTO = 0,       // reference symamd when available, else builtin
  ORDER_REFERENCE = 1,  // cusolverSpXcsrsymamdHost (the reference's call, PermClass.cpp:88-95)
  ORDER_BUILTIN = 2,    // approximate minimum degree written for this project
  ORDER_IDENTITY = 3,   // natural order (the Cholesky component tests factor as given)
};

struct SymbolicOptions {
  int ordering = ORDER_AUTO;
  int small_front_max = 96;  // fronts with n_J <= this are factored in shared memory
  int panel = 32;            // panel width of the blocked large-front factorization
  int solve_piece = 1 << 30; // max columns of one triangular-solve item (whole supernodes)
  int relax = 1;             // relaxed supernode amalgamation
  int chunk_fma = 4096;      // multiply-adds of one triangular-solve product task (sets rows per task)
  int unit_cols = 1024;      // columns of one unit of a staged item's panel product (64..kMaxUnitCols)
  int warp_subtree = 16;     // most items of one warp-subtree task (< 2: no subtree tasks; <= kMaxSubtree)
};

// Work item lists for one tree level of the factorization.
struct FactorLevel {
  std::vector<int> small;  // supernodes factored by one CTA in shared memory
  std::vector<int> large;  // supernodes factored by the blocked multi-CTA path
  int max_panels = 0;      // panels of the widest large front
};

struct Symbolic {
  // sizes
  int n_x = 0, m_c = 0, m_d = 0;
  int nnz_h = 0, nnz_jc = 0, nnz_jd = 0, nnz_ds = 0;
  bool jd_flag = false;

  // input patterns (copied)
  CsrPattern H, Jc, Jd, Ds;
  Transposed JcT, JdT;

  // H~ = H + Jd^T Ds Jd : full symmetric sorted pattern, per slot the H
  // source index (or -1) and the list of Jd contributions (a,b,k):
  // value = H[hsrc] + sum_k (Jd[a]*Jd[b]) * Ds[k], k ascending.
  CsrPattern Ht;
  std::vector<int> ht_hsrc;
  std::vector<int> ht_cp;               // nnz(H~)+1
  std::vector<int> ht_ca, ht_cb, ht_ck; // contributions

  // Hgamma = H~ + gamma Jc^T Jc : full symmetric sorted pattern (what the
  // ordering sees, the same structure cuSPARSE SpGEMM+geam produce).
  CsrPattern Hg;

  // ordering: perm[new] = old, rev_perm[old] = new (PermClass conventions,
  // src/PermClass.cpp:101-105, permcheck.cu:126-132)
  std::vector<int> perm, rev_perm;
  int ordering_used = ORDER_IDENTITY;
  std::string ordering_note;

  // permuted lower triangle of Hgamma in CSC (column = permuted column,
  // rows sorted); per entry: the H~ slot (or -1), the Jc contribution list
  // (pairs of Jc value indices), and the local position inside the front.
  std::vector<int> lp_cp;     // n_x+1
  std::vector<int> lp_row;    // permuted row
  std::vector<int> lp_htsrc;  // H~ slot or -1
  std::vector<int> lp_ccp;    // contributions offsets (nnz_lower+1)
  std::vector<int> lp_ca, lp_cb;
  std::vector<int> lp_lrow;   // row position inside rows(J) of the column's supernode

  // elimination tree and L structure (structural, before amalgamation)
  std::vector<int> parent;    // etree parent of each permuted column, -1 root
  std::vector<int> colcount;  // structural column counts of L (incl. diagonal)
  int64_t nnz_L = 0;          // structural nnz of L (sum of colcount)
  double factor_flops = 0;    // sum of colcount^2

  // supernodes
  int nsn = 0;
  std::vector<int> sn_first;  // nsn+1; columns [sn_first[J], sn_first[J+1])
  std::vector<int> sn_of;     // column -> supernode
  std::vector<int> sn_parent; // supernodal etree, -1 root
  std::vector<int> sn_nrows;  // n_J = |rows(J)| (diagonal block + R)
  std::vector<int> sn_rp;     // nsn+1 offsets into sn_rows
  std::vector<int> sn_rows;   // rows(J), sorted, starting with J's own columns
  std::vector<int64_t> sn_off;  // front offset (doubles); front is n_J x n_J col-major, ld n_J
  int64_t front_arena = 0;      // total doubles of all fronts
  int64_t L_stored = 0;         // sum n_J * ncols_J (stored L incl. explicit zeros)
  std::vector<int> sn_child_rp, sn_children;  // children lists (increasing)
  std::vector<int> sn_rel;    // for J with parent P: position in rows(P) of each R_J row; offsets sn_relp
  std::vector<int> sn_relp;   // nsn+1 (length |R_J| each)
  std::vector<int> sn_level;
  int nlevels = 0;
  std::vector<FactorLevel> flevels;

  // triangular-solve items: pieces of <= solve_piece columns of a supernode.
  // item q: supernode sq_sn, local columns [sq_c0, sq_c1) of that supernode.
  int nsq = 0;
  std::vector<int> sq_sn, sq_c0, sq_c1, sq_level;
  int nsq_levels = 0;
  std::vector<int> sq_level_rp, sq_level_items;  // items grouped by level
  // u-arena: item q writes u_q = L(rows below the item) * x_q at uoff[q]
  std::vector<int64_t> sq_uoff;
  int64_t u_arena = 0;
  // gather lists for the forward solve: for permuted column i, the u-arena
  // positions whose rows are i (ascending item order)
  std::vector<int> g_rp;      // n_x+1
  std::vector<int64_t> g_pos;

  // Task schedule of the persistent triangular solves.  Items are whole
  // supernodes (or column pieces); a diagonal block is applied through its
  // inverse X = L_qq^{-1} (computed after the factorization).  Per item mode
  // (nrow = n_J - c0 rows from the item's first column, nc columns):
  //   ITEM_WARP  (nrow <= 32): one warp per direction, 8 such items per task
  //   ITEM_FUSED (nrow <= 256, nc <= 64): one CTA task per direction
  //   ITEM_HEAD  (nc <= 64, more rows): forward HEAD (b', x = X b') then L21
  //              row chunks; backward L21T row chunks then TAIL (y', X^T y')
  //   ITEM_STAGED (nc > 64): forward GATHER (32-column chunks), INV (row
  //              panels of X), L21 (row chunks); backward L21T, REDUCE, INVT
  // "Chunks" (ch_*) are the row chunks below an item (one chunk for warp and
  // fused items); they carry the dependencies to and from the items owning
  // their rows (ct_*, ic_*, diag_need).
  std::vector<int> sq_mode;                      // per item: ItemMode
  std::vector<int> sq_rows_x;                    // rows per INV/INVT chunk (large items)
  std::vector<int64_t> sq_doff;                  // offsets of X (ncols^2) in the inverse arena
  int64_t dinv_arena = 0;
  // Large items also keep X as row panels of sq_rows_x (RT) rows, each
  // column-major with leading dimension RT, so that every product task
  // streams one contiguous block: forward panel b = rows [b RT, b RT + RT)
  // of X, columns [0, min(nc, (b+1) RT)); backward panel b = rows of X^T
  // (columns of X) [b RT, b RT + RT), columns k in [b RT, nc).  Offsets inside
  // an item's storage follow from RT and nc (xpanel_fwd / xpanel_bwd).
  std::vector<int64_t> sq_xpoff;                 // per item: start in the panel arena (-1: small item)
  int64_t xpanel_arena = 0;
  // A panel product is split into units of unit_cols columns; the units'
  // partial sums (RT each) meet in a per-panel slot, the last unit of a
  // panel adds them in order.  Per staged item: first panel counter and
  // first partial slot (ceil(nc / unit_cols) slots per panel).
  int unit_cols = 1024;
  std::vector<int> sq_pcoff;
  std::vector<int64_t> sq_ppoff;
  int npanels = 0;
  int64_t ppart_arena = 0;
  std::vector<int> ch_row0, ch_rows, ch_item, ch0, nch;  // L21 chunks: first row below, rows, item
  std::vector<int64_t> ch_poff;                  // offsets of the backward partial vectors (ncols each)
  int64_t part_arena = 0;
  std::vector<int> ct_rp, ct_item, diag_need;    // chunk -> distinct items owning its rows
  std::vector<int> ic_rp, ic_chunk;              // item -> chunks with rows in its columns
  std::vector<int> wg_rp, wg_item;               // groups of up to 8 warp items (same level)
  // Warp subtrees: small subtrees of the item tree whose items are all warp
  // items (the leaves of the elimination tree), each solved by one CTA level
  // by level with barriers instead of cross-CTA signals.  sg_item: members
  // by ascending item level (sg_lvl), the subtree root last.
  std::vector<int> sg_rp, sg_item, sg_lvl;
  // Forward look-ahead.  The leading rows of an item's R that are columns of
  // its parent item (the item owning R's first row) are multiplied by the
  // parent itself, from the item's fresh x (child dot products cd_*), so a
  // parent waits for its children's x only; the rest of R forms the item's
  // forward chunks (fch_*), whose products go through the update arena u
  // and the gather lists g_* (rebuilt here without the parent rows).
  std::vector<int> sq_parent;                    // parent item (-1: none)
  std::vector<int> sq_rpar;                      // leading rows of R in the parent's columns
  std::vector<int> nchild;                       // items whose parent is this item
  std::vector<int> cd_rp, cd_item, cd_lr;        // per permuted column: (child item, row in the child's front)
  std::vector<int64_t> cd_loff;                  // per entry: L(row, first column of the child) within its front
  std::vector<int> cd_ld, cd_nc, cd_x;           // per entry: front leading dimension, child columns, child's first column
  std::vector<int> fch_row0, fch_rows, fch0, nfch;  // forward chunks: first row below the item, rows
  std::vector<int> fct_rp, fct_item, fdiag_need;    // forward chunk -> distinct items owning its rows
  // Forward chunks of items wider than unit_cols are computed in column units
  // (task argument chunk | unit << kUnitShift); the units' partial sums (rows
  // of the chunk each) meet in the chunk's slot, the last unit adds them in
  // unit order.  fch_slot: per forward chunk, first slot entry (-1: one unit).
  std::vector<int64_t> fch_slot;
  int64_t fslot_arena = 0;
  // Panelized items (staged, wider than unit_cols, with rows below: the
  // column pieces of a wide supernode): their rows-below block L21 (R x nc)
  // is also stored packed, forward as 16-row chunks [col][16] (offset
  // sq_l21f + row0 * nc) and backward as 16-column panels [row][16] (offset
  // sq_l21b + panel * R * 16), so that every product task streams one
  // contiguous block.  Their backward chunks hold unit_cols rows and each
  // is split into one task per 16-column panel (argument chunk | panel <<
  // kUnitShift).  bd_need: backward product tasks of each item.
  std::vector<int64_t> sq_l21f, sq_l21b;
  int64_t l21f_arena = 0, l21b_arena = 0;
  std::vector<int> bd_need;
  // task queues: kind, item, argument (chunk id, first column, first row or warp group)
  std::vector<int> tf_kind, tf_item, tf_arg, tb_kind, tb_item, tb_arg;

  // Jc with permuted column indices (Jc_p = Jc P^T, values in Jc order)
  std::vector<int> jcp_ci;
  // Jc_p^T rows in permuted order: row i = Jc^T row perm[i]
  std::vector<int> jctp_rp, jctp_ci, jctp_src;
};

Symbolic build_symbolic(const CsrPattern& H, const CsrPattern& Ds, const CsrPattern& Jc,
                        const CsrPattern& Jd, const SymbolicOptions& opt,
                        const int* user_perm = nullptr);

// Task queues of the persistent triangular solves (called by build_symbolic).
enum ItemMode : int { ITEM_WARP = 0, ITEM_FUSED = 1, ITEM_HEAD = 2, ITEM_STAGED = 3 };
enum SolveTask : int {
  T_FUSED = 0,   // fused item, whole direction in one task
  T_GATHER = 1,  // forward: b' for a 32-column chunk
  T_INV = 2,     // forward: x rows = X b' (one unit of a row panel)
  T_L21 = 3,     // forward: u rows = L21 x (one row chunk)
  T_L21T = 4,    // backward: partial = L21^T x_R for one row chunk
  T_REDUCE = 5,  // backward: y' for a 32-column chunk
  T_INVT = 6,    // backward: x rows = X^T y' (one unit of a row panel of X^T)
  T_WARP = 7,    // up to 8 warp items, one per warp, whole direction
  T_HEAD = 8,    // forward: b' and x = X b' of a head item
  T_TAIL = 9,    // backward: y' and x = X^T y' of a head item
  T_WSUB = 10,   // a subtree of warp items in one CTA, level by level (both directions)
};
constexpr int kWarpItemRows = 32;    // warp items: n_J - c0 <= this
constexpr int kSmallItemRows = 256;  // fused items: n_J - c0 <= this and ncols <= 64
constexpr int kColChunk = 32;        // columns per GATHER / REDUCE task
constexpr int kWarpsPerTask = 8;     // warp items per T_WARP task
constexpr int kMaxSubtree = 64;      // largest warp_subtree setting
constexpr int kUnitShift = 20;       // INV / INVT argument: panel | (unit << kUnitShift)
constexpr int kMaxUnitCols = 2048;   // widest INV / INVT unit (its vector segment is staged whole)
void build_solve_schedule(Symbolic& S, int chunk_fma = 4096, int unit_cols = 1024, int warp_subtree = 16);

// Offsets of the row panels of a large item's X inside its panel storage
// (RT rows per panel, nc columns in the item); usable on host and device.
#if defined(__CUDACC__)
#define HYKKT_HD __host__ __device__
#else
#define HYKKT_HD
#endif
HYKKT_HD inline int64_t xpanel_fwd(int64_t RT, int64_t nc, int64_t b) {
  (void)nc;
  return RT * RT * (b * (b + 1) / 2);  // panels before b are unclipped: width (b'+1) RT
}
HYKKT_HD inline int64_t xpanel_fwd_total(int64_t RT, int64_t nc) {
  const int64_t np = (nc + RT - 1) / RT;
  return xpanel_fwd(RT, nc, np - 1) + RT * nc;
}
HYKKT_HD inline int64_t xpanel_bwd(int64_t RT, int64_t nc, int64_t b) {
  return xpanel_fwd_total(RT, nc) + RT * (b * nc - RT * (b * (b - 1) / 2));
}
HYKKT_HD inline int64_t xpanel_total(int64_t RT, int64_t nc) {
  const int64_t np = (nc + RT - 1) / RT;
  return xpanel_bwd(RT, nc, np);
}

// Process-wide lock around CUDA set-up and tear-down (allocation, frees,
// library handles) and around graph capture (engine.cu).  Plans solve
// concurrently from several host threads; a capture must not overlap another
// thread's device-wide calls (a cudaFree or a library handle's set-up can
// end it), and capture takes milliseconds once per plan, so these calls
// simply take turns.
std::mutex& cuda_setup_mutex();

// Orderings (ordering.cpp)
bool order_reference_symamd(const CsrPattern& A, std::vector<int>& perm, std::string& note);
void order_builtin_amd(const CsrPattern& A, std::vector<int>& perm);

// Structural L pattern of P A P^T (lower, by columns) -- used by the parity
// tests to show the symbolic factor is the exact one for the given ordering.
void structural_L(const Symbolic& S, std::vector<int>& cp, std::vector<int>& ri);

}  // namespace hykkt
