"""The task schedule of the persistent triangular solves, emulated on the CPU.

The GPU kernels claim tasks in queue order and wait on dependency counters.
Here one "CTA" runs the queues sequentially: every wait must already be
satisfied when its task is claimed (the queues are topological, so no
claimed task can wait on an unclaimed one), and the dataflow through the
update arena u, the gather lists, the staged vectors and the partial-sum
chunks must reproduce L L^T x = b as a dense triangular solve does.
Task kinds follow SolveTask (symbolic.hpp): 0 fused, 1 gather, 2 inverse,
3 rows below, 4 rows below transposed, 5 reduce, 6 inverse transposed,
7 warp items, 8 head, 9 tail, 10 warp subtree; item modes follow ItemMode: 0 warp, 1 fused,
2 head, 3 staged.
"""
import numpy as np
import pytest
import scipy.linalg as sla

import helpers as H
import hykkt_gb300 as hk

FUSED, GATHER, INV, L21, L21T, REDUCE, INVT, WARP, HEAD, TAIL, WSUB = range(11)
M_WARP, M_FUSED, M_HEAD, M_STAGED = range(4)
COL_CHUNK = 32
UNIT_SHIFT = 20


def emulate(sym, Ld, b):
    INV_SEG = int(sym["unit_cols"][0])
    n = len(b)
    g = {k: sym[k] for k in ("sn_first", "sn_nrows", "sn_rp", "sn_rows", "sq_sn", "sq_c0", "sq_c1", "sq_uoff",
                              "sq_mode", "sq_rows_x", "wg_rp", "wg_item", "sq_parent", "sq_rpar", "nchild", "cd_rp",
                              "cd_item", "cd_lr", "fch_row0", "fch_rows", "fch0", "nfch", "fct_rp", "fct_item", "fch_slot", "sq_l21b",
                              "bd_need", "sg_rp", "sg_item", "sg_lvl", "sq_level",
                              "fdiag_need", "g_rp", "g_pos", "ch_row0", "ch_rows", "ch_item", "ch0", "nch",
                              "ch_poff", "ct_rp", "ct_item", "diag_need", "ic_rp", "ic_chunk", "tf_kind", "tf_item",
                              "tf_arg", "tb_kind", "tb_item", "tb_arg")}
    nsq = len(g["sq_sn"])
    nchk = len(g["ch_row0"])
    u = np.zeros(int(g["sq_uoff"][-1]) + 1)
    ncs = g["sq_c1"] - g["sq_c0"]
    part = np.zeros(int(ncs[g["ch_item"]].sum()) + 1)
    x = np.zeros(n)
    sv = np.full(n, np.nan)
    sv2 = np.full(n, np.nan)  # x of the staged items without rows below, kept by the forward pass
    diag_cnt = np.zeros(nsq, int)
    g_done = np.zeros(nsq, int)
    inv_done = np.zeros(nsq, int)
    slots = {}

    def item(q):
        J = g["sq_sn"][q]
        rows = g["sn_rows"][g["sn_rp"][J]:g["sn_rp"][J + 1]]
        c0, c1 = g["sq_c0"][q], g["sq_c1"][q]
        cols = g["sn_first"][J] + np.arange(c0, c1)
        return c0, c1, g["sn_nrows"][J], rows, cols

    def chunk_rows(q, ch):
        c0, c1, nJ, rows, cols = item(q)
        r0 = g["ch_row0"][ch]
        lrs = np.arange(c1 + r0, c1 + r0 + g["ch_rows"][ch])
        assert lrs[-1] < nJ
        return lrs

    child_done = np.zeros(nsq, int)

    def gathered(c):
        """b - (updates of the forward chunks) - (children's dot products)"""
        v = b[c] - u[g["g_pos"][g["g_rp"][c]:g["g_rp"][c + 1]]].sum()
        for e in range(g["cd_rp"][c], g["cd_rp"][c + 1]):
            qc, lr = g["cd_item"][e], g["cd_lr"][e]
            _, _, _, rows_c, cols_c = item(qc)
            assert rows_c[lr] == c
            v -= Ld[rows_c[lr], cols_c] @ x[cols_c]
        return v

    def ready(q):
        assert diag_cnt[q] == g["fdiag_need"][q] and child_done[q] == g["nchild"][q], q

    def x_done(q):  # x_q complete: the parent may use it
        if g["sq_parent"][q] >= 0:
            child_done[g["sq_parent"][q]] += 1

    def fchunk_rows(q, ch):
        c0, c1, nJ, rows, cols = item(q)
        r0 = g["fch_row0"][ch]
        return np.arange(c1 + r0, c1 + r0 + g["fch_rows"][ch])

    def fsignal(ch):
        for p in range(g["fct_rp"][ch], g["fct_rp"][ch + 1]):
            diag_cnt[g["fct_item"][p]] += 1

    def one_task_fwd(q):
        c0, c1, nJ, rows, cols = item(q)
        nc = c1 - c0
        X = sla.solve_triangular(Ld[np.ix_(cols, cols)], np.eye(nc), lower=True)
        ready(q)
        x[cols] = X @ np.array([gathered(c) for c in cols])
        assert g["nfch"][q] <= 1
        for ch in range(g["fch0"][q], g["fch0"][q] + g["nfch"][q]):
            lrs = fchunk_rows(q, ch)
            assert lrs[0] == c1 + g["sq_rpar"][q] and lrs[-1] == nJ - 1
            u[g["sq_uoff"][q] + (lrs - c1)] = Ld[np.ix_(rows[lrs], cols)] @ x[cols]
            fsignal(ch)
        x_done(q)

    for kind, q, arg in zip(g["tf_kind"], g["tf_item"], g["tf_arg"]):
        if kind == WARP:
            grp = g["wg_item"][g["wg_rp"][arg]:g["wg_rp"][arg + 1]]
            assert 1 <= len(grp) <= 8 and grp[0] == q
            for qq in grp:
                c0, c1, nJ, rows, cols = item(qq)
                assert g["sq_mode"][qq] == M_WARP and nJ - c0 <= 32
                one_task_fwd(qq)
            continue
        if kind == WSUB:  # members leaves first; their contributors are earlier members
            grp = g["sg_item"][g["sg_rp"][arg]:g["sg_rp"][arg + 1]]
            assert 2 <= len(grp) <= 64 and grp[-1] == q
            assert np.all(np.diff(g["sg_lvl"][g["sg_rp"][arg]:g["sg_rp"][arg + 1]]) >= 0)
            # one level runs concurrently: a member's parent sits on a higher level
            col_item = {int(c): int(qq) for qq in grp for c in item(qq)[4]}
            for qq in grp:
                _, c1m, nJm, rows_m, _ = item(qq)
                if c1m < nJm and int(rows_m[c1m]) in col_item:
                    assert g["sq_level"][col_item[int(rows_m[c1m])]] > g["sq_level"][qq]
            for qq in grp:
                assert g["sq_mode"][qq] == M_WARP
                one_task_fwd(qq)
            continue
        c0, c1, nJ, rows, cols = item(q)
        nc = c1 - c0
        X = sla.solve_triangular(Ld[np.ix_(cols, cols)], np.eye(nc), lower=True)
        RT = g["sq_rows_x"][q]
        mode = g["sq_mode"][q]
        if kind == FUSED:
            assert mode == M_FUSED and nJ - c0 <= 256 and nc <= 64
            one_task_fwd(q)
        elif kind == HEAD:
            assert mode == M_HEAD and nc <= 64
            ready(q)
            x[cols] = X @ np.array([gathered(c) for c in cols])
            inv_done[q] += 1
            x_done(q)
        elif kind == GATHER:
            assert mode == M_STAGED
            ready(q)
            for c in cols[arg:arg + COL_CHUNK]:
                sv[c] = gathered(c)
            g_done[q] += 1
        elif kind == INV:
            assert g_done[q] == -(-nc // COL_CHUNK)
            b_, unit = arg & ((1 << UNIT_SHIFT) - 1), arg >> UNIT_SHIFT
            K = min(nc, (b_ + 1) * RT)
            k = np.arange(unit * INV_SEG, min(K, (unit + 1) * INV_SEG))
            r = np.arange(b_ * RT, min(nc, b_ * RT + RT))
            key = ("f", q, b_)
            slots.setdefault(key, []).append((unit, X[np.ix_(r, k)] @ sv[cols[k]]))
            if len(slots[key]) == -(-K // INV_SEG):
                x[cols[r]] = sum(v for _, v in sorted(slots[key], key=lambda uv: uv[0]))
                if g["nch"][q] == 0:
                    sv2[cols[r]] = x[cols[r]]
                inv_done[q] += 1
                if inv_done[q] == -(-nc // RT):
                    x_done(q)
        else:
            assert kind == L21 and mode in (M_HEAD, M_STAGED)
            assert inv_done[q] == (1 if mode == M_HEAD else -(-nc // RT))
            ch, unit = arg & ((1 << UNIT_SHIFT) - 1), arg >> UNIT_SHIFT
            lrs = fchunk_rows(q, ch)
            assert lrs[0] >= c1 + g["sq_rpar"][q]
            if g["fch_slot"][ch] < 0:
                assert unit == 0
                u[g["sq_uoff"][q] + (lrs - c1)] = Ld[np.ix_(rows[lrs], cols)] @ x[cols]
                fsignal(ch)
            else:
                # column units of a wide item's chunk: partials summed in unit order by the last
                assert mode == M_STAGED and nc > INV_SEG
                k = np.arange(unit * INV_SEG, min(nc, (unit + 1) * INV_SEG))
                key = ("l21", ch)
                slots.setdefault(key, []).append((unit, Ld[np.ix_(rows[lrs], cols[k])] @ x[cols[k]]))
                if len(slots[key]) == -(-nc // INV_SEG):
                    u[g["sq_uoff"][q] + (lrs - c1)] = sum(v for _, v in sorted(slots[key], key=lambda uv: uv[0]))
                    fsignal(ch)
    assert np.array_equal(diag_cnt, g["fdiag_need"]) and np.array_equal(child_done, g["nchild"])
    y = x.copy()
    bg_cnt = np.zeros(nchk, int)
    bd_cnt = np.zeros(nsq, int)
    red_done = np.zeros(nsq, int)
    invt_done = np.zeros(nsq, int)
    done = np.zeros(nsq, bool)
    sv[:] = np.nan

    def finish(q):
        assert not done[q]
        done[q] = True
        for p in range(g["ic_rp"][q], g["ic_rp"][q + 1]):
            bg_cnt[g["ic_chunk"][p]] += 1

    def one_task_bwd(q):
        c0, c1, nJ, rows, cols = item(q)
        nc = c1 - c0
        X = sla.solve_triangular(Ld[np.ix_(cols, cols)], np.eye(nc), lower=True)
        if g["nch"][q]:
            ch = g["ch0"][q]
            assert bg_cnt[ch] == g["ct_rp"][ch + 1] - g["ct_rp"][ch]
        lrs = np.arange(c1, nJ)
        ys = x[cols] - Ld[np.ix_(rows[lrs], cols)].T @ x[rows[lrs]]
        x[cols] = X.T @ ys
        finish(q)

    def head_tail(q, X, cols):
        v = x[cols].copy()
        for ch in range(g["ch0"][q], g["ch0"][q] + g["nch"][q]):
            v -= part[g["ch_poff"][ch] + np.arange(len(cols))]
        x[cols] = X.T @ v
        finish(q)

    for kind, q, arg in zip(g["tb_kind"], g["tb_item"], g["tb_arg"]):
        if kind == WARP:
            for qq in g["wg_item"][g["wg_rp"][arg]:g["wg_rp"][arg + 1]]:
                one_task_bwd(qq)
            continue
        if kind == WSUB:
            # the kernel waits on the root's chunk alone: every row below a
            # member is a column of the subtree or a row below the root
            grp = g["sg_item"][g["sg_rp"][arg]:g["sg_rp"][arg + 1]]
            c0, c1, nJ, rows, cols = item(q)
            if g["nch"][q]:
                ch = g["ch0"][q]
                assert bg_cnt[ch] == g["ct_rp"][ch + 1] - g["ct_rp"][ch]
            inside = set(np.concatenate([item(qq)[4] for qq in grp]).tolist())
            root_rows = set(rows[c1:].tolist())
            for qq in grp:
                _, c1m, _, rows_m, _ = item(qq)
                assert set(rows_m[c1m:].tolist()) <= inside | root_rows, qq
            for qq in grp[::-1]:
                one_task_bwd(qq)
            continue
        c0, c1, nJ, rows, cols = item(q)
        nc = c1 - c0
        X = sla.solve_triangular(Ld[np.ix_(cols, cols)], np.eye(nc), lower=True)
        RT = g["sq_rows_x"][q]
        if kind == FUSED:
            one_task_bwd(q)
        elif kind == L21T:
            ch, pb = arg & ((1 << UNIT_SHIFT) - 1), arg >> UNIT_SHIFT
            assert bg_cnt[ch] == g["ct_rp"][ch + 1] - g["ct_rp"][ch]
            lrs = chunk_rows(q, ch)
            po = g["ch_poff"][ch]
            if g["sq_l21b"][q] >= 0:  # panelized: 16 columns per task
                t = np.arange(16 * pb, min(nc, 16 * pb + 16))
                part[po + t] = Ld[np.ix_(rows[lrs], cols[t])].T @ x[rows[lrs]]
            else:
                assert pb == 0
                part[po:po + nc] = Ld[np.ix_(rows[lrs], cols)].T @ x[rows[lrs]]
            bd_cnt[q] += 1
            # the chunk that completes a head item's partials finishes the item
            if g["sq_mode"][q] == M_HEAD and bd_cnt[q] == g["nch"][q]:
                head_tail(q, X, cols)
        elif kind == TAIL:
            # the queue keeps one task per head item; it finishes only an
            # item without chunks (the last chunk did the others)
            assert g["sq_mode"][q] == M_HEAD
            if g["nch"][q] == 0:
                head_tail(q, X, cols)
            assert done[q]
        elif kind == REDUCE:
            assert bd_cnt[q] == g["bd_need"][q]
            t = np.arange(arg, min(nc, arg + COL_CHUNK))
            v = x[cols[t]].copy()
            for ch in range(g["ch0"][q], g["ch0"][q] + g["nch"][q]):
                v -= part[g["ch_poff"][ch] + t]
            sv[cols[t]] = v
            red_done[q] += 1
        else:
            # an item without rows below has no REDUCE tasks: y' = x, kept by the forward INV
            own = g["nch"][q] == 0
            assert kind == INVT and red_done[q] == (0 if own else -(-nc // COL_CHUNK))
            b, unit = arg & ((1 << UNIT_SHIFT) - 1), arg >> UNIT_SHIFT
            K = nc - b * RT
            k = b * RT + np.arange(unit * INV_SEG, min(K, (unit + 1) * INV_SEG))
            r = np.arange(b * RT, min(nc, b * RT + RT))
            key = ("b", q, b)
            yv = sv2 if own else sv
            slots.setdefault(key, []).append((unit, X.T[np.ix_(r, k)] @ yv[cols[k]]))
            if len(slots[key]) == -(-K // INV_SEG):
                x[cols[r]] = sum(v for _, v in sorted(slots[key], key=lambda uv: uv[0]))
                invt_done[q] += 1
                if invt_done[q] == -(-nc // RT):
                    finish(q)
    assert done.all()
    return y, x


def dense_factor(s, sym):
    """Dense Cholesky of a random SPD matrix on the permuted Hgamma pattern."""
    n = s.n_x
    perm = sym["perm"]
    rp, ci = sym["hg_rp"], sym["hg_ci"]
    rng = np.random.default_rng(0)
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    vals = rng.uniform(-1, 1, len(ci))
    A[rows, ci] = vals
    A = (A + A.T) / 2
    A += np.diag(np.abs(A).sum(axis=1) + 1.0)
    Ap = A[np.ix_(perm, perm)]
    return np.linalg.cholesky(Ap)


@pytest.mark.parametrize("case", ["grid150", "a200_AC_00", "grid400_identity", "grid1500", "grid1500_pieces",
                                  "grid1500_pieces_subtrees", "grid1500_subtrees4", "a200_AC_10_pieces_subtrees",
                                  "chain_identity"])
def test_schedule_emulation(case, monkeypatch):
    if case.startswith("grid1500_pieces"):
        # supernodes wider than 48 columns split into pieces: updates between
        # pieces of one supernode go through the gather lists; pieces keep
        # warp items one per warp unless the subtree size is set
        if case.endswith("subtrees"):
            monkeypatch.setenv("HYKKT_SOLVE_WARP_SUBTREE", "16")
        s = H.small_grid_system(n_bus=1500, seed=3)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN, solve_piece=48)
        assert np.any(sym["sq_c0"] > 0)
        assert (len(sym["sg_rp"]) > 1) == case.endswith("subtrees")
    elif case == "a200_AC_10_pieces_subtrees":
        monkeypatch.setenv("HYKKT_SOLVE_WARP_SUBTREE", "16")
        s = H.load_system("a200_AC_10")
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN, solve_piece=16)
        assert np.any(sym["sq_c0"] > 0) and len(sym["sg_rp"]) > 1
    elif case == "chain_identity":
        # one long chain of warp items (tridiagonal Hessian in its own order):
        # the bottom of the chain is a subtree task, the rest single warps
        from hykkt_gb300 import gridgen as gg
        n = 3000
        i = np.arange(n)
        rows = np.concatenate([i, i[:-1], i[1:]])
        cols = np.concatenate([i, i[1:], i[:-1]])
        o = np.lexsort((cols, rows))
        rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int32)
        Hm = gg.CSR(n, n, rp, cols[o].astype(np.int32), np.concatenate([np.full(n, 4.0), np.full(2 * n - 2, -1.0)])[o])
        mc = n // 2
        Jc = gg.CSR(mc, n, (2 * np.arange(mc + 1)).astype(np.int32), np.arange(2 * mc).astype(np.int32), np.ones(2 * mc))
        jd = gg.CSR(0, n, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
        ds = gg.CSR(0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
        s = gg.KKTSystem(Hm, ds, Jc, jd, np.ones(n), np.zeros(0), np.ones(mc), np.zeros(0), 10.0)
        sym = hk.Symbolic(s, ordering=hk.ORDER_IDENTITY)
        assert len(sym["sg_rp"]) == 2
    elif case == "grid1500_subtrees4":
        monkeypatch.setenv("HYKKT_SOLVE_WARP_SUBTREE", "4")  # larger subtrees split into their children's
        s = H.small_grid_system(n_bus=1500, seed=3)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
        sizes = np.diff(sym["sg_rp"])
        assert len(sizes) > 0 and sizes.max() <= 4 and sizes.min() >= 2
    elif case == "grid150":
        s = H.small_grid_system(n_bus=150, seed=1)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    elif case == "grid400_identity":
        s = H.small_grid_system(n_bus=60, seed=2)
        sym = hk.Symbolic(s, ordering=hk.ORDER_IDENTITY)  # deep tree, wide dense supernodes
    elif case == "grid1500":
        s = H.small_grid_system(n_bus=1500, seed=3)  # staged items with several chunks
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    else:
        s = H.load_system(case)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    Ld = dense_factor(s, sym)
    b = np.random.default_rng(1).standard_normal(s.n_x)
    y, x = emulate(sym, Ld, b)
    assert np.allclose(y, sla.solve_triangular(Ld, b, lower=True), rtol=1e-10, atol=1e-10)
    assert np.allclose(x, sla.solve_triangular(Ld.T, y, lower=False), rtol=1e-9, atol=1e-9)


@pytest.mark.gpu
def test_schedule_emulation_reference_ordering():
    """The 500-bus workload under cusolverSpXcsrsymamdHost's ordering (it needs a
    CUDA context): the same schedule checks as above."""
    from hykkt_gb300 import gridgen as gg
    grid, systems = gg.workload_systems("grid500")
    s = systems[0]
    sym = hk.Symbolic(s, ordering=hk.ORDER_REFERENCE)
    Ld = dense_factor(s, sym)
    b = np.random.default_rng(1).standard_normal(s.n_x)
    y, x = emulate(sym, Ld, b)
    assert np.allclose(y, sla.solve_triangular(Ld, b, lower=True), rtol=1e-10, atol=1e-10)
    assert np.allclose(x, sla.solve_triangular(Ld.T, y, lower=False), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("case", ["a200_AC_10", "grid1500"])
def test_schedule_counts_consistent(case):
    if case == "grid1500":
        s = H.small_grid_system(n_bus=1500, seed=3)
    else:
        s = H.load_system(case)
    sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    ct_rp, ct_item, need = sym["ct_rp"], sym["ct_item"], sym["diag_need"]
    assert np.array_equal(np.bincount(ct_item, minlength=len(need)), need)
    assert sym["ic_rp"][-1] == ct_rp[-1]
    nc = sym["sq_c1"] - sym["sq_c0"]
    mode = sym["sq_mode"]
    rows_x = sym["sq_rows_x"]
    assert np.all((rows_x >= 16) & (rows_x <= 256) & ((rows_x & (rows_x - 1)) == 0))
    ng = -(-nc // COL_CHUNK)
    np_ = -(-nc // rows_x)
    INV_SEG = int(sym["unit_cols"][0])
    ninv = np.array([sum(-(-min(n, (b + 1) * r) // INV_SEG) for b in range(p)) for n, r, p in zip(nc, rows_x, np_)])
    ninvt = np.array([sum(-(-(n - b * r) // INV_SEG) for b in range(p)) for n, r, p in zip(nc, rows_x, np_)])
    nch = sym["nch"]
    assert np.all(nch[mode <= M_FUSED] <= 1)
    n_groups = len(sym["wg_rp"]) - 1 + len(sym["sg_rp"]) - 1
    nfch = sym["nfch"]
    assert np.all(nfch <= np.maximum(nch, 1))
    base = n_groups + (mode == M_FUSED).sum()
    nf = base + (1 + nfch)[mode == M_HEAD].sum() + (ng + nfch + ninv)[mode == M_STAGED].sum()
    # backward: REDUCE tasks only for staged items with rows below (y' = x otherwise)
    nb = base + (1 + nch)[mode == M_HEAD].sum() + (np.where(nch > 0, ng, 0) + nch + ninvt)[mode == M_STAGED].sum()
    assert len(sym["tf_kind"]) == len(sym["tf_item"]) == len(sym["tf_arg"]) == nf
    assert len(sym["tb_kind"]) == nb
    # look-ahead: every item with rows below has a parent, the parent rows
    # lead its R, and the child dot lists cover exactly those rows
    par, rpar = sym["sq_parent"], sym["sq_rpar"]
    assert np.all((par >= 0) == (rpar > 0))
    assert np.array_equal(np.bincount(par[par >= 0], minlength=len(par)), sym["nchild"])
    assert len(sym["cd_item"]) == rpar.sum()
    assert np.array_equal(np.sort(np.concatenate([sym["wg_item"], sym["sg_item"]])), np.flatnonzero(mode == M_WARP))
    if case == "grid1500":
        assert (mode == M_STAGED).any() and (mode == M_HEAD).any() and (mode == M_WARP).any()
