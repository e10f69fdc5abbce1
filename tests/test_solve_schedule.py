"""The task schedule of the persistent triangular solves, emulated on the CPU.

The GPU kernels claim tasks in queue order and wait on dependency counters.
Here one "CTA" runs the queues sequentially: every wait must already be
satisfied (the queues are topological, so no claimed task can wait on an
unclaimed one), and the dataflow through the update arena u, the gather
lists and the partial-sum chunks must reproduce L L^T x = b exactly as a
dense triangular solve does.
"""
import numpy as np
import pytest
import scipy.linalg as sla

import helpers as H
import hykkt_gb300 as hk


def emulate(sym, Ld, b):
    n = len(b)
    g = {k: sym[k] for k in ("sn_first", "sn_nrows", "sn_rp", "sn_rows", "sq_sn", "sq_c0", "sq_c1", "sq_uoff",
                              "g_rp", "g_pos", "ch_row0", "ch0", "nch", "ct_rp", "ct_item", "diag_need", "ic_rp",
                              "ic_chunk", "tf_item", "tf_chunk", "tb_item", "tb_chunk")}
    nsq = len(g["sq_sn"])
    nchk = len(g["ch_row0"])
    chunk_rows = 256
    u = np.zeros(int(g["sq_uoff"][-1]) + 1)
    x = np.zeros(n)
    diag_cnt = np.zeros(nsq, int)
    diag_done = np.zeros(nsq, bool)

    def item(q):
        J = g["sq_sn"][q]
        rows = g["sn_rows"][g["sn_rp"][J]:g["sn_rp"][J + 1]]
        return J, g["sq_c0"][q], g["sq_c1"][q], g["sn_first"][J], g["sn_nrows"][J], rows

    for q, ch in zip(g["tf_item"], g["tf_chunk"]):
        J, c0, c1, first, nJ, rows = item(q)
        cols = first + np.arange(c0, c1)
        if ch < 0:
            assert diag_cnt[q] == g["diag_need"][q]
            xs = np.array([b[c] - u[g["g_pos"][g["g_rp"][c]:g["g_rp"][c + 1]]].sum() for c in cols])
            xs = sla.solve_triangular(Ld[np.ix_(cols, cols)], xs, lower=True)
            x[cols] = xs
            diag_done[q] = True
        else:
            assert diag_done[q]
            r0 = g["ch_row0"][ch]
            lrs = np.arange(c1 + r0, min(nJ, c1 + r0 + chunk_rows))
            u[g["sq_uoff"][q] + (lrs - c1)] = Ld[np.ix_(rows[lrs], cols)] @ x[cols]
            for p in range(g["ct_rp"][ch], g["ct_rp"][ch + 1]):
                diag_cnt[g["ct_item"][p]] += 1
    y = x.copy()
    bg_cnt = np.zeros(nchk, int)
    bd_cnt = np.zeros(nsq, int)
    part = np.zeros((max(nchk, 1), 64))
    for q, ch in zip(g["tb_item"], g["tb_chunk"]):
        J, c0, c1, first, nJ, rows = item(q)
        cols = first + np.arange(c0, c1)
        if ch >= 0:
            assert bg_cnt[ch] == g["ct_rp"][ch + 1] - g["ct_rp"][ch]
            r0 = g["ch_row0"][ch]
            lrs = np.arange(c1 + r0, min(nJ, c1 + r0 + chunk_rows))
            part[ch, : len(cols)] = Ld[np.ix_(rows[lrs], cols)].T @ x[rows[lrs]]
            bd_cnt[q] += 1
        else:
            assert bd_cnt[q] == g["nch"][q]
            v = x[cols] - part[g["ch0"][q]:g["ch0"][q] + g["nch"][q], : len(cols)].sum(axis=0)
            x[cols] = sla.solve_triangular(Ld[np.ix_(cols, cols)].T, v, lower=False)
            for p in range(g["ic_rp"][q], g["ic_rp"][q + 1]):
                bg_cnt[g["ic_chunk"][p]] += 1
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


@pytest.mark.parametrize("case", ["grid150", "a200_AC_00", "grid400_identity"])
def test_schedule_emulation(case):
    if case == "grid150":
        s = H.small_grid_system(n_bus=150, seed=1)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    elif case == "grid400_identity":
        s = H.small_grid_system(n_bus=60, seed=2)
        sym = hk.Symbolic(s, ordering=hk.ORDER_IDENTITY)  # deep tree, wide dense supernodes
    else:
        s = H.load_system(case)
        sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    Ld = dense_factor(s, sym)
    b = np.random.default_rng(1).standard_normal(s.n_x)
    y, x = emulate(sym, Ld, b)
    assert np.allclose(y, sla.solve_triangular(Ld, b, lower=True), rtol=1e-10, atol=1e-10)
    assert np.allclose(x, sla.solve_triangular(Ld.T, y, lower=False), rtol=1e-9, atol=1e-9)


def test_schedule_counts_consistent():
    s = H.load_system("a200_AC_10")
    sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    ct_rp, ct_item, need = sym["ct_rp"], sym["ct_item"], sym["diag_need"]
    assert np.array_equal(np.bincount(ct_item, minlength=len(need)), need)
    assert len(sym["tf_item"]) == len(sym["tb_item"]) == len(sym["sq_sn"]) + len(sym["ch_row0"])
    assert sym["ic_rp"][-1] == ct_rp[-1]
