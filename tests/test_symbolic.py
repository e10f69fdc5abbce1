"""Host integer work of the product, bit-exact against the oracle (CPU).

The permutation maps, the H~/Hgamma patterns, the elimination tree and the
structural L pattern are integer results: they must match exactly.
"""
import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk
from oracle import oracle as O


def test_perm_maps_kat_product():
    """PermClass maps through the C ABI (examples/perm_driver.cpp:15-108)."""
    a_i, a_j = H.PERM_A_I, H.PERM_A_J
    r = hk.perm_maps(H.PERM_PERM, a_i, a_j, a_i, a_j, 4, a_i, a_j, 4)
    assert r["rc_rows"].tolist() == H.PERM_RC_I
    assert r["rc_cols"].tolist() == H.PERM_RC_J
    assert r["r_rows"].tolist() == H.PERM_R_I
    assert r["r_cols"].tolist() == H.PERM_R_J
    assert r["c_cols"].tolist() == H.PERM_C_J


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_perm_maps_random_vs_oracle(seed):
    rng = np.random.default_rng(seed)
    s = H.small_grid_system(n_bus=60, seed=seed)
    n = s.n_x
    perm = rng.permutation(n).astype(np.int32)
    JcT = H._transpose(s.m_c, n, s.Jc.rowptr, s.Jc.colidx, s.Jc.vals)
    p = hk.perm_maps(perm, s.H.rowptr, s.H.colidx, s.Jc.rowptr, s.Jc.colidx, s.m_c, JcT[0], JcT[1], n)
    o = O.perm_maps(perm, s.H.rowptr, s.H.colidx, s.m_c, s.Jc.rowptr, s.Jc.colidx, n, JcT[0], JcT[1])
    for k in o:
        assert np.array_equal(p[k], o[k]), k


def _oracle_patterns(s, perm):
    r = O.solve(s, perm=perm)
    return r


@pytest.mark.parametrize("name", ["a200_AC_09", "a200_AC_00", "a2000_AC_10"])
def test_symbolic_exact_fixtures(name):
    s = H.load_system(name)
    sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    perm = sym["perm"]
    assert sorted(perm.tolist()) == list(range(s.n_x))
    r = _oracle_patterns(s, perm)
    # H~ and Hgamma structure (SpGEMM + geam union, sorted)
    assert np.array_equal(sym["ht_rp"], r["ht_rp"])
    assert np.array_equal(sym["ht_ci"], r["ht_ci"])
    assert np.array_equal(sym["hg_rp"], r["hg_rp"])
    assert np.array_equal(sym["hg_ci"], r["hg_ci"])
    # elimination tree and the structural factor pattern for this ordering
    assert np.array_equal(sym["etree"], r["parent"])
    assert np.array_equal(sym["L_cp"], r["L_cp"])
    assert np.array_equal(sym["L_ri"], r["L_ri"])


def test_symbolic_user_perm_and_identity():
    s = H.small_grid_system(n_bus=50, seed=7)
    perm = np.random.default_rng(0).permutation(s.n_x).astype(np.int32)
    sym = hk.Symbolic(s, perm=perm)
    assert np.array_equal(sym["perm"], perm)
    r = O.solve(s, perm=perm)
    assert np.array_equal(sym["etree"], r["parent"])
    assert np.array_equal(sym["L_cp"], r["L_cp"])
    assert np.array_equal(sym["L_ri"], r["L_ri"])
    sym_id = hk.Symbolic(s, ordering=hk.ORDER_IDENTITY)
    assert np.array_equal(sym_id["perm"], np.arange(s.n_x))


def test_supernode_invariants():
    """Supernodes cover the columns contiguously; rows(J) start with J's own
    columns, are sorted, and contain the structure of every column of J."""
    s = H.load_system("a2000_AC_09")
    sym = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)
    first = sym["sn_first"]
    nrows = sym["sn_nrows"]
    rows = sym["sn_rows"]
    parent = sym["sn_parent"]
    Lcp, Lri = sym["L_cp"], sym["L_ri"]
    n = s.n_x
    assert first[0] == 0 and first[-1] == n and np.all(np.diff(first) > 0)
    off = np.concatenate([[0], np.cumsum(nrows)])
    for J in range(len(first) - 1):
        rj = rows[off[J]:off[J + 1]]
        assert np.all(np.diff(rj) > 0)
        assert np.array_equal(rj[: first[J + 1] - first[J]], np.arange(first[J], first[J + 1]))
        rset = set(rj.tolist())
        for c in range(first[J], first[J + 1]):
            assert set(Lri[Lcp[c]:Lcp[c + 1]].tolist()) <= rset
        if parent[J] >= 0:
            assert parent[J] > J


def test_pattern_errors_reported():
    """Unsorted columns and bad sizes are rejected with INVALID, not a crash."""
    s = H.small_grid_system(n_bus=20, seed=1)
    bad = s.H.copy()
    bad.colidx = bad.colidx.copy()
    bad.colidx[[0, 1]] = bad.colidx[[1, 0]]
    s.H = bad
    with pytest.raises(hk.HykktError) as e:
        hk.Symbolic(s)
    assert e.value.code == hk.INVALID


def test_long_chain_of_warp_items():
    """A tridiagonal Hessian in its own order (Jc pairing neighbours, no Jd): the
    elimination tree is one chain of 2,000,000 columns, 125,000 warp-sized items
    deep.  The analysis walks it without recursion and cuts it into subtree
    tasks of at most 16 items."""
    from hykkt_gb300 import gridgen as gg

    def csr(n, m, rows, cols, vals):
        o = np.lexsort((cols, rows))
        rp = np.zeros(n + 1, np.int64)
        np.add.at(rp, rows + 1, 1)
        return gg.CSR(n, m, np.cumsum(rp).astype(np.int32), cols[o].astype(np.int32), vals[o].astype(np.float64))

    n = 2_000_000
    i = np.arange(n)
    Hm = csr(n, n, np.concatenate([i, i[:-1], i[1:]]), np.concatenate([i, i[1:], i[:-1]]),
             np.concatenate([np.full(n, 4.0), np.full(2 * (n - 1), -1.0)]))
    mc = n // 2
    Jc = csr(mc, n, np.repeat(np.arange(mc), 2), np.arange(2 * mc), np.ones(2 * mc))
    jd = gg.CSR(0, n, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    ds = gg.CSR(0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    s = gg.KKTSystem(Hm, ds, Jc, jd, np.ones(n), np.zeros(0), np.ones(mc), np.zeros(0), 10.0)
    sym = hk.Symbolic(s, ordering=hk.ORDER_IDENTITY)
    levels = int(sym["sq_level"].max()) + 1
    assert levels == len(sym["sq_sn"]) > 100_000  # one chain
    sizes = np.diff(sym["sg_rp"])
    assert len(sizes) >= 1 and sizes.max() <= 16
