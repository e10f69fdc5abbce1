"""The CPU port's multithreaded configuration (oracle_set_threads > 1:
supernodal multifrontal Cholesky, parallel solves and CG loops) against the
pinned one-thread checker, and the H_gamma pattern that the reference's host
ordering is given.  CPU only."""
import numpy as np

import helpers as H
import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O
from oracle import ref_ordering as RO


def _solve(s, perm, threads, **kw):
    O.set_threads(threads)
    try:
        return O.solve(s, perm=perm, **kw)
    finally:
        O.set_threads(1)


def test_threaded_port_matches_checker():
    s = H.small_grid_system(n_bus=600, seed=11)
    perm = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)["perm"]
    kw = dict(itmax=5000, rtol=1e-11, refine_max=4, refine_target=1e-8, refine_rtol=1e-4)
    a = _solve(s, perm, 1, **kw)
    b = _solve(s, perm, 4, **kw)
    for k in ("x", "s", "y", "yd"):
        assert np.linalg.norm(a[k] - b[k]) <= 1e-11 * np.linalg.norm(a[k]), k
    assert b.scalar("rel_res_full") <= 1e-8
    assert abs(a.scalar("cg_iters") - b.scalar("cg_iters")) <= 3
    # a second threaded solve reuses the cached analysis and repeats itself exactly
    c = _solve(s, perm, 4, **kw)
    assert np.array_equal(b["x"], c["x"])


def test_threaded_port_identity_order_and_components():
    """Different ordering (identity: one long chain of supernodes) and the
    Cholesky component on its own."""
    s = H.small_grid_system(n_bus=150, seed=3)
    kw = dict(itmax=5000, rtol=1e-11, refine_max=2, refine_target=1e-8, refine_rtol=1e-4)
    a = _solve(s, None, 1, **kw)
    b = _solve(s, None, 3, **kw)
    assert np.linalg.norm(a["x"] - b["x"]) <= 1e-10 * np.linalg.norm(a["x"])
    rp, ci, v = a["hg_rp"], a["hg_ci"], a["hg_v"]
    rhs = np.random.default_rng(0).normal(size=s.n_x)
    O.set_threads(2)
    try:
        c = O.Chol(s.n_x, rp, ci, v, a["perm"])
        assert c.status == -1
        x = c.solve(rhs)
    finally:
        O.set_threads(1)
    import scipy.sparse as sp
    A = sp.csr_matrix((v, ci, rp), shape=(s.n_x, s.n_x))
    assert np.linalg.norm(A @ x - rhs) <= 1e-9 * np.linalg.norm(rhs) * max(1.0, abs(v).max())


def test_hgamma_pattern_matches_oracle():
    for seed, nb in ((1, 200), (2, 700)):
        s = H.small_grid_system(n_bus=nb, seed=seed)
        r = O.solve(s, itmax=1)
        rp, ci = RO.hgamma_pattern(s)
        assert np.array_equal(rp, r["hg_rp"]) and np.array_equal(ci, r["hg_ci"])
    # without inequality rows (Jd empty)
    s = H.load_system("a200_AC_00")
    r = O.solve(s, itmax=1)
    rp, ci = RO.hgamma_pattern(s)
    assert np.array_equal(rp, r["hg_rp"]) and np.array_equal(ci, r["hg_ci"])
