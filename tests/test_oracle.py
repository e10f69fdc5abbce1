"""The oracle pinned against the reference's own known-answer tests (CPU).

The oracle is the checker every GPU parity test relies on, so it is first
checked here against every known answer the reference's test drivers hold.
"""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O


def test_perm_maps_kat():
    """examples/perm_driver.cpp:15-108: exact integer maps for perm {2,0,3,1}."""
    a_i, a_j = H.PERM_A_I, H.PERM_A_J
    r = O.perm_maps(H.PERM_PERM, a_i, a_j, 4, a_i, a_j, 4, a_i, a_j)
    assert r["rc_rows"].tolist() == H.PERM_RC_I
    assert r["rc_cols"].tolist() == H.PERM_RC_J
    assert r["r_rows"].tolist() == H.PERM_R_I
    assert r["r_cols"].tolist() == H.PERM_R_J
    assert r["c_cols"].tolist() == H.PERM_C_J
    assert r["rev"].tolist() == [1, 3, 0, 2]


def test_ruiz_kat():
    """examples/Ruiz_driver.cpp:145-182: six scaled values within 1e-8."""
    Hm, A, At, rhs = H.ruiz_test_blocks()
    n = 1024
    hv, atv, av, r1, r2, md = O.ruiz_scale(2, n, n, (Hm.rowptr, Hm.colidx, Hm.vals), (At.rowptr, At.colidx, At.vals),
                                           (A.rowptr, A.colidx, A.vals), rhs[:n], rhs[n:])
    Hm.vals[:], A.vals[:], At.vals[:] = hv, av, atv
    got = H.ruiz_kat_values(Hm, A, At, np.concatenate([r1, r2]), md)
    for k, v in H.RUIZ_KAT.items():
        assert abs(got[k] - v) <= 1e-8, (k, got[k], v)


def test_cholesky_kat():
    """examples/cuSolver_driver_cholesky.cpp:32-75: lower-triangle a200 H
    factored in the given order, x[0] and x[6] within 3e-2."""
    z = np.load(H.GOLDEN + "/a200_chol.npz")
    n = int(z["H_shape"][0])
    A = H.coo_to_csr(n, n, z["H_r"], z["H_c"], z["H_v"])
    c = O.Chol(n, A.rowptr, A.colidx, A.vals)
    assert c.status == -1
    x = c.solve(z["rhs"])
    for i, v in H.CHOL_KAT.items():
        assert abs(x[i] - v) <= 3e-2, (i, x[i], v)


def test_schur_cg_kat():
    """examples/cuSolver_driver_schur_cg.cpp:44-154: CG on Jc H^-1 Jc^T with
    x0 = 0, x[0] and x[6] within 1e-6."""
    z = np.load(H.GOLDEN + "/a200_schur.npz")
    m, n = (int(t) for t in z["Jc_shape"])
    Jc = H.coo_to_csr(m, n, z["Jc_r"], z["Jc_c"], z["Jc_v"])
    Hm = H.coo_to_csr(n, n, z["H_r"], z["H_c"], z["H_v"])
    c = O.Chol(n, Hm.rowptr, Hm.colidx, Hm.vals)
    x, it, err = c.schur_cg(m, Jc.rowptr, Jc.colidx, Jc.vals, z["rhs"], np.zeros(m))
    for i, v in H.SCHUR_KAT.items():
        assert abs(x[i] - v) <= 1e-6, (i, x[i], v)


@pytest.mark.parametrize("name", ["a200_AC_09", "a200_AC_10", "a200_AC_00", "a2000_AC_09", "a2000_AC_10"])
def test_end_to_end_fixtures(name):
    """hybrid1/hybrid2/solver1/solver2 (examples/CMakeLists.txt:22-86):
    relative residual below 1e-2; the oracle also reaches 1e-8."""
    import hykkt_gb300 as hk
    s = H.load_system(name, gamma=1e4)
    perm = hk.Symbolic(s, ordering=hk.ORDER_BUILTIN)["perm"]
    r = O.solve(s, perm=perm)
    assert r.scalar("pivot_col") == -1
    assert r.scalar("rel_res_ref") < 1e-2
    assert r.scalar("rel_res_full") < 1e-8
    # independent check of the 4x4 residual with scipy
    res = H.kkt_residual(s, r["x"], r["s"], r["y"], r["yd"])
    assert res < 1e-8


def test_oracle_matches_direct_solve():
    """On a small well-conditioned synthetic grid the HyKKT oracle agrees with
    a direct sparse LU solve of the 4x4 KKT system."""
    import scipy.sparse.linalg as spla
    s = H.small_grid_system(n_bus=80, seed=3)
    r = O.solve(s)
    K = H.kkt_matrix(s)
    b = np.concatenate([s.rx, s.rs, s.ry, s.ryd])
    z = spla.spsolve(K.tocsc(), b)
    got = np.concatenate([r["x"], r["s"], r["y"], r["yd"]])
    assert np.linalg.norm(got - z) / np.linalg.norm(z) < 1e-8


def test_oracle_without_inequality_block():
    """Jd and Ds empty (the reference's jd_flag == 0 path): the oracle solves the
    2x2 system [H Jc^T; Jc 0] (x, y) = (rx, ry) like a direct LU solve."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    import hykkt_gb300 as hk
    from hykkt_gb300 import gridgen as gg
    s = H.small_grid_system(n_bus=80, seed=3)
    jd = gg.CSR(0, s.n_x, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    ds = gg.CSR(0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    s0 = gg.KKTSystem(s.H, ds, s.Jc, jd, s.rx, np.zeros(0), s.ry, np.zeros(0), s.gamma)
    r = O.solve(s0)
    Hm, Jc = H.to_sp(s.H), H.to_sp(s.Jc)
    K = sp.bmat([[Hm, Jc.T], [Jc, None]]).tocsc()
    z = spla.spsolve(K, np.concatenate([s.rx, s.ry]))
    got = np.concatenate([r["x"], r["y"]])
    assert len(r["s"]) == 0 and len(r["yd"]) == 0
    assert np.linalg.norm(got - z) / np.linalg.norm(z) < 1e-8
    sym = hk.Symbolic(s0, ordering=hk.ORDER_BUILTIN)
    assert len(sym["sq_sn"]) > 0


def test_oracle_regularization_adds_delta_to_present_diagonal():
    """add_diag (HykktSolver.cpp:392; matrix_vector_ops.cu:344-358) with
    delta != 0: exactly the diagonal entries the Hgamma pattern holds change,
    each by one addition; delta = 0 is the reference path bit for bit."""
    s = H.small_grid_system(n_bus=60, seed=2)
    r0 = O.solve(s)
    r1 = O.solve(s, delta=0.0)
    assert np.array_equal(r0["x"], r1["x"])
    rd = O.solve(s, delta=0.5)
    n = s.n_x
    rp, ci = r0.get("hg_rp", n + 1), r0.get("hg_ci", r0.get("hg_rp", n + 1)[-1])
    v0, vd = r0["hg_v"], rd["hg_v"]
    diag = np.zeros(len(v0), dtype=bool)
    for i in range(n):
        for q in range(rp[i], rp[i + 1]):
            if ci[q] == i:
                diag[q] = True
                break
    assert diag.any()
    assert np.array_equal(vd[~diag], v0[~diag])
    assert np.array_equal(vd[diag], v0[diag] + 0.5)
