"""Shared helpers of the test suite: golden fixtures, small synthetic
systems and dense/sparse reference algebra (numpy/scipy) for residual checks."""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse as sp

from hykkt_gb300 import gridgen as gg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Known answers from the reference's own tests
RUIZ_KAT = {  # examples/Ruiz_driver.cpp:145-182 (tolerance 1e-8, :56)
    "H[n/2-1]": 0.062378167641326,
    "A[last]": 0.005524271728020,
    "At[1]": 0.5,
    "rhs[n/2-1]": 0.044151078568835,
    "rhs[3n/2-1]": 0.044194173824159,
    "max_d[32]": 0.171498585142,
}
CHOL_KAT = {0: -97.663191790329750, 6: -1.389053208413921}  # cuSolver_driver_cholesky.cpp:66-75, abs tol 3e-2
SCHUR_KAT = {0: 22.171865776354700, 6: -4.446628667344612e03}  # cuSolver_driver_schur_cg.cpp:145-154, abs tol 1e-6
# perm_driver.cpp:15-25
PERM_A_I = [0, 2, 5, 7, 9]
PERM_A_J = [0, 2, 0, 1, 2, 1, 2, 1, 3]
PERM_PERM = [2, 0, 3, 1]
PERM_RC_I = [0, 2, 4, 6, 9]
PERM_RC_J = [0, 3, 0, 1, 2, 3, 0, 1, 3]
PERM_R_I = [0, 2, 4, 6, 9]
PERM_R_J = [1, 2, 0, 2, 1, 3, 0, 1, 2]
PERM_C_J = [0, 1, 0, 1, 3, 0, 3, 2, 3]


def coo_to_csr(n, m, r, c, v) -> gg.CSR:
    return gg.coo_to_csr(n, m, r, c, v)


def sym_lower_to_full(n, r, c, v) -> gg.CSR:
    off = r != c
    rr = np.concatenate([r, c[off]])
    cc = np.concatenate([c, r[off]])
    vv = np.concatenate([v, v[off]])
    return gg.coo_to_csr(n, n, rr, cc, vv)


def load_system(name: str, gamma: float = 1e4) -> gg.KKTSystem:
    """One of the reference's KKT fixtures (a200_AC_09, a200_AC_10, a200_AC_00,
    a2000_AC_09, a2000_AC_10)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    n, _ = z["H_shape"]
    H = sym_lower_to_full(int(n), z["H_r"], z["H_c"], z["H_v"])
    blocks = {}
    for key in ("Ds", "Jc", "Jd"):
        bn, bm = (int(t) for t in z[f"{key}_shape"])
        blocks[key] = coo_to_csr(bn, bm, z[f"{key}_r"], z[f"{key}_c"], z[f"{key}_v"])
    return gg.KKTSystem(H, blocks["Ds"], blocks["Jc"], blocks["Jd"], z["rx"].copy(), z["rs"].copy(),
                        z["ry"].copy(), z["ryd"].copy(), gamma)


def fixture_skip(name: str) -> int:
    return int(np.load(os.path.join(GOLDEN, name + ".npz"))["skip"])


def write_fixture_files(name: str, folder: str) -> list[str]:
    """Write the fixture back as the reference's eight Matrix-Market files
    (H lower triangle; a200 layout without banner for skip 2, a2000 layout
    with banner + comment for skip 3)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    skip = int(z["skip"])
    os.makedirs(folder, exist_ok=True)
    paths = []
    for key in ("H", "Ds", "Jc", "Jd"):
        n, m = (int(t) for t in z[f"{key}_shape"])
        p = os.path.join(folder, f"{key}.mtx")
        with open(p, "w") as f:
            if skip == 3:
                kind = "symmetric" if key == "H" else "general"
                f.write(f"%%MatrixMarket matrix coordinate real {kind}\n")
            f.write("% Generated for tests\n")
            f.write(f"{n} {m} {len(z[f'{key}_r'])}\n")
            for a, b, v in zip(z[f"{key}_r"].tolist(), z[f"{key}_c"].tolist(), z[f"{key}_v"].tolist()):
                f.write(f"{a + 1} {b + 1} {v!r}\n")
        paths.append(p)
    for key in ("rx", "rs", "ry", "ryd"):
        p = os.path.join(folder, f"{key}.mtx")
        with open(p, "w") as f:
            f.write("%%MatrixMarket matrix array real general\n")
            f.write(f"{len(z[key])} 1\n")
            for v in z[key].tolist():
                f.write(f"{v!r}\n")
        paths.append(p)
    return paths


def small_grid_system(n_bus=120, seed=0, gamma=1e4, dx=(1e-4, 1e4), ds=(1e-4, 1e4)) -> gg.KKTSystem:
    grid = gg.make_grid(n_bus, seed)
    return gg.make_system(grid, seed + 1, gamma, dx, ds)


def to_sp(A: gg.CSR):
    return sp.csr_matrix((A.vals, A.colidx, A.rowptr), shape=(A.n, A.m))


def kkt_matrix(s: gg.KKTSystem):
    H, Jc, Jd = to_sp(s.H), to_sp(s.Jc), to_sp(s.Jd)
    Ds = sp.diags(s.Ds.vals) if s.m_d else sp.csr_matrix((0, 0))
    md = s.m_d
    return sp.bmat([[H, None, Jc.T, Jd.T], [None, Ds, None, -sp.eye(md)], [Jc, None, None, None],
                    [Jd, -sp.eye(md), None, None]]).tocsr()


def kkt_residual(s: gg.KKTSystem, x, ds, y, yd) -> float:
    """||K z - b|| / ||b|| of the 4-block KKT system, the products and the
    subtraction accumulated in extended precision (np.longdouble): with D
    entries up to 1e8 a plain double residual carries rounding noise of
    about 1e-9 relative, the size of the quantity being checked."""
    K = kkt_matrix(s).tocsr()
    K.sort_indices()
    z = np.concatenate([x, ds, y, yd]).astype(np.longdouble)
    b = np.concatenate([s.rx, s.rs, s.ry, s.ryd])
    prods = K.data.astype(np.longdouble) * z[K.indices]
    rows = np.repeat(np.arange(K.shape[0]), np.diff(K.indptr))
    kz = np.zeros(K.shape[0], dtype=np.longdouble)
    np.add.at(kz, rows, prods)
    r = (kz - b.astype(np.longdouble)).astype(np.float64)
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def ruiz_test_blocks(n=1024):
    """The Ruiz driver's synthetic blocks (examples/Ruiz_driver.cpp:22-49,
    58-89): A lower bidiagonal with A[i][i-1] = i+1 and a zero diagonal that
    add_diag(1.0) turns into 1, H = sqrt(n) I, rhs = 1."""
    a_i = np.zeros(n + 1, np.int32)
    a_j = np.zeros(2 * n - 1, np.int32)
    a_v = np.zeros(2 * n - 1)
    a_i[0] = 0
    for i in range(n):
        if i:
            a_v[2 * i - 1] = i + 1
            a_j[2 * i - 1] = i - 1
            a_i[i] = 2 * i - 1
        a_v[2 * i] = 0
        a_j[2 * i] = i
    a_i[n] = 2 * n - 1
    a_v[a_j == np.repeat(np.arange(n), np.diff(a_i))] += 1.0  # add_diag(1.0)
    h_i = np.arange(n + 1, dtype=np.int32)
    h_j = np.arange(n, dtype=np.int32)
    h_v = np.full(n, np.sqrt(n))
    A = gg.CSR(n, n, a_i, a_j, a_v)
    At = gg.CSR(n, n, *_transpose(n, n, a_i, a_j, a_v))
    return gg.CSR(n, n, h_i, h_j, h_v), A, At, np.ones(2 * n)


def _transpose(n, m, rp, ci, v):
    S = sp.csr_matrix((v, ci, rp), shape=(n, m)).T.tocsr()
    S.sort_indices()
    return S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.copy()


def ruiz_kat_values(H, A, At, rhs, max_d, n=1024) -> dict:
    return {
        "H[n/2-1]": H.vals[n // 2 - 1],
        "A[last]": A.vals[-1],
        "At[1]": At.vals[1],
        "rhs[n/2-1]": rhs[n // 2 - 1],
        "rhs[3n/2-1]": rhs[3 * n // 2 - 1],
        "max_d[32]": max_d[32],
    }
