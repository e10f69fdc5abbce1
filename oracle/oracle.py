"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  It is the checker; nothing in the product
imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built (hykkt_gb300.build.build_oracle())")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.oracle_mm_header.argtypes = [C.c_char_p, C.c_int, vp, vp, vp]
        L.oracle_mm_read.argtypes = [C.c_char_p, C.c_int, vp, vp, vp]
        L.oracle_coo_to_csr.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        L.oracle_sym_coo_count.argtypes = [C.c_int, vp, vp]
        L.oracle_sym_coo_to_csr.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        L.oracle_read_rhs.argtypes = [C.c_char_p, vp, C.c_int]
        L.oracle_reverse_perm.argtypes = [C.c_int, vp, vp]
        L.oracle_vec_map_rc.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_vec_map_c.argtypes = [C.c_int, vp, vp, vp, vp, vp]
        L.oracle_vec_map_r.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp]
        L.oracle_ruiz_scale.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 12
        L.oracle_chol_factor.argtypes = [C.c_int, vp, vp, vp, vp, vp]
        L.oracle_chol_factor.restype = vp
        L.oracle_chol_solve.argtypes = [vp, vp, vp]
        L.oracle_chol_nnz.argtypes = [vp]
        L.oracle_chol_nnz.restype = C.c_long
        L.oracle_chol_free.argtypes = [vp]
        L.oracle_schur_cg.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.c_int, C.c_double, vp]
        L.oracle_solve.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, vp,
                                   vp, vp, vp, vp, C.c_double, vp, C.c_int, C.c_double]
        L.oracle_solve.restype = vp
        L.oracle_solve_ex.argtypes = L.oracle_solve.argtypes + [C.c_double, C.c_int, C.c_double, C.c_double]
        L.oracle_solve_ex.restype = vp
        L.oracle_solve_reg.argtypes = L.oracle_solve_ex.argtypes + [C.c_double]
        L.oracle_solve_reg.restype = vp
        L.oracle_size.argtypes = [vp, C.c_char_p]
        L.oracle_size.restype = C.c_long
        L.oracle_get.argtypes = [vp, C.c_char_p, vp, C.c_long]
        L.oracle_scalar.argtypes = [vp, C.c_char_p]
        L.oracle_scalar.restype = C.c_double
        L.oracle_free.argtypes = [vp]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_get_threads.restype = C.c_int
        _lib = L
    return _lib


def set_threads(threads: int) -> None:
    """Threads of the factorization, solves and CG (1 = the pinned checker)."""
    lib().oracle_set_threads(int(threads))


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def read_mm(path: str, skip: int):
    """(n, m, rows, cols, vals) with the reference reader's skip semantics."""
    n, m, nnz = C.c_int(), C.c_int(), C.c_int()
    rc = lib().oracle_mm_header(path.encode(), skip, C.byref(n), C.byref(m), C.byref(nnz))
    if rc:
        raise ValueError(f"oracle_mm_header({path}) = {rc}")
    r = np.zeros(nnz.value, np.int32)
    c = np.zeros(nnz.value, np.int32)
    v = np.zeros(nnz.value)
    rc = lib().oracle_mm_read(path.encode(), skip, _p(r), _p(c), _p(v))
    if rc:
        raise ValueError(f"oracle_mm_read({path}) = {rc}")
    return n.value, m.value, r, c, v


def coo_to_csr(n, r, c, v):
    nnz = len(r)
    rp, ci, vv = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
    lib().oracle_coo_to_csr(n, nnz, _p(_i(r)), _p(_i(c)), _p(_d(v)), _p(rp), _p(ci), _p(vv))
    return rp, ci, vv


def sym_coo_to_csr(n, r, c, v):
    r, c, v = _i(r), _i(c), _d(v)
    cnt = lib().oracle_sym_coo_count(len(r), _p(r), _p(c))
    rp, ci, vv = np.zeros(n + 1, np.int32), np.zeros(cnt, np.int32), np.zeros(cnt)
    lib().oracle_sym_coo_to_csr(n, len(r), _p(r), _p(c), _p(v), _p(rp), _p(ci), _p(vv))
    return rp, ci, vv


def read_rhs(path: str, n: int) -> np.ndarray:
    out = np.zeros(n)
    cnt = lib().oracle_read_rhs(path.encode(), _p(out), n)
    if cnt < 0:
        raise ValueError(path)
    return out


def perm_maps(perm, rows, cols, n_j, j_rows, j_cols, m_j, jt_rows, jt_cols):
    n = len(perm)
    perm = _i(perm)
    rev = np.zeros(n, np.int32)
    lib().oracle_reverse_perm(n, _p(perm), _p(rev))
    rows, cols = _i(rows), _i(cols)
    prc_r, prc_c, prc_m = np.zeros(n + 1, np.int32), np.zeros(len(cols), np.int32), np.zeros(len(cols), np.int32)
    lib().oracle_vec_map_rc(n, _p(rows), _p(cols), _p(perm), _p(rev), _p(prc_r), _p(prc_c), _p(prc_m))
    j_rows, j_cols = _i(j_rows), _i(j_cols)
    pc_c, pc_m = np.zeros(len(j_cols), np.int32), np.zeros(len(j_cols), np.int32)
    lib().oracle_vec_map_c(n_j, _p(j_rows), _p(j_cols), _p(rev), _p(pc_c), _p(pc_m))
    jt_rows, jt_cols = _i(jt_rows), _i(jt_cols)
    pr_r, pr_c, pr_m = np.zeros(m_j + 1, np.int32), np.zeros(len(jt_cols), np.int32), np.zeros(len(jt_cols), np.int32)
    lib().oracle_vec_map_r(m_j, _p(jt_rows), _p(jt_cols), _p(perm), _p(pr_r), _p(pr_c), _p(pr_m))
    return dict(rev=rev, rc_rows=prc_r, rc_cols=prc_c, rc_map=prc_m, c_cols=pc_c, c_map=pc_m, r_rows=pr_r,
                r_cols=pr_c, r_map=pr_m)


def ruiz_scale(its, n, m, a, bt, b, rhs1, rhs2):
    """a, bt, b: (rowptr, colidx, vals) tuples; returns scaled copies and max_d."""
    av, btv, bv = _d(a[2]).copy(), _d(bt[2]).copy(), _d(b[2]).copy()
    r1, r2 = _d(rhs1).copy(), _d(rhs2).copy()
    md = np.zeros(n + m)
    ai, aj, bti, btj, bi, bj = (_i(x) for x in (a[0], a[1], bt[0], bt[1], b[0], b[1]))
    lib().oracle_ruiz_scale(its, n, m, _p(av), _p(ai), _p(aj), _p(btv), _p(bti), _p(btj), _p(bv), _p(bi), _p(bj),
                            _p(r1), _p(r2), _p(md))
    return av, btv, bv, r1, r2, md


class Chol:
    def __init__(self, n, rp, ci, v, perm=None):
        self.n = n
        st = C.c_int()
        self._perm = None if perm is None else _i(perm)
        self.h = lib().oracle_chol_factor(n, _p(_i(rp)), _p(_i(ci)), _p(_d(v)), _p(self._perm), C.byref(st))
        self.status = st.value

    def solve(self, b):
        x = np.zeros(self.n)
        lib().oracle_chol_solve(self.h, _p(_d(b)), _p(x))
        return x

    def schur_cg(self, m, jc_rp, jc_ci, jc_v, b, x0, itmax=100, tol=1e-12):
        x = _d(x0).copy()
        err = C.c_double()
        it = lib().oracle_schur_cg(self.h, m, self.n, _p(_i(jc_rp)), _p(_i(jc_ci)), _p(_d(jc_v)), _p(_d(b)), _p(x),
                                   itmax, tol, C.byref(err))
        return x, it, err.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_chol_free(self.h)
            self.h = None


class Result:
    _INT = {"ht_rp", "ht_ci", "hg_rp", "hg_ci", "parent", "L_cp", "L_ri", "perm"}

    def __init__(self, h):
        self.h = h

    def __getitem__(self, name):
        n = lib().oracle_size(self.h, name.encode())
        if n == -1 and name == "jc_s":
            raise KeyError("use get('jc_s', n)")
        if n < 0:
            raise KeyError(name)
        return self.get(name, n)

    def get(self, name, n):
        out = np.zeros(n, np.int32 if name in self._INT else np.float64)
        rc = lib().oracle_get(self.h, name.encode(), _p(out), n)
        if rc:
            raise KeyError(name)
        return out

    def scalar(self, name):
        return lib().oracle_scalar(self.h, name.encode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_free(self.h)
            self.h = None


def solve(s, perm=None, itmax=100, tol=1e-12, y0=None, rtol=0.0, refine_max=0, refine_target=1e-10,
          refine_rtol=None, delta=0.0) -> Result:
    """Run the oracle on a gridgen.KKTSystem-like object (defaults: the
    reference's CG budget and tolerance, no refinement, no regularization;
    delta is added to the diagonal of Hgamma before the factorization)."""
    H, Jc, Jd = s.H, s.Jc, s.Jd
    keep = [_i(H.rowptr), _i(H.colidx), _d(H.vals), _d(s.Ds.vals), _i(Jc.rowptr), _i(Jc.colidx), _d(Jc.vals),
            _i(Jd.rowptr), _i(Jd.colidx), _d(Jd.vals), _d(s.rx), _d(s.rs), _d(s.ry), _d(s.ryd)]
    pp = None if perm is None else _i(perm)
    y0a = None if y0 is None else _d(y0)
    h = lib().oracle_solve_reg(s.n_x, s.m_c, s.m_d, *[_p(a) for a in keep[:10]], int(Jd.nnz),
                               *[_p(a) for a in keep[10:]], _p(y0a), float(s.gamma), _p(pp), itmax, tol, rtol,
                               refine_max, refine_target, -1.0 if refine_rtol is None else float(refine_rtol),
                               float(delta))
    return Result(h)
