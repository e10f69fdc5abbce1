"""The reference's host ordering for the CPU baseline.

MEASUREMENT INFRASTRUCTURE ONLY.  The reference orders H_gamma with
cusolverSpXcsrsymamdHost on its full symmetric pattern with a general
zero-based descriptor (src/PermClass.cpp:88-95).  The CPU baseline calls the
same routine here through ctypes (it runs on the host but needs a CUDA
context for its handle), times it on its own, and hands the permutation to
the oracle.  The pattern is H ∪ Jd^T Jd ∪ Jc^T Jc with sorted columns
(src/SpgemmClass.cpp:96-143), formed with scipy.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import scipy.sparse as sp


def hgamma_pattern(s):
    """Sorted CSR pattern (rowptr, colidx) of H + Jd^T Jd + Jc^T Jc."""
    def ones(A, n, m):
        return sp.csr_matrix((np.ones(A.nnz), A.colidx, A.rowptr), shape=(n, m))
    H = ones(s.H, s.n_x, s.n_x)
    Jc = ones(s.Jc, s.m_c, s.n_x)
    P = H + (Jc.T @ Jc)
    if s.Jd.nnz:
        Jd = ones(s.Jd, s.m_d, s.n_x)
        P = P + (Jd.T @ Jd)
    P = P.tocsr()
    P.sort_indices()
    return P.indptr.astype(np.int32), P.indices.astype(np.int32)


_libs = None


def _load():
    global _libs
    if _libs is None:
        sol = None
        for name in ("libcusolver.so.12", "libcusolver.so"):
            try:
                sol = C.CDLL(name)
                break
            except OSError:
                pass
        spa = None
        for name in ("libcusparse.so.12", "libcusparse.so"):
            try:
                spa = C.CDLL(name)
                break
            except OSError:
                pass
        if sol is None or spa is None:
            raise RuntimeError("cuSOLVER/cuSPARSE not loadable")
        vp = C.c_void_p
        sol.cusolverSpCreate.argtypes = [C.POINTER(vp)]
        sol.cusolverSpDestroy.argtypes = [vp]
        sol.cusolverSpXcsrsymamdHost.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp]
        spa.cusparseCreateMatDescr.argtypes = [C.POINTER(vp)]
        spa.cusparseDestroyMatDescr.argtypes = [vp]
        _libs = (sol, spa)
    return _libs


def symamd(rp: np.ndarray, ci: np.ndarray) -> np.ndarray:
    """perm[new] = old from cusolverSpXcsrsymamdHost (raises where it cannot run)."""
    sol, spa = _load()
    h, d = C.c_void_p(), C.c_void_p()
    if sol.cusolverSpCreate(C.byref(h)) != 0:
        raise RuntimeError("cusolverSpCreate failed (no CUDA context)")
    try:
        if spa.cusparseCreateMatDescr(C.byref(d)) != 0:
            raise RuntimeError("cusparseCreateMatDescr failed")
        n = len(rp) - 1
        rp = np.ascontiguousarray(rp, np.int32)
        ci = np.ascontiguousarray(ci, np.int32)
        perm = np.zeros(n, np.int32)
        st = sol.cusolverSpXcsrsymamdHost(h, n, int(rp[-1]), d, rp.ctypes.data, ci.ctypes.data, perm.ctypes.data)
        spa.cusparseDestroyMatDescr(d)
        if st != 0:
            raise RuntimeError(f"cusolverSpXcsrsymamdHost returned {st}")
        return perm
    finally:
        sol.cusolverSpDestroy(h)


def timed_symamd(s):
    """(perm, seconds of the ordering call alone, seconds of the pattern)."""
    t0 = time.perf_counter()
    rp, ci = hgamma_pattern(s)
    t1 = time.perf_counter()
    perm = symamd(rp, ci)
    return perm, time.perf_counter() - t1, t1 - t0
