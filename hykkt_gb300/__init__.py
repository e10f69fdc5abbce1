"""hykkt_gb300: GB300-native HyKKT KKT solve path.

The product is the native library ``lib/libhykkt_gb300.so`` (C ABI in
``include/hykkt_gb300.h``, drop-in C++ API in ``include/HykktSolver.hpp``).
This module is a thin ctypes binding used by the tests and the benchmark;
it never computes anything itself, and it raises if the library has not
been built (there is no fallback path).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libhykkt_gb300.so")
BIN_DIR = os.path.join(_HERE, "bin")

(OK, NOT_SPD, CG_NOT_CONVERGED, PATTERN_CHANGED, OOM, TIMEOUT, INVALID, CUDA_ERROR, RESIDUAL_FAILED, NOT_READY,
 ACCURACY_NOT_MET, CANCELLED) = range(12)
# statuses of a solve that ran to the end (the solution is readable)
SOLVE_STATUSES = (OK, NOT_SPD, CG_NOT_CONVERGED, ACCURACY_NOT_MET)
ORDER_AUTO, ORDER_REFERENCE, ORDER_BUILTIN, ORDER_IDENTITY = range(4)

_lib = None

# hykkt_serve_fn(user, plan, worker, inputs[9], outputs[4]) -> status
SERVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.POINTER(C.c_double)),
                       C.POINTER(C.POINTER(C.c_double)))

# hykkt_server_memory hooks: bytes_fn(user, plan) -> int64; the others -> status
BYTES_FN = C.CFUNCTYPE(C.c_int64, C.c_void_p, C.c_void_p)
PLAN_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)


class ServerMemory(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("bytes_fn", BYTES_FN), ("resident_fn", PLAN_FN),
                ("load_fn", PLAN_FN), ("evict_fn", PLAN_FN), ("user", C.c_void_p)]


_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class HykktError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hykkt error {code}: {msg}")
        self.code = code


class Info(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("cg_iterations", C.c_int), ("pivot_col", C.c_int), ("ordering", C.c_int),
        ("cg_residual", C.c_double), ("rel_residual", C.c_double), ("rel_residual_full", C.c_double),
        ("nnz_L", C.c_int64), ("L_stored", C.c_int64), ("factor_flops", C.c_double), ("device_bytes", C.c_int64),
        ("n_supernodes", C.c_int), ("n_levels", C.c_int), ("n_solve_levels", C.c_int),
        ("kernels_per_solve", C.c_int), ("kernels_per_cg_iteration", C.c_int),
        ("cg_iterations_total", C.c_int), ("refine_steps", C.c_int), ("rel_residual_first", C.c_double),
        ("kernels_per_refine_step", C.c_int), ("pad_", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib() -> C.CDLL:
    """Load libhykkt_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.hykkt_last_error.restype = C.c_char_p
    L.hykkt_version.restype = C.c_char_p
    L.hykkt_plan_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int] + [vp, vp, C.c_int] * 4 + [C.c_double, C.c_int, vp]
    L.hykkt_plan_create_ex.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int] + [vp, vp, C.c_int] * 4 + [C.c_double, C.c_int, vp, C.c_int]
    L.hykkt_plan_destroy.argtypes = [vp]
    L.hykkt_plan_destroy.restype = None
    L.hykkt_plan_solve.argtypes = [vp] + [vp] * 9 + [C.c_int, vp, C.c_int]
    L.hykkt_plan_wait.argtypes = [vp, vp]
    L.hykkt_plan_get_solution.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp]
    L.hykkt_plan_get_info.argtypes = [vp, C.POINTER(Info)]
    L.hykkt_plan_set_gamma.argtypes = [vp, C.c_double]
    L.hykkt_plan_set_accuracy.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_double]
    L.hykkt_solver_set_accuracy.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_double]
    L.hykkt_plan_get_perm.argtypes = [vp, vp]
    L.hykkt_plan_get_L_pattern.argtypes = [vp, vp, vp, C.POINTER(C.c_int64)]
    L.hykkt_plan_get_etree.argtypes = [vp, vp]
    L.hykkt_plan_run_stages.argtypes = [vp, C.c_int, vp]
    L.hykkt_plan_debug_read.argtypes = [vp, C.c_char_p, vp, C.c_int64]
    L.hykkt_plan_get_sizes.argtypes = [vp, vp]
    L.hykkt_plan_get_patterns.argtypes = [vp, vp, vp, vp, vp]
    L.hykkt_plan_time_solves.argtypes = [vp, C.c_int, vp, vp]
    L.hykkt_plan_profile.argtypes = [vp, C.c_int, C.c_char_p, C.c_int]
    L.hykkt_plan_time_trisolve.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.hykkt_plans_time_trisolve.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.hykkt_fp64_peak.argtypes = [dp]
    L.hykkt_solver_create.argtypes = [C.c_double]
    L.hykkt_solver_create.restype = vp
    L.hykkt_solver_destroy.argtypes = [vp]
    L.hykkt_solver_destroy.restype = None
    L.hykkt_solver_read_matrix_files.argtypes = [vp] + [C.c_char_p] * 8 + [C.c_int]
    for nm in ("H", "Ds", "Jc", "Jd"):
        getattr(L, f"hykkt_solver_set_{nm}").argtypes = [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]
    for nm in ("rx", "rs", "ry", "ryd", "x_host", "s_host", "y_host", "yd_host"):
        getattr(L, f"hykkt_solver_set_{nm}").argtypes = [vp, vp, C.c_int]
    L.hykkt_solver_set_gamma.argtypes = [vp, C.c_double]
    L.hykkt_solver_execute.argtypes = [vp]
    L.hykkt_solver_get_solution.argtypes = [vp, vp, vp, vp, vp]
    L.hykkt_solver_get_info.argtypes = [vp, C.POINTER(Info)]
    L.hykkt_solver_set_ordering.argtypes = [vp, C.c_int]
    L.hykkt_perm_maps.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, vp, vp] + [vp] * 9
    L.hykkt_map_index.argtypes = [C.c_int, vp, vp, vp, vp]
    L.hykkt_ruiz_scale.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 12 + [vp]
    L.hykkt_ruiz_scale_noalloc.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 12 + [vp]
    L.hykkt_ruiz_scale_noalloc_max_rows.argtypes = []
    L.hykkt_plan_trace_trisolve.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.hykkt_plan_debug_set.argtypes = [vp, C.c_char_p, C.c_double]
    L.hykkt_fp64_probe.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.hykkt_plan_autotune.argtypes = [vp] + [vp] * 8 + [C.c_int, C.c_char_p, vp]
    L.hykkt_plan_release_device.argtypes = [vp]
    L.hykkt_plan_reload_device.argtypes = [vp]
    L.hykkt_plan_residency.argtypes = [vp, vp, vp]
    L.hykkt_server_create_managed.argtypes = [C.c_int, SERVE_FN, vp, C.POINTER(ServerMemory), C.POINTER(vp)]
    L.hykkt_plan_create_deferred.argtypes = L.hykkt_plan_create_ex.argtypes
    L.hykkt_server_memory_stats.argtypes = [vp] + [vp] * 7
    L.hykkt_server_set_heavy.argtypes = [vp, C.c_int64, C.c_int]
    L.hykkt_server_wait_phases.argtypes = [vp, C.c_int64, vp, vp, vp, vp]
    L.hykkt_server_cancel.argtypes = [vp, C.c_int64, vp]
    L.hykkt_plan_clone.argtypes = [vp, C.POINTER(vp)]
    L.hykkt_plan_set_concurrency.argtypes = [vp, C.c_int]
    L.hykkt_plan_set_refine_rtol.argtypes = [vp, C.c_double]
    L.hykkt_plan_set_delta.argtypes = [vp, C.c_double]
    L.hykkt_plan_solve_regularized.argtypes = [vp] + [vp] * 9 + [C.c_int, vp, C.c_double, C.c_double, C.c_double, dp]
    L.hykkt_chol_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, vp, vp, C.c_int]
    L.hykkt_chol_factor.argtypes = [vp, vp]
    L.hykkt_chol_solve.argtypes = [vp, vp, vp]
    L.hykkt_chol_destroy.argtypes = [vp]
    L.hykkt_chol_destroy.restype = None
    L.hykkt_schur_cg.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, C.c_int, vp, vp, C.c_int, C.c_double, ip, dp]
    L.hykkt_symbolic_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int] + [vp, vp, C.c_int] * 4 + [C.c_int, vp]
    L.hykkt_symbolic_create_ex.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int] + [vp, vp, C.c_int] * 4 + [C.c_int, vp, C.c_int]
    L.hykkt_symbolic_destroy.argtypes = [vp]
    L.hykkt_symbolic_destroy.restype = None
    L.hykkt_symbolic_size.argtypes = [vp, C.c_char_p]
    L.hykkt_symbolic_size.restype = C.c_int64
    L.hykkt_symbolic_get.argtypes = [vp, C.c_char_p, vp, C.c_int64]
    L.hykkt_plan_symbolic_size.argtypes = [vp, C.c_char_p]
    L.hykkt_plan_symbolic_size.restype = C.c_int64
    L.hykkt_plan_symbolic_get.argtypes = [vp, C.c_char_p, vp, C.c_int64]
    L.hykkt_server_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.hykkt_server_create_ex.argtypes = [C.c_int, SERVE_FN, vp, C.POINTER(vp)]
    L.hykkt_server_submit.argtypes = [vp, vp] + [vp] * 13 + [C.POINTER(C.c_int64)]
    L.hykkt_server_wait.argtypes = [vp, C.c_int64, ip, dp, C.POINTER(Info)]
    L.hykkt_server_poll.argtypes = [vp, C.c_int64, ip]
    L.hykkt_server_stats.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.hykkt_server_destroy.argtypes = [vp]
    _lib = L
    return L


class Symbolic:
    """Host-only symbolic analysis of one KKT pattern (no GPU needed)."""

    def __init__(self, system, ordering: int = ORDER_BUILTIN, perm=None, solve_piece: int = 0):
        s = system
        k = [_i32(s.H.rowptr), _i32(s.H.colidx), _i32(s.Ds.rowptr), _i32(s.Ds.colidx),
             _i32(s.Jc.rowptr), _i32(s.Jc.colidx), _i32(s.Jd.rowptr), _i32(s.Jd.colidx)]
        pp = _i32(perm) if perm is not None else None
        h = C.c_void_p()
        _check(lib().hykkt_symbolic_create_ex(C.byref(h), s.n_x, s.m_c, s.m_d, _p(k[0]), _p(k[1]), s.H.nnz,
                                              _p(k[2]), _p(k[3]), s.Ds.nnz, _p(k[4]), _p(k[5]), s.Jc.nnz, _p(k[6]),
                                              _p(k[7]), s.Jd.nnz, ordering, _p(pp), int(solve_piece)))
        self.h = h

    def __getitem__(self, what: str) -> np.ndarray:
        n = lib().hykkt_symbolic_size(self.h, what.encode())
        if n < 0:
            raise KeyError(what)
        out = np.zeros(n, np.int32)
        _check(lib().hykkt_symbolic_get(self.h, what.encode(), _p(out), n))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().hykkt_symbolic_destroy(self.h)
            self.h = None


def _check(rc: int) -> int:
    if rc != OK:
        raise HykktError(rc, lib().hykkt_last_error().decode())
    return rc


def _p(a) -> C.c_void_p | None:
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    if hasattr(a, "data_ptr"):  # torch tensor
        return C.c_void_p(a.data_ptr())
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class TuneInfo(C.Structure):
    _fields_ = [("from_cache", C.c_int), ("candidates", C.c_int), ("concurrent", C.c_int),
                ("solve_piece", C.c_int), ("warp_subtree", C.c_int), ("chunk_fma", C.c_int),
                ("best_solves_per_s", C.c_double), ("cand_piece", C.c_int * 8), ("cand_subtree", C.c_int * 8),
                ("cand_chunk_fma", C.c_int * 8), ("solves_per_s", C.c_double * 8)]

    def as_dict(self) -> dict:
        n = min(self.candidates, 8)
        return {"from_cache": bool(self.from_cache), "candidates": self.candidates, "concurrent": self.concurrent,
                "solve_piece": self.solve_piece, "warp_subtree": self.warp_subtree, "chunk_fma": self.chunk_fma,
                "best_solves_per_s": self.best_solves_per_s,
                "timed": [{"solve_piece": self.cand_piece[i], "warp_subtree": self.cand_subtree[i],
                           "chunk_fma": self.cand_chunk_fma[i], "solves_per_s": self.solves_per_s[i]}
                          for i in range(n)]}


class Plan:
    """Symbolic plan of one KKT sparsity pattern + its device engine."""

    def __init__(self, system, ordering: int = ORDER_AUTO, perm=None, solve_piece: int = 0, deferred: bool = False):
        L = lib()
        s = system
        self._keep = [_i32(s.H.rowptr), _i32(s.H.colidx), _i32(s.Ds.rowptr), _i32(s.Ds.colidx),
                      _i32(s.Jc.rowptr), _i32(s.Jc.colidx), _i32(s.Jd.rowptr), _i32(s.Jd.colidx)]
        k = self._keep
        h = C.c_void_p()
        pp = _i32(perm) if perm is not None else None
        create = L.hykkt_plan_create_deferred if deferred else L.hykkt_plan_create_ex
        _check(create(C.byref(h), s.n_x, s.m_c, s.m_d, _p(k[0]), _p(k[1]), s.H.nnz, _p(k[2]),
                      _p(k[3]), s.Ds.nnz, _p(k[4]), _p(k[5]), s.Jc.nnz, _p(k[6]), _p(k[7]),
                      s.Jd.nnz, float(s.gamma), ordering, _p(pp), int(solve_piece)))
        self.h = h
        self.n_x, self.m_c, self.m_d = s.n_x, s.m_c, s.m_d

    def clone(self) -> "Plan":
        """A plan for the same pattern and settings, sharing the symbolic
        analysis, with its own device memory (for concurrent solves)."""
        h = C.c_void_p()
        _check(lib().hykkt_plan_clone(self.h, C.byref(h)))
        p = Plan.__new__(Plan)
        p.h = h
        p._keep = self._keep
        p.n_x, p.m_c, p.m_d = self.n_x, self.m_c, self.m_d
        return p

    def set_refine_rtol(self, rtol: float) -> None:
        _check(lib().hykkt_plan_set_refine_rtol(self.h, float(rtol)))

    def set_delta(self, delta: float) -> None:
        """Regularization: delta added to the diagonal of Hgamma (add_diag)."""
        _check(lib().hykkt_plan_set_delta(self.h, float(delta)))

    def solve_regularized(self, s, delta_first=1e-8, delta_max=1e4, growth=10.0, y0=None):
        """Inertia-correction loop: returns (status, delta used)."""
        arrs = [_f64(s.H.vals), _f64(s.Ds.vals), _f64(s.Jc.vals), _f64(s.Jd.vals), _f64(s.rx), _f64(s.rs),
                _f64(s.ry), _f64(s.ryd), None if y0 is None else _f64(y0)]
        self._last_inputs = arrs
        used = C.c_double()
        rc = lib().hykkt_plan_solve_regularized(self.h, *[_p(a) for a in arrs], 0, None, float(delta_first),
                                                float(delta_max), float(growth), C.byref(used))
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return rc, used.value

    def set_concurrency(self, share: int) -> None:
        _check(lib().hykkt_plan_set_concurrency(self.h, int(share)))

    def release_device(self) -> None:
        _check(lib().hykkt_plan_release_device(self.h))

    def reload_device(self) -> None:
        _check(lib().hykkt_plan_reload_device(self.h))

    def residency(self):
        """(resident, device bytes when resident)."""
        r, b = C.c_int(), C.c_int64()
        _check(lib().hykkt_plan_residency(self.h, C.byref(r), C.byref(b)))
        return bool(r.value), b.value

    def autotune(self, s, share: int = 1, cache: str | None = None) -> dict:
        """Pick the fastest triangular-solve layout for this pattern with
        `share` plans solving at once (hykkt_plan_autotune); s: a system of
        the pattern (host values) to time."""
        arrs = [_f64(s.H.vals), _f64(s.Ds.vals), _f64(s.Jc.vals), _f64(s.Jd.vals), _f64(s.rx), _f64(s.rs),
                _f64(s.ry), _f64(s.ryd)]
        info = TuneInfo()
        _check(lib().hykkt_plan_autotune(self.h, *[_p(a) for a in arrs], int(share),
                                         None if cache is None else cache.encode(), C.byref(info)))
        return info.as_dict()

    def close(self):
        if getattr(self, "h", None):
            lib().hykkt_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, s, y0=None, on_device=False, stream=None, sync=True) -> int:
        if on_device:
            arrs = [s.H.vals, s.Ds.vals, s.Jc.vals, s.Jd.vals, s.rx, s.rs, s.ry, s.ryd, y0]
        else:
            arrs = [_f64(s.H.vals), _f64(s.Ds.vals), _f64(s.Jc.vals), _f64(s.Jd.vals), _f64(s.rx), _f64(s.rs),
                    _f64(s.ry), _f64(s.ryd), None if y0 is None else _f64(y0)]
        self._last_inputs = arrs
        rc = lib().hykkt_plan_solve(self.h, *[_p(a) for a in arrs], 1 if on_device else 0, _p(stream),
                                    1 if sync else 0)
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return rc

    def wait(self, stream=None) -> int:
        return lib().hykkt_plan_wait(self.h, _p(stream))

    def solution(self):
        x, s, y, yd = (np.zeros(self.n_x), np.zeros(self.m_d), np.zeros(self.m_c), np.zeros(self.m_d))
        _check(lib().hykkt_plan_get_solution(self.h, _p(x), _p(s), _p(y), _p(yd), 0, None))
        return x, s, y, yd

    def info(self) -> dict:
        inf = Info()
        _check(lib().hykkt_plan_get_info(self.h, C.byref(inf)))
        return inf.as_dict()

    def set_accuracy(self, cg_itmax=100, cg_rtol=0.0, refine_max=0, refine_target=1e-10):
        _check(lib().hykkt_plan_set_accuracy(self.h, cg_itmax, cg_rtol, refine_max, refine_target))

    def perm(self) -> np.ndarray:
        p = np.zeros(self.n_x, dtype=np.int32)
        _check(lib().hykkt_plan_get_perm(self.h, _p(p)))
        return p

    def etree(self) -> np.ndarray:
        p = np.zeros(self.n_x, dtype=np.int32)
        _check(lib().hykkt_plan_get_etree(self.h, _p(p)))
        return p

    def L_pattern(self):
        nnz = C.c_int64()
        _check(lib().hykkt_plan_get_L_pattern(self.h, None, None, C.byref(nnz)))
        cp = np.zeros(self.n_x + 1, dtype=np.int32)
        ri = np.zeros(nnz.value, dtype=np.int32)
        _check(lib().hykkt_plan_get_L_pattern(self.h, _p(cp), _p(ri), C.byref(nnz)))
        return cp, ri

    def sizes(self) -> dict:
        s = np.zeros(8, dtype=np.int64)
        _check(lib().hykkt_plan_get_sizes(self.h, _p(s)))
        keys = ["nnz_ht", "nnz_lower", "nnz_hg", "nnz_L", "front_arena", "n_supernodes", "n_solve_items", "u_arena"]
        return dict(zip(keys, s.tolist()))

    def patterns(self):
        sz = self.sizes()
        ht_rp = np.zeros(self.n_x + 1, dtype=np.int32)
        ht_ci = np.zeros(sz["nnz_ht"], dtype=np.int32)
        lp_cp = np.zeros(self.n_x + 1, dtype=np.int32)
        lp_row = np.zeros(sz["nnz_lower"], dtype=np.int32)
        _check(lib().hykkt_plan_get_patterns(self.h, _p(ht_rp), _p(ht_ci), _p(lp_cp), _p(lp_row)))
        return ht_rp, ht_ci, lp_cp, lp_row

    def symbolic(self, what: str) -> np.ndarray:
        n = lib().hykkt_plan_symbolic_size(self.h, what.encode())
        if n < 0:
            raise KeyError(what)
        out = np.zeros(n, np.int32)
        _check(lib().hykkt_plan_symbolic_get(self.h, what.encode(), _p(out), n))
        return out

    def read(self, what: str, n: int) -> np.ndarray:
        out = np.zeros(n)
        _check(lib().hykkt_plan_debug_read(self.h, what.encode(), _p(out), n))
        return out

    def run_stages(self, upto: int = 3) -> list[float]:
        ms = (C.c_float * 5)()
        rc = lib().hykkt_plan_run_stages(self.h, upto, ms)
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return list(ms)

    def profile(self, upto: int = 3) -> dict:
        """Per-kernel device time of one uncaptured solve: {name: (launches, ms)}."""
        import json
        buf = C.create_string_buffer(1 << 16)
        rc = lib().hykkt_plan_profile(self.h, upto, buf, len(buf))
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return {k: tuple(v) for k, v in json.loads(buf.value.decode()).items()}

    def time_trisolve(self, nrep: int = 20) -> float:
        ms = C.c_float()
        rc = lib().hykkt_plan_time_trisolve(self.h, nrep, C.byref(ms))
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return ms.value

    def debug_set(self, what: str, value: float) -> None:
        """Test hooks of the bounded device waits (hykkt_plan_debug_set)."""
        _check(lib().hykkt_plan_debug_set(self.h, what.encode(), float(value)))

    def trace_trisolve(self) -> np.ndarray:
        """Per-task timeline of one forward + backward solve: rows of
        (claimed, dependencies met, done, SM id), forward tasks first; times
        in ns."""
        n = C.c_int64()
        _check(lib().hykkt_plan_trace_trisolve(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.uint64)
        _check(lib().hykkt_plan_trace_trisolve(self.h, _p(out), n.value, C.byref(n)))
        return out.reshape(-1, 4)

    def time_solves(self, nsteps: int, stream=None) -> np.ndarray:
        ms = np.zeros(nsteps, dtype=np.float32)
        rc = lib().hykkt_plan_time_solves(self.h, nsteps, _p(ms), _p(stream))
        if rc not in SOLVE_STATUSES:
            _check(rc)
        return ms


def time_trisolve_group(plans, nrep: int = 20, mode: int = 0) -> float:
    """ms of one solve pair of every plan (same pattern): mode 0 lockstep,
    1 concurrent streams, 2 sequential."""
    arr = (C.c_void_p * len(plans))(*[p.h.value for p in plans])
    ms = C.c_float()
    _check(lib().hykkt_plans_time_trisolve(arr, len(plans), nrep, mode, C.byref(ms)))
    return ms.value


def fp64_probe_tflops(mode: int) -> float:
    """0: DFMA chains, 1: FP64 mma.sync chains, 2: both in one kernel."""
    v = C.c_double()
    _check(lib().hykkt_fp64_probe(int(mode), C.byref(v)))
    return v.value


def fp64_peak_tflops() -> float:
    v = C.c_double()
    _check(lib().hykkt_fp64_peak(C.byref(v)))
    return v.value


def perm_maps(perm, a_rows, a_cols, j_rows, j_cols, n_j, jt_rows, jt_cols, m_j):
    """PermClass maps (rc on A, c on J, r on J^T); host integer work."""
    n = len(perm)
    perm, a_rows, a_cols = _i32(perm), _i32(a_rows), _i32(a_cols)
    j_rows, j_cols, jt_rows, jt_cols = _i32(j_rows), _i32(j_cols), _i32(jt_rows), _i32(jt_cols)
    nnz_a, nnz_j = int(a_rows[-1]), int(j_rows[-1])
    rev = np.zeros(n, np.int32)
    rc_rows, rc_cols, rc_map = np.zeros(n + 1, np.int32), np.zeros(nnz_a, np.int32), np.zeros(nnz_a, np.int32)
    c_cols, c_map = np.zeros(nnz_j, np.int32), np.zeros(nnz_j, np.int32)
    r_rows, r_cols, r_map = np.zeros(m_j + 1, np.int32), np.zeros(nnz_j, np.int32), np.zeros(nnz_j, np.int32)
    _check(lib().hykkt_perm_maps(n, _p(perm), _p(a_rows), _p(a_cols), nnz_a, n_j, _p(j_rows), _p(j_cols), nnz_j, m_j,
                                 _p(jt_rows), _p(jt_cols), _p(rev), _p(rc_rows), _p(rc_cols), _p(rc_map), _p(c_cols),
                                 _p(c_map), _p(r_rows), _p(r_cols), _p(r_map)))
    return dict(rev=rev, rc_rows=rc_rows, rc_cols=rc_cols, rc_map=rc_map, c_cols=c_cols, c_map=c_map, r_rows=r_rows,
                r_cols=r_cols, r_map=r_map)


class Chol:
    """CholeskyClass mirror on the GPU (lower triangle of the CSR is read)."""

    def __init__(self, n, rowptr, colidx, ordering=ORDER_IDENTITY):
        self._rp, self._ci = _i32(rowptr), _i32(colidx)
        self.n = n
        h = C.c_void_p()
        _check(lib().hykkt_chol_create(C.byref(h), n, int(self._rp[-1]), _p(self._rp), _p(self._ci), ordering))
        self.h = h

    def factor(self, vals) -> int:
        v = _f64(vals)
        return lib().hykkt_chol_factor(self.h, _p(v))

    def solve(self, b) -> np.ndarray:
        b = _f64(b)
        x = np.zeros(self.n)
        _check(lib().hykkt_chol_solve(self.h, _p(x), _p(b)))
        return x

    def schur_cg(self, m, jc_rp, jc_ci, jc_v, b, x0, itmax=100, tol=1e-12):
        rp, ci, v, b = _i32(jc_rp), _i32(jc_ci), _f64(jc_v), _f64(b)
        x = _f64(x0).copy()
        it, err = C.c_int(), C.c_double()
        rc = lib().hykkt_schur_cg(self.h, m, self.n, _p(rp), _p(ci), _p(v), int(rp[-1]), _p(b), _p(x), itmax, tol,
                                  C.byref(it), C.byref(err))
        if rc not in (OK, CG_NOT_CONVERGED):
            _check(rc)
        return x, it.value, err.value, rc

    def close(self):
        if getattr(self, "h", None):
            lib().hykkt_chol_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Served solves (hykkt_server_*): a thread-safe request queue over plans.

    ``submit(plan, system)`` may be called from any thread and returns a
    ticket; ``wait(ticket)`` returns (status, latency_ms, info, (x, s, y, yd)).
    ``serve_fn`` (tests) replaces the GPU solve: fn(plan_key, worker, inputs,
    outputs) -> status, with plan handles as opaque integer keys."""

    def __init__(self, workers: int, serve_fn=None, budget: int | None = None, hooks: dict | None = None):
        """budget: device bytes the served plans may hold together (0 = 90%
        of free memory; None = no admission control).  hooks (tests, with
        serve_fn): {"bytes": f(plan) -> int, "resident": f(plan) -> bool,
        "load": f(plan) -> status, "evict": f(plan) -> status}."""
        self.h = C.c_void_p()
        self._fn = None
        fnp = SERVE_FN()  # NULL: the GPU solve
        if serve_fn is not None:
            def tramp(user, plan, worker, ins, outs):
                try:
                    return int(serve_fn(plan or 0, worker, ins, outs))
                except Exception:
                    return INVALID
            self._fn = SERVE_FN(tramp)
            fnp = self._fn
        if budget is None:
            if serve_fn is None:
                _check(lib().hykkt_server_create(int(workers), C.byref(self.h)))
            else:
                _check(lib().hykkt_server_create_ex(int(workers), fnp, None, C.byref(self.h)))
        else:
            hooks = hooks or {}

            def wrap(proto, f, default):
                if f is None:
                    return proto()
                def g(user, plan):
                    try:
                        return int(f(plan or 0))
                    except Exception:
                        return default
                return proto(g)
            self._mem = ServerMemory(int(budget), wrap(BYTES_FN, hooks.get("bytes"), -1),
                                     wrap(PLAN_FN, hooks.get("resident"), 0), wrap(PLAN_FN, hooks.get("load"), INVALID),
                                     wrap(PLAN_FN, hooks.get("evict"), INVALID), None)
            _check(lib().hykkt_server_create_managed(int(workers), fnp, None, C.byref(self._mem), C.byref(self.h)))
        self._bufs = {}

    def set_heavy(self, heavy_bytes: int, max_heavy: int) -> None:
        """Requests of plans of at least heavy_bytes of device storage take at
        most max_heavy workers at a time (heavy_bytes <= 0: no limit)."""
        _check(lib().hykkt_server_set_heavy(self.h, int(heavy_bytes), int(max_heavy)))

    def memory_stats(self) -> dict:
        v = [C.c_int64() for _ in range(7)]
        _check(lib().hykkt_server_memory_stats(self.h, *[C.byref(x) for x in v]))
        keys = ["budget", "resident_bytes", "peak_bytes", "resident_plans", "admissions", "evictions", "deferrals"]
        return dict(zip(keys, [x.value for x in v]))

    def submit(self, plan, s=None, y0=None, arrays=None, out=None) -> int:
        """plan: a Plan (or an integer key with serve_fn); s: a KKTSystem with
        host values, or ``arrays`` = the nine input arrays directly."""
        if arrays is None:
            arrays = [_f64(s.H.vals), _f64(s.Ds.vals), _f64(s.Jc.vals), _f64(s.Jd.vals), _f64(s.rx), _f64(s.rs),
                      _f64(s.ry), _f64(s.ryd), None if y0 is None else _f64(y0)]
        if out is None:
            n_x, m_c, m_d = plan.n_x, plan.m_c, plan.m_d
            out = (np.zeros(n_x), np.zeros(m_d), np.zeros(m_c), np.zeros(m_d))
        ph = plan.h if isinstance(plan, Plan) else C.c_void_p(int(plan))
        t = C.c_int64()
        _check(lib().hykkt_server_submit(self.h, ph, *[_p(a) for a in arrays], *[_p(o) for o in out], C.byref(t)))
        self._bufs[t.value] = (arrays, out)
        return t.value

    def wait(self, ticket: int):
        """(status, latency_ms, info, outputs); info also carries where the
        latency went: queue_ms, admission_ms, solve_ms."""
        st, lat, info = C.c_int(), C.c_double(), Info()
        ph = (C.c_double * 3)()
        _check(lib().hykkt_server_wait_phases(self.h, int(ticket), C.byref(st), C.byref(lat), C.byref(info), ph))
        _, out = self._bufs.pop(ticket)
        d = info.as_dict()
        d.update(queue_ms=ph[0], admission_ms=ph[1], solve_ms=ph[2])
        return st.value, lat.value, d, out

    def cancel(self, ticket: int) -> bool:
        """Withdraw a request no worker has taken yet (its wait then returns
        CANCELLED); False when it is already being solved or done."""
        c = C.c_int()
        _check(lib().hykkt_server_cancel(self.h, int(ticket), C.byref(c)))
        return bool(c.value)

    def poll(self, ticket: int) -> bool:
        d = C.c_int()
        _check(lib().hykkt_server_poll(self.h, int(ticket), C.byref(d)))
        return bool(d.value)

    def stats(self) -> dict:
        c, q, f = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().hykkt_server_stats(self.h, C.byref(c), C.byref(q), C.byref(f)))
        return {"completed": c.value, "queued": q.value, "in_flight": f.value}

    def close(self):
        if self.h:
            lib().hykkt_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
