"""hykkt_ruiz_scale_noalloc: Ruiz scaling with its scale vector in a fixed
device array (no allocation), against hykkt_ruiz_scale on the same inputs
and against the host oracle.

Kept in its own file, collected last, so that it runs after the other GPU
tests; one case starts a fresh Python process whose first call into the
library is a no-alloc call (the first call on a device does the array's
set-up there).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _square_blocks(seed):
    """Ruiz driver blocks (n = m) with seeded random values (same patterns):
    returns n, m, A (n x n), B^T (n x m), B (m x n), rhs1, rhs2."""
    Hm, A, At, rhs = H.ruiz_test_blocks()
    rng = np.random.default_rng(seed)
    for M in (Hm, A, At):
        M.vals = M.vals * rng.uniform(0.5, 2.0, len(M.vals))
    rhs = rhs * rng.uniform(-1.0, 1.0, len(rhs))
    n = Hm.n
    # [H A^T; A 0]: the Ruiz driver's block roles (examples/Ruiz_driver.cpp:58-89)
    return n, n, Hm, At, A, rhs[:n].copy(), rhs[n:].copy()


def _rect_blocks(n, m, seed):
    """Random blocks with m != n: A n x n (diagonal plus 4 entries per row),
    B m x n (3 entries per row), B^T its transpose."""
    rng = np.random.default_rng(seed)

    def csr(rows, cols, per_row, diag):
        rp, ci = [0], []
        for i in range(rows):
            c = set(rng.choice(cols, per_row, replace=False).tolist())
            if diag:
                c.add(i)
            ci += sorted(c)
            rp.append(len(ci))
        v = rng.normal(0.0, 1.0, len(ci)) * np.exp(rng.uniform(-4, 4, len(ci)))
        return gg.CSR(rows, cols, np.array(rp, np.int32), np.array(ci, np.int32), v)

    A = csr(n, n, 4, True)
    B = csr(m, n, 3, False)
    Bt = gg.CSR(n, m, *H._transpose(m, n, B.rowptr, B.colidx, B.vals))
    return n, m, A, Bt, B, rng.uniform(-1, 1, n), rng.uniform(-1, 1, m)


def _run(torch, fn, n, m, A, Bt, B, rhs1, rhs2):
    d = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    av, btv, bv, r1, r2 = d(A.vals), d(Bt.vals), d(B.vals), d(rhs1), d(rhs2)
    ai, aj = d(A.rowptr, torch.int32), d(A.colidx, torch.int32)
    bti, btj = d(Bt.rowptr, torch.int32), d(Bt.colidx, torch.int32)
    bi, bj = d(B.rowptr, torch.int32), d(B.colidx, torch.int32)
    md = torch.zeros(n + m, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    p = lambda t: t.data_ptr()
    rc = fn(2, n, m, p(av), p(ai), p(aj), p(btv), p(bti), p(btj), p(bv), p(bi), p(bj), p(r1), p(r2), p(md), None)
    assert rc == hk.OK, hk.lib().hykkt_last_error()
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (av, btv, bv, r1, r2, md)]


def _oracle(n, m, A, Bt, B, rhs1, rhs2):
    return list(O.ruiz_scale(2, n, m, (A.rowptr, A.colidx, A.vals), (Bt.rowptr, Bt.colidx, Bt.vals),
                             (B.rowptr, B.colidx, B.vals), rhs1, rhs2))


def _same(got, want):
    for w, g in zip(want, got):
        # same operation order everywhere: identical, tolerance 0
        np.testing.assert_allclose(g, w, rtol=0, atol=0)


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = hk.lib()
    for seed in (1, 2):  # two calls in a row: the second reuses the array as left by the first
        blocks = _square_blocks(seed)
        _same(_run(torch, L.hykkt_ruiz_scale_noalloc, *blocks), _run(torch, L.hykkt_ruiz_scale, *blocks))


def test_noalloc_rectangular_blocks_against_oracle():
    """m != n: B's rows, rhs2 and the scale entries n..n+m-1 sit at offsets
    that a square case cannot tell apart."""
    torch = pytest.importorskip("torch")
    L = hk.lib()
    for n, m, seed in ((700, 350, 3), (300, 900, 4)):
        blocks = _rect_blocks(n, m, seed)
        got = _run(torch, L.hykkt_ruiz_scale_noalloc, *blocks)
        _same(got, _oracle(*blocks))
        _same(got, _run(torch, L.hykkt_ruiz_scale, *blocks))


_FRESH = r"""
import sys
import numpy as np
sys.path[:0] = [{root!r}, {tests!r}]
import torch
import test_zz_no_alloc as T
import hykkt_gb300 as hk
blocks = T._rect_blocks(500, 200, 5)
out = T._run(torch, hk.lib().hykkt_ruiz_scale_noalloc, *blocks)
np.savez({path!r}, *out)
"""


def test_noalloc_first_call_in_fresh_process(tmp_path):
    """A new process whose first call into the library is the no-alloc entry
    point (the array's set-up on the device happens inside that call)."""
    torch = pytest.importorskip("torch")
    path = str(tmp_path / "fresh.npz")
    code = _FRESH.format(root=ROOT, tests=os.path.join(ROOT, "tests"), path=path)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [np.load(path)[f"arr_{i}"] for i in range(6)]
    blocks = _rect_blocks(500, 200, 5)
    _same(got, _oracle(*blocks))
    _same(got, _run(torch, hk.lib().hykkt_ruiz_scale, *blocks))


def test_noalloc_known_answers():
    torch = pytest.importorskip("torch")
    Hm, A, At, rhs = H.ruiz_test_blocks()
    n = Hm.n
    hv, atv, av, r1, r2, md = _run(torch, hk.lib().hykkt_ruiz_scale_noalloc, n, n, Hm, At, A, rhs[:n].copy(),
                                   rhs[n:].copy())
    Hg, Ag, Atg = Hm.copy(), A.copy(), At.copy()
    Hg.vals, Ag.vals, Atg.vals = hv, av, atv
    got = H.ruiz_kat_values(Hg, Ag, Atg, np.concatenate([r1, r2]), md)
    for k, v in H.RUIZ_KAT.items():
        assert abs(got[k] - v) <= 1e-8, k


def test_noalloc_rejects_oversize():
    L = hk.lib()
    cap = L.hykkt_ruiz_scale_noalloc_max_rows()
    assert cap == 1 << 20
    # rejected on the host before any pointer is used or any work is enqueued
    rc = L.hykkt_ruiz_scale_noalloc(2, cap, 1, *([None] * 12), None)
    assert rc == hk.INVALID
    assert b"exceeds the fixed scratch" in L.hykkt_last_error()
