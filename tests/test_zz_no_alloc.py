"""hykkt_ruiz_scale_noalloc: Ruiz scaling with its scale vector in a fixed
device array (no allocation), against hykkt_ruiz_scale on the same inputs.

Kept in its own file, collected last, so that it runs both after the other
GPU tests and alone in a fresh process (the first call on the device does
the array's set-up).
"""
import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk

pytestmark = pytest.mark.gpu


def _blocks(torch, seed):
    """Ruiz driver blocks with seeded random values (same patterns)."""
    Hm, A, At, rhs = H.ruiz_test_blocks()
    rng = np.random.default_rng(seed)
    for M in (Hm, A, At):
        M.vals = M.vals * rng.uniform(0.5, 2.0, len(M.vals))
    rhs = rhs * rng.uniform(-1.0, 1.0, len(rhs))
    return Hm, A, At, rhs


def _run(torch, fn, Hm, A, At, rhs, stream):
    n = Hm.n
    d = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    hv, av, atv, r = d(Hm.vals), d(A.vals), d(At.vals), d(rhs)
    hi, hj = d(Hm.rowptr, torch.int32), d(Hm.colidx, torch.int32)
    ai, aj = d(A.rowptr, torch.int32), d(A.colidx, torch.int32)
    ati, atj = d(At.rowptr, torch.int32), d(At.colidx, torch.int32)
    md = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    p = lambda t: t.data_ptr()
    rc = fn(2, n, n, p(hv), p(hi), p(hj), p(atv), p(ati), p(atj), p(av), p(ai), p(aj), p(r), r.data_ptr() + 8 * n,
            p(md), stream)
    assert rc == hk.OK, hk.lib().hykkt_last_error()
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (hv, atv, av, r, md)]


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = hk.lib()
    for seed in (1, 2):  # two calls in a row: the second reuses the array as left by the first
        blocks = _blocks(torch, seed)
        want = _run(torch, L.hykkt_ruiz_scale, *blocks, None)
        got = _run(torch, L.hykkt_ruiz_scale_noalloc, *blocks, None)
        for w, g in zip(want, got):
            # same kernels and operation order: identical up to the tolerance of 0
            np.testing.assert_allclose(g, w, rtol=0, atol=0)


def test_noalloc_known_answers():
    torch = pytest.importorskip("torch")
    Hm, A, At, rhs = H.ruiz_test_blocks()
    hv, atv, av, r, md = _run(torch, hk.lib().hykkt_ruiz_scale_noalloc, Hm, A, At, rhs, None)
    Hg, Ag, Atg = Hm.copy(), A.copy(), At.copy()
    Hg.vals, Ag.vals, Atg.vals = hv, av, atv
    got = H.ruiz_kat_values(Hg, Ag, Atg, r, md)
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
