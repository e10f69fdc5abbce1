"""Batched systems of different sparsity and served solves on the GPU.

* mixed batch (the shape of the 256-grid batched workload, at sizes the
  oracle finishes in seconds): one plan per pattern, all plans solving at
  once on their own streams; every solution equals the same plan's solve
  run alone bit for bit (scheduling does not change any sum), matches the
  oracle with the same accuracy controls, and reaches the 1e-8 residual;
* served solves (the shape of the multi-client workload): client threads
  submit solves of their own plans to one request queue; every answer equals
  the direct solve of the same values bit for bit.
"""
import threading

import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ACC = dict(cg_itmax=3000, cg_rtol=1e-12, refine_max=4, refine_target=1e-8)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def mixed_systems(count, lo, hi, seed=0, dx=(1e-4, 1e4), ds=(1e-4, 1e4)):
    """Per-system grids with log-uniform bus counts, gamma 1e4 (D ranges of
    the synthetic parity grids, so that two factorizations of the same
    system agree to 1e-8 and the oracle comparison is meaningful)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(int)
    return [gg.make_system(gg.make_grid(int(n), seed + i), 100 + i, 1e4, dx, ds) for i, n in enumerate(sizes)]


def test_mixed_sparsity_batch_concurrent():
    systems = mixed_systems(5, 200, 2000, seed=7)
    assert len({s.n_x for s in systems}) == len(systems)
    plans = [hk.Plan(s) for s in systems]
    for p in plans:
        p.set_accuracy(**ACC)
    alone = []
    for p, s in zip(plans, systems):
        assert p.solve(s) == hk.OK
        alone.append(tuple(v.copy() for v in p.solution()))
    for p in plans:
        p.set_concurrency(len(plans))
    for p, s in zip(plans, systems):  # every plan on its own stream, all in flight
        p.solve(s, sync=False)
    for p in plans:
        assert p.wait() == hk.OK
    for p, s, a in zip(plans, systems, alone):
        sol = p.solution()
        for u, v in zip(sol, a):
            assert np.array_equal(u, v)
        assert p.info()["rel_residual_full"] <= 1e-8
        assert H.kkt_residual(s, *sol) <= 1e-8
        r = O.solve(s, perm=p.perm(), itmax=ACC["cg_itmax"], rtol=ACC["cg_rtol"], refine_max=ACC["refine_max"],
                    refine_target=ACC["refine_target"])
        for got, key in zip(sol, ("x", "s", "y", "yd")):
            assert rel(got, r[key]) < 1e-8, key


def test_served_clients_match_direct_solves():
    grids = [gg.make_grid(n, 20 + i) for i, n in enumerate((300, 600, 900))]
    seqs = [[gg.make_system(g, 200 + 10 * i + k, 1e4, (1e-4, 1e4), (1e-4, 1e4)) for k in range(3)]
            for i, g in enumerate(grids)]
    plans = [hk.Plan(seq[0]) for seq in seqs]
    direct = []
    for p, seq in zip(plans, seqs):
        p.set_accuracy(**ACC)
        d = []
        for s in seq:
            assert p.solve(s) == hk.OK
            d.append((tuple(v.copy() for v in p.solution()), p.info()["rel_residual_full"]))
        direct.append(d)
    srv = hk.Server(2)
    for p in plans:
        p.set_concurrency(2)
    got = [[None] * 3 for _ in plans]
    errors = []

    def client(i):
        try:
            ts = [srv.submit(plans[i], s) for s in seqs[i]]
            for k, t in enumerate(ts):
                st, lat, info, out = srv.wait(t)
                assert st == hk.OK and lat > 0.0
                got[i][k] = (out, info["rel_residual_full"])
        except Exception as e:  # reported by the main thread
            errors.append(e)

    th = [threading.Thread(target=client, args=(i,)) for i in range(len(plans))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    assert srv.stats()["completed"] == 9
    srv.close()
    for i in range(len(plans)):
        for k in range(3):
            (out, res), (ref, ref_res) = got[i][k], direct[i][k]
            for u, v in zip(out, ref):
                assert np.array_equal(u, v)
            assert res == ref_res <= 1e-8


def test_managed_server_evicts_plans_and_matches_direct_solves():
    """Admission by device memory: three plans created without device
    storage, a budget that holds two of them, requests of all three
    interleaved.  Plans are evicted and reloaded as the queue needs them;
    every answer equals a direct solve bit for bit, and the bytes resident
    never exceed the budget."""
    grids = [gg.make_grid(n, 40 + i) for i, n in enumerate((300, 600, 900))]
    seqs = [[gg.make_system(g, 400 + 10 * i + k, 1e4, (1e-4, 1e4), (1e-4, 1e4)) for k in range(3)]
            for i, g in enumerate(grids)]
    direct = []
    for seq in seqs:
        p = hk.Plan(seq[0])
        p.set_accuracy(**ACC)
        d = []
        for s in seq:
            assert p.solve(s) == hk.OK
            d.append(tuple(v.copy() for v in p.solution()))
        direct.append(d)
        p.close()
    plans = [hk.Plan(seq[0], deferred=True) for seq in seqs]
    sizes = []
    for p in plans:
        res, b = p.residency()
        assert not res and b > 0
        sizes.append(b)
        p.set_accuracy(**ACC)
        p.set_concurrency(2)
    budget = sum(sorted(sizes)[1:])  # the two largest fit, all three do not
    srv = hk.Server(2, budget=budget)
    tickets = []
    for k in range(3):
        for i in range(3):
            tickets.append((i, k, srv.submit(plans[i], seqs[i][k])))
    for i, k, t in tickets:
        st, lat, info, out = srv.wait(t)
        assert st == hk.OK
        for u, v in zip(out, direct[i][k]):
            assert np.array_equal(u, v)
        assert info["rel_residual_full"] <= 1e-8
    ms = srv.memory_stats()
    srv.close()
    assert ms["budget"] == budget and ms["peak_bytes"] <= budget
    assert ms["evictions"] >= 1 and ms["admissions"] >= 3
    resident = [p.residency()[0] for p in plans]
    assert sum(resident) <= 2


def test_reload_while_another_plan_holds_the_gpu():
    """A plan whose device storage is released and taken back solves on a
    non-blocking stream right after the reload, while another plan's solves
    keep every SM busy: the reload's copies and zero fills have completed
    before the solve starts (a fill still queued behind the other plan's
    kernels would overwrite the solve's state), so every status is OK and
    every answer equals the first one bit for bit."""
    big = gg.make_system(gg.make_grid(3000, 71), 710, 1e4, (1e-4, 1e4), (1e-4, 1e4))
    small = gg.make_system(gg.make_grid(400, 72), 720, 1e4, (1e-4, 1e4), (1e-4, 1e4))
    pa, pb = hk.Plan(big), hk.Plan(small, deferred=True)
    for p in (pa, pb):
        p.set_accuracy(**ACC)
    assert pb.solve(small) == hk.OK
    first = tuple(v.copy() for v in pb.solution())
    stop, a_status = threading.Event(), []

    def keep_busy():
        while not stop.is_set():
            a_status.append(pa.solve(big))

    th = threading.Thread(target=keep_busy)
    th.start()
    try:
        for _ in range(8):
            pb.release_device()
            assert not pb.residency()[0]
            assert pb.solve(small) == hk.OK
            for u, v in zip(pb.solution(), first):
                assert np.array_equal(u, v)
    finally:
        stop.set()
        th.join()
    assert a_status and set(a_status) == {hk.OK}
    pa.close()
    pb.close()
