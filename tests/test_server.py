"""Served-solve request queue (hykkt_server_*), host logic on the CPU.

The workers call a Python stand-in for the GPU solve (hykkt_server_create_ex),
so these tests check the queue itself: every request completes with its own
outputs, one plan's requests run one at a time and in submission order,
different plans run concurrently up to the worker count, and shutdown
completes what was queued.
"""
import threading
import time

import numpy as np
import pytest

import hykkt_gb300 as hk


class FakeSolver:
    def __init__(self, delay=0.002):
        self.lock = threading.Lock()
        self.active_plans = set()
        self.active = 0
        self.max_active = 0
        self.order = {}
        self.overlap = False
        self.delay = delay

    def __call__(self, plan, worker, ins, outs):
        with self.lock:
            if plan in self.active_plans:
                self.overlap = True
            self.active_plans.add(plan)
            self.active += 1
            self.max_active = max(self.max_active, self.active)
            self.order.setdefault(plan, []).append(ins[0][0])
        time.sleep(self.delay)
        # the "solution": x[0] = 2 * h[0], y[0] = worker
        outs[0][0] = 2.0 * ins[0][0]
        outs[2][0] = float(worker)
        with self.lock:
            self.active -= 1
            self.active_plans.discard(plan)
        return hk.CG_NOT_CONVERGED if ins[0][0] < 0 else hk.OK


def _arrays(v):
    return [np.array([v], dtype=np.float64)] + [np.zeros(1) for _ in range(7)] + [None]


def _out():
    return tuple(np.zeros(1) for _ in range(4))


def test_server_queue_semantics():
    fake = FakeSolver()
    srv = hk.Server(3, serve_fn=fake)
    plans = [11, 12, 13, 14]
    tickets = {}
    lock = threading.Lock()

    def client(c):
        for k in range(10):
            p = plans[(c + k) % len(plans)]
            v = float(1000 * p + 10 * c + k)
            t = srv.submit(p, arrays=_arrays(v), out=_out())
            with lock:
                tickets[t] = (p, v)

    th = [threading.Thread(target=client, args=(c,)) for c in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for t, (p, v) in tickets.items():
        st, lat, info, out = srv.wait(t)
        assert st == hk.OK
        assert out[0][0] == 2.0 * v
        assert 0 <= out[2][0] < 3
        assert lat >= 0.0
    assert not fake.overlap, "one plan was solved by two workers at once"
    assert 1 < fake.max_active <= 3
    assert srv.stats() == {"completed": 60, "queued": 0, "in_flight": 0}
    srv.close()


def test_server_per_plan_submission_order():
    fake = FakeSolver(delay=0.001)
    srv = hk.Server(4, serve_fn=fake)
    ts = [srv.submit(7, arrays=_arrays(float(i)), out=_out()) for i in range(25)]
    ts += [srv.submit(8, arrays=_arrays(float(100 + i)), out=_out()) for i in range(25)]
    for t in ts:
        assert srv.wait(t)[0] == hk.OK
    assert fake.order[7] == [float(i) for i in range(25)]
    assert fake.order[8] == [float(100 + i) for i in range(25)]
    srv.close()


def test_server_status_errors_and_shutdown_drains():
    fake = FakeSolver(delay=0.003)
    srv = hk.Server(2, serve_fn=fake)
    bad = srv.submit(5, arrays=_arrays(-1.0), out=_out())
    good = [srv.submit(6 + (i % 2), arrays=_arrays(float(i)), out=_out()) for i in range(8)]
    assert srv.wait(bad)[0] == hk.CG_NOT_CONVERGED
    with pytest.raises(hk.HykktError):
        srv.wait(bad)  # collected once
    with pytest.raises(hk.HykktError):
        srv.wait(123456)
    outs = [srv._bufs[t][1] for t in good]
    srv.close()  # completes the queued requests before the workers stop
    assert [o[0][0] for o in outs] == [2.0 * i for i in range(8)]
    assert fake.active == 0


def test_server_rejects_bad_arguments():
    with pytest.raises(hk.HykktError):
        hk.Server(0, serve_fn=FakeSolver())


def test_server_one_waiter_per_ticket():
    """Two threads waiting for one ticket: one collects the result, the other
    is turned away with HYKKT_INVALID (the request is claimed under the
    queue's lock, so it is never read after the first waiter freed it)."""
    fake = FakeSolver(delay=0.3)
    srv = hk.Server(1, serve_fn=fake)
    t = srv.submit(3, arrays=_arrays(4.0), out=_out())
    results, lock = [], threading.Lock()

    def waiter():
        try:
            st, _, _, out = srv.wait(t)
            r = ("ok", st, out[0][0])
        except hk.HykktError:
            r = ("err",)
        with lock:
            results.append(r)

    th = [threading.Thread(target=waiter) for _ in range(2)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert sorted(r[0] for r in results) == ["err", "ok"]
    assert [r for r in results if r[0] == "ok"][0][1:] == (hk.OK, 8.0)
    srv.close()


class FakeMemory:
    """Stand-in plans with sizes: records what is resident and checks that
    the resident bytes never exceed the budget."""

    def __init__(self, sizes, budget, resident=()):
        self.sizes = dict(sizes)
        self.budget = budget
        self.resident = set(resident)
        self.lock = threading.Lock()
        self.peak = sum(self.sizes[p] for p in self.resident)
        self.loads, self.evicts = [], []

    def hooks(self):
        return {"bytes": lambda p: self.sizes[p], "resident": lambda p: p in self.resident,
                "load": self.load, "evict": self.evict}

    def load(self, p):
        with self.lock:
            assert p not in self.resident
            self.resident.add(p)
            self.loads.append(p)
            self.peak = max(self.peak, sum(self.sizes[q] for q in self.resident))
        return hk.OK

    def evict(self, p):
        with self.lock:
            assert p in self.resident
            self.resident.discard(p)
            self.evicts.append(p)
        return hk.OK


def test_managed_server_admits_by_memory_and_evicts_idle_plans():
    sizes = {21: 60, 22: 60, 23: 30, 24: 30}
    mem = FakeMemory(sizes, 100)
    fake = FakeSolver(delay=0.01)

    def solve(plan, worker, ins, outs):
        with mem.lock:
            assert plan in mem.resident, "a plan solved without its device storage"
        return fake(plan, worker, ins, outs)

    srv = hk.Server(3, serve_fn=solve, budget=100, hooks=mem.hooks())
    order = [21, 22, 23, 24, 21, 23, 22, 24, 21, 22]
    ts = [(srv.submit(p, arrays=_arrays(float(10 * i + p)), out=_out()), p, 10 * i + p) for i, p in enumerate(order)]
    for t, p, v in ts:
        st, _, _, out = srv.wait(t)
        assert st == hk.OK and out[0][0] == 2.0 * v
    ms = srv.memory_stats()
    assert mem.peak <= 100 and ms["peak_bytes"] <= 100
    assert ms["evictions"] >= 1 and ms["admissions"] == len(mem.loads)
    assert ms["evictions"] == len(mem.evicts)
    assert ms["resident_bytes"] == sum(sizes[p] for p in mem.resident)
    assert not fake.overlap
    srv.close()


def test_managed_server_oldest_deferred_request_is_not_starved():
    """A large plan waits for memory while small ones keep arriving: its
    reservation stops newer admissions, so it runs before the later small
    requests that need new memory."""
    sizes = {31: 80, 32: 30, 33: 30, 34: 30, 35: 30}
    mem = FakeMemory(sizes, 100, resident=[32])
    done_order, lock = [], threading.Lock()

    def solve(plan, worker, ins, outs):
        time.sleep(0.05 if plan == 32 else 0.01)
        with lock:
            done_order.append(plan)
        outs[0][0] = ins[0][0]
        return hk.OK

    srv = hk.Server(2, serve_fn=solve, budget=100, hooks=mem.hooks())
    t32 = srv.submit(32, arrays=_arrays(1.0), out=_out())   # resident, runs first
    t31 = srv.submit(31, arrays=_arrays(2.0), out=_out())   # 80 bytes: must wait for 32 to end
    later = [srv.submit(p, arrays=_arrays(3.0), out=_out()) for p in (33, 34, 35)]
    for t in [t32, t31] + later:
        assert srv.wait(t)[0] == hk.OK
    assert done_order.index(31) < min(done_order.index(p) for p in (33, 34, 35))
    assert mem.peak <= 100
    assert srv.memory_stats()["deferrals"] >= 1
    srv.close()


def test_managed_server_rejects_a_plan_larger_than_the_budget():
    mem = FakeMemory({41: 500, 42: 10}, 100)
    srv = hk.Server(2, serve_fn=lambda plan, w, ins, outs: hk.OK, budget=100, hooks=mem.hooks())
    big = srv.submit(41, arrays=_arrays(1.0), out=_out())
    small = srv.submit(42, arrays=_arrays(1.0), out=_out())
    assert srv.wait(big)[0] == hk.OOM
    assert srv.wait(small)[0] == hk.OK
    assert 41 not in mem.loads
    srv.close()


def test_managed_server_needs_hooks_with_a_stand_in():
    with pytest.raises(hk.HykktError):
        hk.Server(1, serve_fn=lambda *a: hk.OK, budget=100, hooks={"bytes": lambda p: 1})


def test_heavy_requests_leave_workers_for_small_plans():
    """Two slow requests of large plans and a stream of fast small ones on
    three workers: with at most one heavy request at a time the large plans
    take one worker and the small requests finish long before the second
    large one; heavy requests keep their order."""
    sizes = {51: 1000, 52: 1000, 53: 10, 54: 10}
    mem = FakeMemory(sizes, 10_000)
    lock, active, peak_heavy, done = threading.Lock(), [0], [0], []

    def solve(plan, worker, ins, outs):
        heavy = sizes[plan] >= 500
        with lock:
            if heavy:
                active[0] += 1
                peak_heavy[0] = max(peak_heavy[0], active[0])
        time.sleep(0.3 if heavy else 0.005)
        with lock:
            if heavy:
                active[0] -= 1
            done.append((plan, time.perf_counter()))
        outs[0][0] = ins[0][0]
        return hk.OK

    srv = hk.Server(3, serve_fn=solve, budget=10_000, hooks=mem.hooks())
    srv.set_heavy(500, 1)
    t0 = time.perf_counter()
    heavy = [srv.submit(p, arrays=_arrays(float(p)), out=_out()) for p in (51, 52)]
    light = [srv.submit(53 + k % 2, arrays=_arrays(float(k)), out=_out()) for k in range(20)]
    lat_light = [srv.wait(t)[1] for t in light]
    for t in heavy:
        assert srv.wait(t)[0] == hk.OK
    srv.close()
    assert peak_heavy[0] == 1
    order = [p for p, _ in done if p in (51, 52)]
    assert order == [51, 52]
    t_second_heavy = [t for p, t in done if p == 52][0]
    assert max(t for p, t in done if p in (53, 54)) < t_second_heavy
    assert max(lat_light) < 0.3e3  # ms: no small request waited for a large one


def test_heavy_limit_arguments():
    srv = hk.Server(2, serve_fn=lambda *a: hk.OK)
    with pytest.raises(hk.HykktError):  # a stand-in without sizes
        srv.set_heavy(100, 1)
    srv.set_heavy(0, 0)  # no limit: always accepted
    srv.close()
    mem = FakeMemory({1: 5}, 100)
    srv = hk.Server(2, serve_fn=lambda *a: hk.OK, budget=100, hooks=mem.hooks())
    for bad in (0, 3):
        with pytest.raises(hk.HykktError):
            srv.set_heavy(100, bad)
    srv.set_heavy(100, 2)
    srv.close()


def test_wait_reports_where_the_latency_went():
    """queue + admission + solve phases add up to the latency; the solve
    phase holds the stand-in's time, admission the load hook's."""
    sizes = {61: 10}
    mem = FakeMemory(sizes, 100)
    slow_load = mem.load

    def load(p):
        time.sleep(0.05)
        return slow_load(p)

    hooks = mem.hooks()
    hooks["load"] = load

    def solve(plan, worker, ins, outs):
        time.sleep(0.1)
        return hk.OK

    srv = hk.Server(1, serve_fn=solve, budget=100, hooks=hooks)
    t1 = srv.submit(61, arrays=_arrays(1.0), out=_out())
    t2 = srv.submit(61, arrays=_arrays(2.0), out=_out())
    for t, queued in ((t1, False), (t2, True)):
        st, lat, info, _ = srv.wait(t)
        assert st == hk.OK
        q, a, sv = info["queue_ms"], info["admission_ms"], info["solve_ms"]
        assert min(q, a, sv) >= 0.0 and abs(q + a + sv - lat) < 1.0
        assert sv >= 95.0
        assert (a >= 45.0) == (not queued)  # only the first request loads the plan
        assert (q >= 95.0) == queued        # the second waits for the first's solve
    srv.close()


def test_heavy_request_waiting_for_a_worker_reserves_no_memory():
    """A heavy request held back by the worker limit does not claim memory:
    small plans that need new memory are still admitted beside the heavy
    plan that runs."""
    sizes = {71: 60, 72: 60, 73: 5, 74: 5, 75: 5}
    mem = FakeMemory(sizes, 100)
    lock, order = threading.Lock(), []

    def solve(plan, worker, ins, outs):
        time.sleep(0.3 if sizes[plan] >= 50 else 0.01)
        with lock:
            order.append(plan)
        return hk.OK

    srv = hk.Server(3, serve_fn=solve, budget=100, hooks=mem.hooks())
    srv.set_heavy(50, 1)
    heavy = [srv.submit(p, arrays=_arrays(1.0), out=_out()) for p in (71, 72)]
    time.sleep(0.05)  # 71 runs, 72 waits for the heavy worker
    small = [srv.submit(p, arrays=_arrays(1.0), out=_out()) for p in (73, 74, 75)]
    for t in small + heavy:
        assert srv.wait(t)[0] == hk.OK
    ms = srv.memory_stats()
    srv.close()
    # the small plans ran before the second heavy one, whose 60 bytes only fit
    # after the first heavy plan was evicted
    assert order.index(72) > max(order.index(p) for p in (73, 74, 75))
    assert mem.peak <= 100 and ms["peak_bytes"] <= 100
    assert 71 in mem.evicts


def test_cancel_withdraws_only_queued_requests():
    """One worker, a slow first request: the queued second one can be
    withdrawn (its wait reports CANCELLED), the running first one cannot,
    and the third completes; a managed server forgets the withdrawn
    request's claim on its plan."""
    started = threading.Event()

    def solve(plan, worker, ins, outs):
        started.set()
        time.sleep(0.2 if ins[0][0] == 1.0 else 0.01)
        outs[0][0] = ins[0][0]
        return hk.OK

    mem = FakeMemory({81: 10, 82: 10}, 100)
    srv = hk.Server(1, serve_fn=solve, budget=100, hooks=mem.hooks())
    t1 = srv.submit(81, arrays=_arrays(1.0), out=_out())
    started.wait(5.0)
    t2 = srv.submit(82, arrays=_arrays(2.0), out=_out())
    t3 = srv.submit(81, arrays=_arrays(3.0), out=_out())
    assert srv.cancel(t2) is True
    assert srv.cancel(t1) is False  # already running
    st2, lat2, info2, out2 = srv.wait(t2)
    assert st2 == hk.CANCELLED and out2[0][0] == 0.0
    assert srv.wait(t1)[0] == hk.OK and srv.wait(t3)[0] == hk.OK
    assert 82 not in mem.loads  # the withdrawn request never admitted its plan
    with pytest.raises(hk.HykktError):
        srv.cancel(t2)  # collected
    srv.close()
