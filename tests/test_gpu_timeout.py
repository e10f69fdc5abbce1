"""Bounded device waits of the persistent triangular solves, on the GPU.

The solve kernels wait on dependency counters with a bounded poll loop
(kernels.cuh wait_ge).  A test hook makes every wait ask for one signal more
than any task sends -- a count that nothing reaches -- with a short spin
limit: the solve must end by itself, report HYKKT_TIMEOUT through the host,
and leave the context usable, so that the same plan solves correctly once
the hook is off.  No fault, trap or endless loop is involved.
"""
import time

import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_plan_recovers():
    s = H.small_grid_system(n_bus=400, seed=5)
    plan = hk.Plan(s)
    plan.set_accuracy(cg_itmax=5000, cg_rtol=1e-11, refine_max=4, refine_target=1e-8)
    assert plan.solve(s) == hk.OK
    x_ok = plan.solution()[0]

    plan.debug_set("spin_limit", 1 << 14)
    plan.debug_set("unsatisfiable_waits", 1)
    t0 = time.perf_counter()
    with pytest.raises(hk.HykktError) as e:
        plan.solve(s)
    dt = time.perf_counter() - t0
    assert e.value.code == hk.TIMEOUT and "gave up" in str(e.value)
    assert plan.info()["status"] == hk.TIMEOUT
    # one spin limit, then every other wait returns at once and the CG stops
    assert dt < 30.0
    assert plan.info()["cg_iterations"] <= 1

    plan.debug_set("unsatisfiable_waits", 0)
    plan.debug_set("spin_limit", 0)
    assert plan.solve(s) == hk.OK
    info = plan.info()
    assert info["rel_residual_full"] <= 1e-8
    # same inputs, same plan: the same answer as before the timed-out solve
    assert np.array_equal(plan.solution()[0], x_ok)


def test_debug_settings_are_validated():
    s = H.small_grid_system(n_bus=120, seed=0)
    plan = hk.Plan(s)
    with pytest.raises(hk.HykktError):
        plan.debug_set("no_such_setting", 1)
    with pytest.raises(hk.HykktError):
        plan.debug_set("spin_limit", -1)
