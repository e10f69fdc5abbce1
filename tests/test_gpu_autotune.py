"""Autotuner of the triangular-solve layout (hykkt_plan_autotune), on the GPU.

The tuner builds candidate layouts from the plan's patterns and ordering,
times concurrent solves of each and keeps the fastest; the choice is cached
per pattern and share.  A tuned plan must solve exactly the problem the
untuned plan solves (same ordering, same accuracy settings): solutions agree
with the oracle at 1e-8, and a cached choice reproduces the tuned layout.
"""
import numpy as np
import pytest

import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_autotune_picks_a_measured_layout_and_caches_it(tmp_path):
    grid = gg.make_grid(1500, 9)
    s0 = gg.make_system(grid, 1, 1e5, (1e-10, 1e8), (1e-10, 1e8))
    s1 = gg.make_system(grid, 2, 1e5, (1e-10, 1e8), (1e-10, 1e8))
    cache = str(tmp_path / "tune.txt")
    plan = hk.Plan(s0)
    plan.set_accuracy(cg_itmax=5000, cg_rtol=1e-11, refine_max=4, refine_target=1e-8)
    plan.set_refine_rtol(1e-4)
    perm = plan.perm()
    t = plan.autotune(s0, share=2, cache=cache)
    assert not t["from_cache"] and t["candidates"] >= 4
    assert t["concurrent"] == 2
    rates = [c["solves_per_s"] for c in t["timed"]]
    assert max(rates) == pytest.approx(t["best_solves_per_s"])
    chosen = [c for c in t["timed"] if c["solves_per_s"] == max(rates)][0]
    assert (chosen["solve_piece"], chosen["warp_subtree"], chosen["chunk_fma"]) == \
        (t["solve_piece"], t["warp_subtree"], t["chunk_fma"])
    # the tuned plan keeps the ordering and the accuracy settings
    assert np.array_equal(plan.perm(), perm)
    assert plan.solve(s1) == hk.OK
    x = plan.solution()
    r = O.solve(s1, perm=perm, itmax=5000, rtol=1e-11, refine_max=4, refine_target=1e-8, refine_rtol=1e-4)
    for g, key in zip(x, ("x", "s", "y", "yd")):
        assert rel(g, r[key]) < 1e-8, key
    assert plan.info()["rel_residual_full"] <= 1e-8
    # a second plan of the pattern takes the cached layout without timing
    p2 = hk.Plan(s0)
    p2.set_accuracy(cg_itmax=5000, cg_rtol=1e-11, refine_max=4, refine_target=1e-8)
    p2.set_refine_rtol(1e-4)
    t2 = p2.autotune(s0, share=2, cache=cache)
    assert t2["from_cache"] and t2["candidates"] == 0
    assert (t2["solve_piece"], t2["warp_subtree"], t2["chunk_fma"]) == \
        (t["solve_piece"], t["warp_subtree"], t["chunk_fma"])
    assert p2.solve(s1) == hk.OK
    for a, b in zip(p2.solution(), x):
        assert np.array_equal(a, b)  # same layout, same inputs: the same answer
