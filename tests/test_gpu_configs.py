"""GPU parity on the measured workload shapes, against the oracle.

* the 500-bus single solve (gamma 1e4, D_x in [1e-8, 1e4], D_s in
  [1e-8, 1e8], CG tolerance 1e-12 absolute as in the reference,
  SchurComplementConjugateGradient.hpp:125-126), to a 4-block residual
  <= 1e-8;
* one system of the 10,000-bus interior-point sequence (gamma 1e5, D_x and
  D_s in [1e-10, 1e8]) with the benchmark's accuracy settings (marked slow:
  the oracle needs about a minute on one core);
* the accuracy contract: a solve that ends above the requested residual
  target reports HYKKT_ACCURACY_NOT_MET, never HYKKT_OK.

Solutions are compared at 1e-8 relative (FP64 path, different summation
orders in the factorization).
"""
import numpy as np
import pytest

import helpers as H
import hykkt_gb300 as hk
from hykkt_gb300 import gridgen as gg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-8


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _compare(s, plan, **acc):
    x, ds, y, yd = plan.solution()
    info = plan.info()
    r = O.solve(s, perm=plan.perm(), **acc)
    for got, key in ((x, "x"), (ds, "s"), (y, "y"), (yd, "yd")):
        assert rel(got, r[key]) < REL_TOL, (key, rel(got, r[key]))
    assert info["rel_residual_full"] <= 1e-8, info
    assert r.scalar("rel_res_full") <= 1e-8
    # the GPU's compensated residual agrees with a host residual of its solution
    assert abs(info["rel_residual_full"] - H.kkt_residual(s, x, ds, y, yd)) < 1e-9
    return info, r


def test_grid500_single_solve_vs_oracle():
    _, (s,) = gg.workload_systems("grid500")
    plan = hk.Plan(s)
    plan.set_accuracy(cg_itmax=5000, cg_rtol=0.0, refine_max=4, refine_target=1e-8)
    plan.set_refine_rtol(1e-4)
    assert plan.solve(s) == hk.OK
    info, r = _compare(s, plan, itmax=5000, tol=1e-12, rtol=0.0, refine_max=4, refine_target=1e-8,
                       refine_rtol=1e-4)
    # same recurrence, same stopping tests: the same number of iterations
    # (over the first CG and the correction's) and refinement steps
    # (the correction's right-hand side is a residual, rounded differently on
    # the two sides: its CG may differ by a few iterations)
    # (cg_iterations is the last CG run's count here, the correction's: totals compare)
    assert abs(info["cg_iterations_total"] - r.scalar("cg_iters_total")) <= 0.05 * r.scalar("cg_iters_total")
    assert info["refine_steps"] == r.scalar("refine_steps")


def test_grid500_reference_settings_do_not_converge():
    """With the reference's own budget (100 iterations, SchurCG.hpp:125) the
    500-bus system stops far from the solution; the GPU path and the oracle
    stop at the same iterate."""
    _, (s,) = gg.workload_systems("grid500")
    plan = hk.Plan(s)
    assert plan.solve(s) == hk.CG_NOT_CONVERGED
    info = plan.info()
    r = O.solve(s, perm=plan.perm())
    assert info["cg_iterations"] == 100 == r.scalar("cg_iters")
    assert abs(info["rel_residual"] - r.scalar("rel_res_ref")) <= 1e-6 * r.scalar("rel_res_ref")
    x = plan.solution()[0]
    assert rel(x, r["x"]) < 1e-6


@pytest.mark.slow
def test_grid10k_sequence_system_vs_oracle():
    _, ss = gg.workload_systems("grid10k_seq20", systems=1)
    s = ss[0]
    plan = hk.Plan(s)
    acc = dict(cg_itmax=5000, cg_rtol=1e-11, refine_max=4, refine_target=1e-8)
    plan.set_accuracy(**acc)
    plan.set_refine_rtol(1e-4)
    assert plan.solve(s) == hk.OK
    info, r = _compare(s, plan, itmax=5000, tol=1e-12, rtol=1e-11, refine_max=4, refine_target=1e-8,
                       refine_rtol=1e-4)
    assert info["refine_steps"] == r.scalar("refine_steps")


def test_accuracy_target_missed_is_reported():
    s = H.small_grid_system(n_bus=300, seed=7)
    plan = hk.Plan(s)
    # one correction cannot reach 1e-30: the solve reports the miss
    plan.set_accuracy(cg_itmax=5000, cg_rtol=1e-11, refine_max=1, refine_target=1e-30)
    assert plan.solve(s) == hk.ACCURACY_NOT_MET
    info = plan.info()
    assert info["status"] == hk.ACCURACY_NOT_MET
    assert info["refine_steps"] == 1 and 0 < info["rel_residual_full"] <= 1e-8
    x = plan.solution()[0]  # the best iterate stays readable
    assert np.isfinite(x).all()
    # a reachable target on the same plan
    plan.set_accuracy(cg_itmax=5000, cg_rtol=1e-11, refine_max=4, refine_target=1e-8)
    assert plan.solve(s) == hk.OK
    assert plan.info()["status"] == hk.OK
