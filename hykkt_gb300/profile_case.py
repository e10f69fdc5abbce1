"""One solve of a synthetic grid system for kernel profilers.

The solve graph of a plan holds conditional (while) nodes, whose kernel
nodes profilers cannot capture, so this runs one solve through the graph (to
upload the inputs) and then the same solve again as plain stream launches
(Plan.run_stages), which a profiler can capture kernel by kernel.

    python -m hykkt_gb300.profile_case --n-bus 10000 [--cg-itmax 400] [--solve-piece 2800]
"""
from __future__ import annotations

import argparse
import json

from . import Plan
from . import gridgen as gg


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-bus", type=int, default=2000)
    ap.add_argument("--gamma", type=float, default=1e5)
    ap.add_argument("--cg-itmax", type=int, default=400)
    ap.add_argument("--refine-max", type=int, default=1)
    ap.add_argument("--solve-piece", type=int, default=0, help="max columns of one solve item (0: whole supernodes)")
    a = ap.parse_args()
    grid = gg.make_grid(a.n_bus, 0)
    s = gg.make_system(grid, 1, a.gamma, (1e-10, 1e8), (1e-10, 1e8))
    plan = Plan(s, solve_piece=a.solve_piece)
    plan.set_accuracy(a.cg_itmax, 1e-12, a.refine_max, 1e-8)
    plan.solve(s)
    stages = plan.run_stages(3)
    info = plan.info()
    print(json.dumps({"n_bus": a.n_bus, "stage_ms": stages, "cg_iterations_total": info["cg_iterations_total"],
                      "rel_residual_full": info["rel_residual_full"]}))


if __name__ == "__main__":
    main()
