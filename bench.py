"""Benchmark of the HyKKT KKT solve path on one GB300 (or N replicas).

Workload (default): 20 same-sparsity FP64 KKT systems on a synthetic
10,000-bus grid (n_x = 24,000, m_c = 20,000, m_d = 28,000; gamma = 1e5;
D_x, D_s log-uniform in [1e-10, 1e8]; seeded).  A solve = one full KKT
solve of a system of the sequence (upload of the values, H~, Ruiz, Hgamma,
multifrontal Cholesky, Schur CG, recovery, 4-block residual); the symbolic
plan is built once before timing, as the reference does on its first
execute().

Batched (the headline): B plans of the pattern (clones sharing one symbolic
analysis), one stream each; one step = B solves of B different systems in
flight at once.  Plain: one plan, one solve per step, sequentially.

* value: batched solves/s with the inputs resident in HBM (device-to-device
  upload inside the timed region), CUDA events around each step.
* plain: the same for one plan (solves/s, p50/p99 latency per solve).
* e2e: batched solves through the C ABI from host buffers (pinned staging,
  H2D of all values and right-hand sides, D2H of dx, ds, dy, dyd).
* roofline: the dominant kernel of one uncaptured solve (CUDA events around
  every launch), its algorithmic FLOPs / bytes per launch over its measured
  average duration.
* cpu_baseline: the CPU port (oracle/, supernodal Cholesky and CG on all
  host threads) on a bounded sample: two complete solves of the workload.

--impl reference times the CPU port, one complete solve per step (the
reference has no CPU solve path); --impl refgpu times the reference's own
GPU build (cuSPARSE/cuSOLVER, built from its sources by oracle/ref_build.py)
through its public API.
"""
from __future__ import annotations

import os

# Concurrent plans run on separate streams; with CUDA's default of 8
# hardware work queues, 8 plan streams plus the framework's own streams alias
# and about half of the plans' graphs wait behind others' (measured: graph
# time 1.0 s per solve against 2.0 s per stream cycle).  32 queues let every
# plan's graph run at once.  Must be set before the CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import argparse
import json
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "KKT solves/s + p50/p99 latency at rel. residual <=1e-8, batched vs plain"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "refgpu"])
    ap.add_argument("--workload", default="grid10k_seq20")
    ap.add_argument("--n-bus", type=int, default=None)
    ap.add_argument("--systems", type=int, default=None)
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-port baseline of the main line")
    ap.add_argument("--refgpu-converged", type=int, default=2,
                    help="refgpu: systems also solved with the CG budget raised to --cg-itmax (0 = skip)")
    ap.add_argument("--refgpu-timeout", type=float, default=1500.0)
    ap.add_argument("--refgpu-calls", type=int, default=-1,
                    help="refgpu: numeric calls after the first execute() (-1 = one per system)")
    # accuracy mode: CG budget / relative tolerance and refinement on the full
    # KKT system (the reference's values are 100 / 0 / 0)
    ap.add_argument("--cg-itmax", type=int, default=5000)
    ap.add_argument("--cg-rtol", type=float, default=1e-11)
    ap.add_argument("--refine-max", type=int, default=4)
    ap.add_argument("--refine-target", type=float, default=1e-8)
    ap.add_argument("--refine-rtol", type=float, default=1e-4,
                    help="relative CG tolerance of the refinement corrections")
    ap.add_argument("--batch", type=int, default=8, help="plans solving concurrently (1 = plain only)")
    ap.add_argument("--served-seconds", type=float, default=60.0, help="served workload: seconds per load level")
    ap.add_argument("--served-sizes", default="1000,5000,20000,70000", help="served workload: bus counts of the clients")
    ap.add_argument("--served-clients", type=int, default=16, help="served workload: clients per size")
    ap.add_argument("--served-heavy-gb", type=float, default=50.0,
                    help="served workload: requests of plans of at least this many GB of device storage take at most "
                         "a quarter of the workers (0: no limit)")
    ap.add_argument("--share", type=int, default=-1,
                    help="batched: concurrency share of every plan (-1 = batch)")
    ap.add_argument("--mixed-share", type=int, default=0,
                    help="mixed workload: concurrency share of every plan in the batched pass (0 = by size)")
    ap.add_argument("--solve-piece", type=int, default=-1,
                    help="batched plans: max columns of one triangular-solve item (0 = whole supernodes, "
                         "-1 = chosen by the autotuner)")
    ap.add_argument("--plain-piece", type=int, default=-1,
                    help="plain plan: max columns of one triangular-solve item (0 = whole supernodes, "
                         "-1 = chosen by the autotuner)")
    ap.add_argument("--tune-cache", default=None, help="autotuner cache file (default: none, tune every run)")
    return ap.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = os.environ.get("HYKKT_BENCH_BACKEND", "nccl")
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.samples.append([t.strip() for t in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and "Active" in s[3 + i]
                          and "Not" not in s[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def workload(args):
    from hykkt_gb300 import gridgen as gg
    w = gg.WORKLOADS[args.workload]
    nb = args.n_bus or w["n_bus"]
    ns = args.systems or w["systems"]
    grid = gg.make_grid(nb, 0)
    systems = [gg.make_system(grid, 1 + i, w["gamma"], w["dx"], w["ds"]) for i in range(ns)]
    cfg = {"workload": args.workload, "n_bus": nb, "systems": ns, "n_x": systems[0].n_x, "m_c": systems[0].m_c,
           "m_d": systems[0].m_d, "gamma": w["gamma"], "dx_range": list(w["dx"]), "ds_range": list(w["ds"]),
           "nnz_H": systems[0].H.nnz, "nnz_Jc": systems[0].Jc.nnz, "nnz_Jd": systems[0].Jd.nnz}
    return systems, cfg


def reference_ordering(s):
    """The reference's host ordering (cusolverSpXcsrsymamdHost on the
    H_gamma pattern, src/PermClass.cpp:88-95), timed alone: (perm, seconds,
    note)."""
    from oracle import ref_ordering as RO
    perm, t_order, _ = RO.timed_symamd(s)
    return perm, t_order, "reference symamd (cusolverSpXcsrsymamdHost), host"


def port_solves(systems, idxs, threads, perm, args):
    """Complete solves of systems[idxs] by the CPU port (oracle/, the
    supernodal factorization and CG on `threads` host threads), to the same
    accuracy target as the GPU path; each timed on its own.  Returns
    [(seconds, rel. residual, CG iterations)]."""
    from oracle import oracle as O
    O.set_threads(threads)
    out = []
    try:
        for i in idxs:
            t = time.perf_counter()
            r = O.solve(systems[i], perm=perm, itmax=args.cg_itmax, tol=1e-12, rtol=args.cg_rtol,
                        refine_max=args.refine_max, refine_target=args.refine_target, refine_rtol=args.refine_rtol)
            out.append((time.perf_counter() - t, r.scalar("rel_res_full"), r.scalar("cg_iters_total")))
    finally:
        O.set_threads(1)
    return out


def cpu_baseline(systems, args) -> dict:
    """Bounded sample: one untimed solve (the once-per-pattern supernodal
    analysis happens there), then two complete timed solves."""
    threads = os.cpu_count() or 1
    try:
        perm, t_order, note = reference_ordering(systems[0])
    except Exception as e:  # noqa: BLE001 - reported, not fatal for the GPU line
        return {"value": None, "unit": "solves/s", "cores": threads, "kind": "port",
                "sample": f"unavailable: {e}"}
    port_solves(systems, [0], threads, perm, args)
    res = port_solves(systems, [1 % len(systems), 2 % len(systems)], threads, perm, args)
    t = sum(r[0] for r in res)
    return {"value": len(res) / t, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"{len(res)} complete solves (systems 1-2 of the sequence) by the CPU port (oracle/: H~, Ruiz, "
                      f"Hgamma, supernodal Cholesky, Schur CG, recovery, refinement to rel. residual <= "
                      f"{args.refine_target:g}) on {threads} threads, {t:.1f} s; the reference's host ordering "
                      f"({note}) timed apart: {t_order:.2f} s once per pattern",
            "ordering_s": t_order, "rel_residual_full_max": float(max(r[1] for r in res)),
            "cg_iterations_total_mean": float(np.mean([r[2] for r in res]))}


def run_reference(args, rank, world):
    """The reference arm: the reference has no CPU solve path, so this times
    the CPU port (oracle/) on all host threads, one complete solve per step,
    on the same workload and accuracy target; the reference's own host
    ordering is computed once and timed apart."""
    systems, cfg = workload(args)
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    try:
        perm, t_order, note = reference_ordering(systems[0])
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"the reference's host ordering could not run: {e}"}))
        return
    idx = lambda k: k % len(systems)
    port_solves(systems, [idx(k) for k in range(args.warmup)], threads, perm, args)
    res = port_solves(systems, [idx(args.warmup + k) for k in range(args.steps)], threads, perm, args)
    times = [r[0] for r in res]
    v = len(times) / sum(times)
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg,
            "p50_ms": float(np.percentile(times, 50) * 1e3), "p99_ms": float(np.percentile(times, 99) * 1e3),
            "rel_residual_full_max": float(max(r[1] for r in res)),
            "solves_above_1e-8": int(sum(r[1] > args.refine_target for r in res)),
            "cg_iterations_total_mean": float(np.mean([r[2] for r in res])),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"each step: one complete solve by the CPU port (oracle/, supernodal Cholesky "
                                       f"and Schur CG on {threads} threads; the reference has no CPU solve path), "
                                       f"to rel. residual <= {args.refine_target:g}; the reference's host ordering "
                                       f"({note}) timed apart: {t_order:.2f} s once per pattern",
                             "ordering_s": t_order},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_refgpu(args, rank, world):
    """The reference's own GPU build (cuSPARSE/cuSOLVER, its sources built by
    oracle/ref_build.py), through its public API as its two-system driver
    uses it: the first execute() (symbolic + numeric) reported apart, then
    one execute() per system of the sequence (wall clock around each, device
    synchronised on both sides).  Stock settings (CG budget 100), and a
    second run with the CG budget raised to --cg-itmax on the first
    --refgpu-converged systems.  The reference has no refinement, so neither
    run reaches the 1e-8 target on these grids; the lines report what it
    reaches."""
    from oracle import refgpu
    systems, cfg = workload(args)
    if rank != 0:
        return
    if not refgpu.available():
        print(json.dumps({"impl": "refgpu", "unavailable": refgpu.why_unavailable()}))
        return

    def summary(recs):
        num = [r for r in recs if not r["first"]] or recs  # only the first call was run
        wall = [r["wall_ms"] for r in num]
        return {"solves": len(num), "value": len(num) / (sum(wall) / 1e3), "unit": "solves/s",
                "p50_ms": float(np.percentile(wall, 50)), "p99_ms": float(np.percentile(wall, 99)),
                "event_ms_mean": float(np.mean([r["event_ms"] for r in num])),
                "first_call_ms": recs[0]["wall_ms"], "cg_iterations": [r["cg_iterations"] for r in num],
                "cg_converged": sum(bool(r["cg_converged"]) for r in num),
                "rel_residual_max": float(max(r["rel_residual"] for r in num)),
                "rel_residual_min": float(min(r["rel_residual"] for r in num)),
                "execute_returned_1": sum(r["execute"] != 0 for r in num)}

    try:
        calls = None if args.refgpu_calls < 0 else args.refgpu_calls
        stock = summary(refgpu.run(systems, calls=calls, timeout=args.refgpu_timeout)[0])
    except RuntimeError as e:
        print(json.dumps({"impl": "refgpu", "config": cfg, "value": None, "unit": "solves/s",
                          "failed": str(e)[-1500:]}), flush=True)
        return
    except subprocess.TimeoutExpired:
        print(json.dumps({"impl": "refgpu", "config": cfg, "value": None, "unit": "solves/s",
                          "did_not_finish_s": args.refgpu_timeout,
                          "note": "the reference's first execute() (symbolic + numeric, 100 CG iterations) did not "
                                  "finish within the time limit; the harness was stopped"}), flush=True)
        return
    conv = None
    if args.refgpu_converged > 0:
        conv = summary(refgpu.run(systems, itmax=args.cg_itmax, calls=args.refgpu_converged,
                                  timeout=args.refgpu_timeout)[0])
        conv["itmax"] = args.cg_itmax
    line = {"metric": METRIC, "value": stock["value"], "unit": "solves/s", "impl": "refgpu", "n_gpus": 1,
            "steps": stock["solves"], "warmup": 1, "ms_per_step": 1e3 / stock["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "residual_target_met": False if stock["rel_residual_max"] > args.refine_target else True,
            "stock": stock, "converged_cg": conv,
            "note": "reference's rel. residual is its check_error definition (rows 1 and 3, "
                    "HykktSolver.cpp:846-930); timing = wall clock of execute()"}
    print(json.dumps(line), flush=True)


def _mixed_system(args):
    i, nb, seed = args
    from hykkt_gb300 import gridgen as gg
    return gg.make_system(gg.make_grid(int(nb), seed + i), 1000 + i, 1e4, (1e-8, 1e4), (1e-8, 1e8))


def run_mixed(args, rank, world):
    """Batched systems of different sparsity (the 256-system workload): per-
    system grids with bus counts log-uniform in [200, 20000] (the 500-bus
    generator's per-bus ratios and value ranges, gamma 1e4), one solve each
    to rel. residual <= 1e-8.  Plans are created on the host with their
    device storage deferred (symbolic analysis with the reference ordering,
    16 host threads).  Plain: one system at a time, its plan released after
    its solve.  Batched: every request submitted at once to the served queue
    with admission by device memory (`--batch` workers, plans of n_x >= 20000
    on the whole GPU, smaller ones at 1/batch of it).  Host wall clock;
    solves/s with and without plan creation."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor, ThreadPoolExecutor
    n = args.systems or 256
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(200), np.log(20000), n)).astype(int)
    # grids generated in spawned processes, before this process touches the GPU
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        systems = list(ex.map(_mixed_system, [(i, int(nb), 0) for i, nb in enumerate(sizes)], chunksize=4))
    import hykkt_gb300 as hk
    B = max(1, args.batch)

    # whole supernodes (`--solve-piece` splits the wide ones) and, batched,
    # plans of n_x >= 20000 on the whole GPU, smaller ones at 1/B of it
    # (`--mixed-share` gives every plan one share): measured on this mix,
    # pieces of 2,048 columns and share B for every plan ran 1.60 / 2.29
    # solves/s plain / batched against 1.75 / 2.66 for this policy
    piece = max(0, args.solve_piece)

    def share_of(i):
        if args.mixed_share > 0:
            return args.mixed_share
        return 1 if systems[i].n_x >= 20000 else B

    def make_plan(i):
        p = hk.Plan(systems[i], deferred=True, solve_piece=piece)
        p.set_accuracy(args.cg_itmax, args.cg_rtol, args.refine_max, args.refine_target)
        p.set_refine_rtol(args.refine_rtol)
        return p

    # warm-up: library, context, first graph
    w = make_plan(int(np.argmin(sizes)))
    w.solve(systems[int(np.argmin(sizes))])
    w.close()
    t = time.perf_counter()
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        plans = list(ex.map(make_plan, range(n)))
    t_plans = time.perf_counter() - t
    order = sorted(range(n), key=lambda i: -systems[i].n_x)
    # plain: one system at a time
    plain_lat, plain_res, plain_st, kept = [], [], [], {}
    flops = 0.0
    t = time.perf_counter()
    for p in plans:
        p.set_concurrency(1)  # one at a time: the whole GPU
    for i in order:
        t1 = time.perf_counter()
        st = plans[i].solve(systems[i])
        plain_lat.append(1e3 * (time.perf_counter() - t1))
        plain_st.append(st)
        inf = plans[i].info()
        plain_res.append(inf["rel_residual_full"])
        flops += inf["factor_flops"]
        if st != hk.OK:  # kept for the report below, outside the timed loop
            kept[i] = (plans[i].solution(), inf)
        plans[i].release_device()
    t_plain = time.perf_counter() - t
    from hykkt_gb300.stress_case import accuracy_report
    misses = []
    for i, (sol, inf) in kept.items():
        a = accuracy_report(systems[i], *sol)
        misses.append({"system": i, "n_bus": int(sizes[i]), "status": int(inf["status"]),
                       "rel_residual_full": inf["rel_residual_full"], "rel_residual_first": inf["rel_residual_first"],
                       "refine_steps": inf["refine_steps"], "fp64_storage_floor": a["fp64_storage_floor"],
                       "backward_error_inf": a["backward_error_inf"]})
    fp64 = hk.fp64_peak_tflops()
    # batched: the served queue, admission by device memory, every plan's
    # persistent kernels sized for the B workers
    for i, p in enumerate(plans):
        p.set_concurrency(share_of(i))
    srv = hk.Server(B, budget=0)
    t = time.perf_counter()
    tickets = [srv.submit(plans[i], systems[i]) for i in order]
    res, lat, sts = [], [], []
    for tk in tickets:
        st, ms, info, _ = srv.wait(tk)
        sts.append(st)
        lat.append(ms)
        res.append(info["rel_residual_full"])
    t_batched = time.perf_counter() - t
    mem = srv.memory_stats()
    srv.close()
    for p in plans:
        p.close()
    all_res = res + plain_res
    line = {"metric": "KKT solves/s, systems of different sparsity, batched vs plain", "value": n / t_batched,
            "unit": "solves/s", "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * t_batched,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded per-system grids, hykkt_gb300/gridgen.py)",
            "config": {"workload": f"mixed{n}_200_20k", "systems": n,
                       "n_bus_range": [int(sizes.min()), int(sizes.max())], "n_bus_median": int(np.median(sizes)),
                       "gamma": 1e4, "dx_range": [1e-8, 1e4], "ds_range": [1e-8, 1e8], "workers": B,
                       "solve_piece": piece, "share": {"n_x >= 20000": big_share, "smaller": W},
                       "heavy": {"plan_bytes_at_least": heavy_bytes, "max_workers": max_heavy} if heavy_bytes > 0
                       else None, "share_batched": args.mixed_share if args.mixed_share > 0 else
                       f"1 for n_x >= 20000, else {B}",
                       "accuracy": {"cg_itmax": args.cg_itmax, "cg_rtol": args.cg_rtol,
                                    "refine_max": args.refine_max, "refine_target": args.refine_target,
                                    "refine_rtol": args.refine_rtol},
                       "timing": "host wall clock; plans created with device storage deferred, 16 host threads"},
            "plan_creation_s": t_plans,
            "batched": {"solves_per_s": n / t_batched, "with_plan_creation": n / (t_plans + t_batched),
                        "seconds": t_batched, "p50_ms": float(np.percentile(lat, 50)),
                        "p99_ms": float(np.percentile(lat, 99)), "memory": mem},
            "plain": {"solves_per_s": n / t_plain, "with_plan_creation": n / (t_plans + t_plain), "seconds": t_plain,
                      "p50_ms": float(np.percentile(plain_lat, 50)), "p99_ms": float(np.percentile(plain_lat, 99))},
            "batched_over_plain": t_plain / t_batched,
            "factor_flops_total": flops,
            "fp64_bound_s": {"factorization_only": flops / (fp64 * 1e12), "fp64_tflops_measured": fp64,
                             "note": "sum over the systems of the column counts squared; the inversion and the "
                                     "CG solves add to it"},
            "plain_misses": misses,
            "rel_residual_full_max": float(max(all_res)), "solves_above_1e-8": int(sum(r > 1e-8 for r in all_res)),
            "statuses": sorted({int(x) for x in sts + plain_st}),
            "solves_accuracy_not_met": int(sum(x == hk.ACCURACY_NOT_MET for x in sts + plain_st))}
    if rank == 0:
        print(json.dumps(line), flush=True)


def _served_system(args):
    c, nb, k = args
    from hykkt_gb300 import gridgen as gg
    return gg.make_system(gg.make_grid(int(nb), 300 + c), 1000 * c + k, 1e5, (1e-10, 1e8), (1e-10, 1e8))


def run_served(args, rank, world):
    """Served solves (the 64-client workload): clients with fixed grids
    (`--served-clients` each at the `--served-sizes` bus counts; gamma 1e5,
    the 10k workload's value ranges) send solve requests with new values to
    one request queue (hykkt_server_*, `--batch` workers) with admission by
    device memory: every client's plan is created on the host with its
    device storage deferred, the server keeps at most 90% of the free device
    memory resident and evicts idle plans; requests of plans of at least
    `--served-heavy-gb` take at most a quarter of the workers, so the small
    clients' requests do not queue behind 70k-bus solves.  Poisson arrivals at 0.5x, 1x and
    2x the plain capacity (the rate that one-at-a-time solving of the same
    request mix sustains, from one timed solve per size) for
    `--served-seconds` each; per load the completed solves/s, p50/p99 latency
    from submission to completion (queueing, admission and reloads
    included), residuals and the memory accounting.  Values come from host
    memory, solutions return to host memory; host wall clock."""
    import multiprocessing as mp
    import threading
    from concurrent.futures import ProcessPoolExecutor, ThreadPoolExecutor
    size_list = [int(x) for x in args.served_sizes.split(",")]
    sizes = [nb for nb in size_list for _ in range(args.served_clients)]
    W = max(1, args.batch)
    dur = float(args.served_seconds)
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        flat = list(ex.map(_served_system, [(c, nb, k) for c, nb in enumerate(sizes) for k in range(2)]))
    seqs = [flat[2 * c:2 * c + 2] for c in range(len(sizes))]
    import hykkt_gb300 as hk

    piece = args.solve_piece if args.solve_piece >= 0 else 2048

    def make_plan(c):
        p = hk.Plan(seqs[c][0], deferred=True, solve_piece=piece)
        p.set_accuracy(args.cg_itmax, args.cg_rtol, args.refine_max, args.refine_target)
        p.set_refine_rtol(args.refine_rtol)
        return p

    t = time.perf_counter()
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        plans = list(ex.map(make_plan, range(len(sizes))))
    t_plans = time.perf_counter() - t
    bytes_by_size = {nb: plans[sizes.index(nb)].residency()[1] for nb in size_list}
    # plain capacity: one client of each size, a warm-up solve then a timed one, released after
    t_size = {}
    for nb in size_list:
        c = sizes.index(nb)
        p = plans[c]
        p.set_concurrency(1)
        p.solve(seqs[c][0])
        t1 = time.perf_counter()
        p.solve(seqs[c][1])
        p.solution()
        t_size[nb] = time.perf_counter() - t1
        p.release_device()
    cap = 1.0 / float(np.mean([t_size[nb] for nb in sizes]))
    # large plans' solve kernels on the whole GPU (half of it measured slower
    # for every size: 70k-bus p50 41 -> 62 s at 1x load, and no gain for the
    # small clients at 2x)
    big_share = 1
    for c, p in enumerate(plans):
        p.set_concurrency(big_share if seqs[c][0].n_x >= 20000 else W)
    rng = np.random.default_rng(0)
    runs = []
    heavy_bytes = int(args.served_heavy_gb * 1e9)
    max_heavy = max(1, W // 4)
    for f in (0.5, 1.0, 2.0):
        srv = hk.Server(W, budget=0)
        if heavy_bytes > 0:
            srv.set_heavy(heavy_bytes, max_heavy)
        lam = f * cap
        n_req = max(4, int(lam * dur))
        gaps = rng.exponential(1.0 / lam, n_req)
        who = rng.integers(0, len(plans), n_req)
        tickets, lock = [], threading.Lock()
        t0 = time.perf_counter()

        def dispatch():
            at = t0
            for gap, c in zip(gaps, who):
                at += gap
                d = at - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                k = len(tickets) % 2
                tk = srv.submit(plans[c], seqs[c][k])
                with lock:
                    tickets.append((tk, c, k))

        th = threading.Thread(target=dispatch)
        th.start()
        th.join()
        lat, res, sts, by, odd, phases = [], [], [], {}, [], {}
        for tk, c, k in tickets:
            st, ms, info, _ = srv.wait(tk)
            lat.append(ms)
            res.append(info["rel_residual_full"])
            sts.append(st)
            by.setdefault(sizes[c], []).append(ms)
            phases.setdefault(sizes[c], []).append((info["queue_ms"], info["admission_ms"], info["solve_ms"]))
            if st != hk.OK:
                odd.append({"client": int(c), "n_bus": int(sizes[c]), "system": int(k), "status": int(st),
                            "rel_residual_full": float(info["rel_residual_full"])})
        span = time.perf_counter() - t0
        mem = srv.memory_stats()
        srv.close()
        for p in plans:  # the next level's server starts with the device memory free
            p.release_device()
        runs.append({"load": f, "offered_per_s": lam, "requests": n_req, "completed_per_s": n_req / span,
                     "span_s": span, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "p50_ms_by_size": {str(k): float(np.percentile(v, 50)) for k, v in sorted(by.items())},
                     "p50_queue_admission_solve_ms_by_size": {
                         str(k): [float(x) for x in np.percentile(np.array(v), 50, axis=0)]
                         for k, v in sorted(phases.items())},
                     "rel_residual_full_max": float(max(res)), "solves_above_1e-8": int(sum(r > 1e-8 for r in res)),
                     "statuses": sorted({int(x) for x in sts}),
                     "solves_accuracy_not_met": int(sum(x == hk.ACCURACY_NOT_MET for x in sts)), "memory": mem,
                     "not_ok": odd})
    # every request that did not return OK, solved again alone on the whole
    # GPU: the same status shows it is the system's, not the concurrency's
    seen = {}
    for r in runs:
        for o in r["not_ok"]:
            key = (o["client"], o["system"])
            if key not in seen:
                p = plans[o["client"]]
                p.set_concurrency(1)
                st = p.solve(seqs[o["client"]][o["system"]])
                seen[key] = {"status": int(st), "rel_residual_full": p.info()["rel_residual_full"]}
                p.release_device()
            o["alone"] = seen[key]
    one = [r for r in runs if r["load"] == 1.0][0]
    line = {"metric": "served KKT solves: throughput and p50/p99 latency under Poisson arrivals",
            "value": one["completed_per_s"], "unit": "solves/s", "n_gpus": world, "steps": len(runs), "warmup": 1,
            "ms_per_step": 1e3 * dur, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded per-client grids, hykkt_gb300/gridgen.py)",
            "config": {"workload": f"served{len(sizes)}", "clients": len(sizes), "n_bus": size_list,
                       "clients_per_size": args.served_clients, "workers": W, "seconds_per_load": dur,
                       "solve_piece": piece, "share": {"n_x >= 20000": big_share, "smaller": W},
                       "heavy": {"plan_bytes_at_least": heavy_bytes, "max_workers": max_heavy} if heavy_bytes > 0
                       else None,
                       "gamma": 1e5, "dx_range": [1e-10, 1e8], "ds_range": [1e-10, 1e8],
                       "timing": "host wall clock; plans created with device storage deferred; admission by "
                                 "device memory (90% of free memory at server creation)"},
            "plan_creation_s": t_plans, "plan_device_bytes_by_size": {str(k): v for k, v in bytes_by_size.items()},
            "plain_solve_s_by_size": {str(k): v for k, v in t_size.items()},
            "plain_capacity_per_s": cap, "loads": runs}
    if rank == 0:
        print(json.dumps(line), flush=True)
    for p in plans:
        p.close()


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.impl == "refgpu":
        run_refgpu(args, rank, world)
        return
    if args.workload.startswith("mixed"):
        run_mixed(args, rank, world)
        return
    if args.workload.startswith("served"):
        run_served(args, rank, world)
        return
    import torch

    import hykkt_gb300 as hk
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    systems, cfg = workload(args)
    B = max(1, args.batch)
    cfg["parallelism"] = f"replicas{world}"
    cfg["batch"] = B
    share_b = B if args.share < 0 else args.share
    t0 = time.perf_counter()
    plan = hk.Plan(systems[0], solve_piece=max(0, args.solve_piece))
    plan_s = time.perf_counter() - t0
    plan.set_accuracy(args.cg_itmax, args.cg_rtol, args.refine_max, args.refine_target)
    plan.set_refine_rtol(args.refine_rtol)
    # each mode with the solve layout that suits it, picked by the autotuner
    # (measured: concurrent plans gain from pieces of the widest supernodes,
    # one plan alone from whole supernodes) unless given
    tune = {}
    if args.solve_piece < 0:
        t0 = time.perf_counter()
        tune["batched"] = plan.autotune(systems[0], share=share_b, cache=args.tune_cache)
        tune["batched"]["seconds"] = time.perf_counter() - t0
    plans = [plan] + [plan.clone() for _ in range(B - 1)]
    cfg["accuracy"] = {"cg_itmax": args.cg_itmax, "cg_rtol": args.cg_rtol, "refine_max": args.refine_max,
                       "refine_target": args.refine_target, "refine_rtol": args.refine_rtol}
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")
    from hykkt_gb300 import gridgen as gg
    dsys = []
    for s in systems:
        d = gg.KKTSystem(*[None] * 8, s.gamma)
        d.H, d.Ds, d.Jc, d.Jd = (gg.CSR(0, 0, None, None, dev(A.vals)) for A in (s.H, s.Ds, s.Jc, s.Jd))
        d.rx, d.rs, d.ry, d.ryd = (dev(v) for v in (s.rx, s.rs, s.ry, s.ryd))
        dsys.append(d)
    streams = [torch.cuda.Stream() for _ in range(B)]
    main_st = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device="cuda")  # 256 MB > L2 (129 MB)
    torch.cuda.synchronize()

    def timed_steps(ps, nsteps, on_device):
        """nsteps * len(ps) solves by the plans of ps, concurrently (one host
        thread and one stream per plan; a thread takes the next system of the
        sequence, solves it, waits, reads the status and residual (and the
        solution, from host inputs), then takes the next).  One 256 MB L2
        flush before the timed region; each solve then rewrites its plan's
        factor storage (about 2 GB, > L2), so no solve finds the previous
        one's data in L2.  Returns the device time of the region (CUDA
        events), per-solve ms, statuses and per-solve info."""
        nb = len(ps)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        last = [torch.cuda.Event() for _ in range(nb)]
        out = [[] for _ in range(nb)]
        with torch.cuda.stream(main_st):
            flush.zero_()
            ev0.record(main_st)
        for i in range(nb):
            streams[i].wait_event(ev0)

        lock = threading.Lock()
        nxt = [0]

        def worker(i):
            # plans pull the next system from one shared queue, so that a
            # plan that drew faster systems does not leave the GPU idle at
            # the end of the region
            p, st = ps[i], streams[i]
            while True:
                with lock:
                    j = nxt[0]
                    nxt[0] += 1
                if j >= nsteps * nb:
                    break
                j %= len(systems)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                if on_device:
                    p.solve(dsys[j], on_device=True, stream=st.cuda_stream, sync=False)
                else:
                    p.solve(systems[j], on_device=False, stream=st.cuda_stream, sync=False)
                b.record(st)
                status = p.wait(st.cuda_stream)
                if not on_device:
                    p.solution()
                out[i].append((a, b, status, p.info()))
            last[i].record(st)

        threads = [threading.Thread(target=worker, args=(i,)) for i in range(nb)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for i in range(nb):
            main_st.wait_event(last[i])
        with torch.cuda.stream(main_st):
            ev1.record(main_st)
        torch.cuda.synchronize()
        solve_ms = [a.elapsed_time(b) for o in out for a, b, _, _ in o]
        infos = [inf for o in out for *_, inf in o]
        return ev0.elapsed_time(ev1), solve_ms, [st for o in out for _, _, st, _ in o], infos

    # warm-up (first call of each plan also builds its CUDA graph)
    plan.set_concurrency(1)
    timed_steps([plan], max(3, args.warmup), True)
    for p in plans:
        p.set_concurrency(share_b)
    timed_steps(plans, max(3, args.warmup), True)
    # ---- batched: B plans, B solves in flight per step ---------------------------
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        tot_ms, solve_ms, statuses, infos = timed_steps(plans, args.steps, True)
    res_full = [inf["rel_residual_full"] for inf in infos]
    its_total = [inf["cg_iterations_total"] for inf in infos]
    barrier(world)
    tot_ms = max_over_ranks(tot_ms, world)
    value = world * B * args.steps / (tot_ms / 1e3)
    info = plan.info()
    # ---- end-to-end through the C ABI from host buffers (batched) --------------
    h2d = sum(a.nbytes for a in (systems[0].H.vals, systems[0].Ds.vals, systems[0].Jc.vals, systems[0].Jd.vals,
                                 systems[0].rx, systems[0].rs, systems[0].ry, systems[0].ryd))
    d2h = 8 * (systems[0].n_x + 2 * systems[0].m_d + systems[0].m_c)
    e2e_tot, e2e_solve, e2e_st, e2e_infos = timed_steps(plans, args.steps, False)
    e2e_res = [inf["rel_residual_full"] for inf in e2e_infos]
    e2e_value = world * B * args.steps / (max_over_ranks(e2e_tot, world) / 1e3)
    # ---- plain: one plan, one solve at a time ------------------------------------
    if args.plain_piece == args.solve_piece and args.plain_piece >= 0:
        plain_plan = plan
    else:
        plain_plan = hk.Plan(systems[0], solve_piece=max(0, args.plain_piece))
        plain_plan.set_accuracy(args.cg_itmax, args.cg_rtol, args.refine_max, args.refine_target)
        plain_plan.set_refine_rtol(args.refine_rtol)
        if args.plain_piece < 0:
            t0 = time.perf_counter()
            tune["plain"] = plain_plan.autotune(systems[0], share=1, cache=args.tune_cache)
            tune["plain"]["seconds"] = time.perf_counter() - t0
    plain_plan.set_concurrency(1)
    cfg["solve_layout"] = {k: {"solve_piece": v["solve_piece"], "warp_subtree": v["warp_subtree"],
                               "chunk_fma": v["chunk_fma"]} for k, v in tune.items()} or \
        {"batched": {"solve_piece": args.solve_piece}, "plain": {"solve_piece": args.plain_piece}}
    timed_steps([plain_plan], max(1, args.warmup), True)  # (re)builds the plan's graph for the full grid
    barrier(world)
    plain_tot, plain_solve, plain_st, plain_infos = timed_steps([plain_plan], args.steps, True)
    plain_res = [inf["rel_residual_full"] for inf in plain_infos]
    plain_value = world * args.steps / (max_over_ranks(plain_tot, world) / 1e3)
    # ---- dominant kernel and roofline ------------------------------------------
    roof = None
    prof = {}
    prof_p = {}
    if not args.no_profile and rank == 0:
        # the batched plans' kernels (FP64 work per solve, aggregate bandwidth
        # under concurrency below), profiled on the whole GPU
        plan.set_concurrency(1)
        plan.solve(dsys[0], on_device=True, stream=streams[0].cuda_stream)
        prof = plan.profile(upto=3)
        # the dominant kernel's roofline: the plain plan, whose layout is the
        # one tuned for a launch that has the GPU to itself
        plain_plan.solve(dsys[0], on_device=True, stream=streams[0].cuda_stream)
        prof_p = plain_plan.profile(upto=3)
        name, (launches, ms, flops, nbytes) = max(prof_p.items(), key=lambda kv: kv[1][1])
        fp64 = hk.fp64_peak_tflops()
        # DRAM bytes per launch of the dominant kernel from the committed ncu
        # capture of the same workload (profiles/), when it covers this case
        traffic = None
        piece = tune["plain"]["solve_piece"] if "plain" in tune else max(0, args.plain_piece)
        tname = "dram_traffic_grid10k.json" if piece == 0 else f"dram_traffic_grid10k_piece{piece}.json"
        tpath = os.path.join(ROOT, "profiles", tname)
        if os.path.exists(tpath) and cfg["n_bus"] == 10000:
            tk = json.load(open(tpath))["kernels"].get(name)
            traffic = tk["dram_bytes_per_launch"] if tk else None
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
            os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
        hbm = peaks.get("hbm_gbs", 6800.0)
        if flops > 0 and flops / max(nbytes, 1) > 0.3:
            ach = flops / (ms / 1e3) / 1e12
            roof = {"bound": "fp64", "kernel": name, "achieved": ach, "peak": fp64, "unit": "TFLOP/s",
                    "frac": ach / fp64, "traffic": traffic, "launches": launches, "avg_launch_ms": ms / launches,
                    "peak_source": "FP64 DFMA loop measured in this run (hykkt_fp64_peak); MEASURED_PEAKS.json has no FP64 figure",
                    "achieved_gbs": nbytes / (ms / 1e3) / 1e9, "hbm_peak_gbs": hbm}
        else:
            ach = nbytes / (ms / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": hbm, "unit": "GB/s",
                    "frac": ach / hbm, "traffic": traffic, "algorithmic_bytes_per_launch": nbytes / launches,
                    "launches": launches, "avg_launch_ms": ms / launches, "plan": "plain (alone on the GPU)",
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s"}
    # whole-solve FP64 roofline of the batched run: algorithmic FP64 work of
    # one solve (factorization and inversion kernels as profiled, plus one
    # forward + backward triangular solve per CG iteration and four more per
    # CG run) times batched solves/s, against the measured DFMA peak
    roof_solve = None
    if prof and "k_trsv_fwd" in prof:
        f_fact = sum(v[2] for k, v in prof.items() if k.startswith(("k_front", "k_panel", "k_trtri", "k_piece")))
        f_pair = prof["k_trsv_fwd"][2] / prof["k_trsv_fwd"][0] + prof["k_trsv_bwd"][2] / prof["k_trsv_bwd"][0]
        ref_steps = float(np.mean([inf["refine_steps"] for inf in infos]))
        pairs = float(np.mean(its_total)) + 4.0 * (1.0 + ref_steps)
        f_solve = f_fact + pairs * f_pair
        ach_t = f_solve * value / 1e12
        # the triangular solves' algorithmic bytes per second over all
        # concurrent plans (every stored entry of L read once per direction)
        b_pair = prof["k_trsv_fwd"][3] / prof["k_trsv_fwd"][0] + prof["k_trsv_bwd"][3] / prof["k_trsv_bwd"][0]
        agg = pairs * b_pair * value / 1e9
        roof_solve = {"bound": "fp64", "achieved": ach_t, "peak": fp64, "unit": "TFLOP/s", "frac": ach_t / fp64,
                      "fp64_gflop_per_solve": f_solve / 1e9, "factor_gflop": f_fact / 1e9,
                      "solve_pairs_per_solve": pairs, "note": "batched value x algorithmic FP64 work per solve",
                      "trisolve_gbs_all_plans": agg,
                      "trisolve_hbm_frac": agg / (roof["peak"] if roof and roof["unit"] == "GB/s" else 6800.0)}
    kernels_per_solve = (info["kernels_per_solve"] + info["kernels_per_cg_iteration"] * info["cg_iterations_total"]
                         + info["kernels_per_refine_step"] * info["refine_steps"])
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(systems, args)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded grid generator, hykkt_gb300/gridgen.py)",
            "config": dict(cfg, l2="256 MB flush before the timed region; every solve rewrites ~2 GB of its plan's "
                              "factor storage (> L2) before reading it", plan_build_s=plan_s,
                           step=f"{B} solves, one per plan, the plans concurrent (batched); plain: 1 solve"),
            "p50_ms": float(np.percentile(solve_ms, 50)), "p99_ms": float(np.percentile(solve_ms, 99)),
            "plain": {"value": plain_value, "unit": "solves/s", "p50_ms": float(np.percentile(plain_solve, 50)),
                      "p99_ms": float(np.percentile(plain_solve, 99)),
                      "rel_residual_full_max": float(np.max(plain_res))},
            "rel_residual_full_max": float(np.max(res_full + e2e_res)),
            "residual_target_met": bool(np.max(res_full + e2e_res + plain_res) <= 1e-8),
            "solves_above_1e-8": int(sum(r > 1e-8 for r in res_full + e2e_res + plain_res)),
            "solves_checked": len(res_full + e2e_res + plain_res),
            "cg_iterations_total_mean": float(np.mean(its_total)),
            "cg_iterations": info["cg_iterations"], "cg_iterations_total": info["cg_iterations_total"],
            "refine_steps": info["refine_steps"], "rel_residual_before_refinement": info["rel_residual_first"],
            "statuses": sorted(set(statuses + e2e_st + plain_st)),
            "solves_accuracy_not_met": int(sum(x == hk.ACCURACY_NOT_MET for x in statuses + e2e_st + plain_st)),
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d) * B,
                    "d2h_bytes_per_step": int(d2h) * B, "p50_ms": float(np.percentile(e2e_solve, 50)),
                    "p99_ms": float(np.percentile(e2e_solve, 99))},
            "gpu_launches": int(kernels_per_solve * B * args.steps),
            "roofline": roof, "roofline_solve": roof_solve, "cpu_baseline": cpu, "clocks": clk.summary(),
            "plan": {k: info[k] for k in ("nnz_L", "L_stored", "factor_flops", "device_bytes", "n_supernodes",
                                          "n_levels", "n_solve_levels", "ordering")},
            "kernel_ms": {k: round(v[1], 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:8]},
            "autotune": tune,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
