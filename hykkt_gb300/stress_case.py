"""Large-grid stress run: one KKT system of a big synthetic grid.

    python -m hykkt_gb300.stress_case --n-bus 40000 [--gamma 1e6]

The shape of the stress workload (80,000 buses, D_x and D_s log-uniform in
[1e-10, 1e10], gamma 1e6) at a chosen bus count.  Reports, as one JSON line:
plan creation time and device memory, one accuracy-mode solve through the
graph (CG iterations, refinement steps, 4-block relative residual, wall
time), and per stage of one uncaptured solve (per-kernel CUDA events) the
device time, algorithmic bytes and GB/s, and for the factorization its FP64
rate, and a host check of the solution's accuracy (backward error and the
residual floor of FP64 storage, accuracy_report):
  * formation (H~ = H + Jd^T Ds Jd, Ruiz, Hgamma = H~ + gamma Jc^T Jc: the
    SpGEMM-shaped steps): values and lists read once, outputs written once;
  * factorization (multifrontal Cholesky and the inversion of the solve
    items' diagonal blocks): bytes = the stored factor written once (8 bytes
    per stored entry of L, the lower bound), flops = the modelled
    factorization and inversion work;
  * triangular solves (one forward + backward pair per CG iteration): every
    stored entry of L read once per direction.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import Plan
from . import gridgen as gg


def accuracy_report(s, x, ds, y, yd) -> dict:
    """Host check of a solution of the 4-block KKT system K z = b (scipy):
    the relative residual ||b - K z|| / ||b|| with products and sums in
    extended precision; the normwise backward error
    ||b - K z||_inf / (||K||_inf ||z||_inf + ||b||_inf), which is a few units
    of FP64 rounding for a backward-stable solve; and the residual floor that
    storing z in FP64 alone leaves: rounding each z_j to the nearest double
    moves row i of K z by about eps * sqrt(sum_j (K_ij z_j)^2) (independent
    roundings, eps = 2^-53), relative to ||b||.  When that floor is above a
    residual target, no FP64 solution vector meets the target."""
    import scipy.sparse as sp

    def csr(A, n, m):
        return sp.csr_matrix((A.vals, A.colidx, A.rowptr), shape=(n, m))
    H = csr(s.H, s.n_x, s.n_x)
    Jc = csr(s.Jc, s.m_c, s.n_x)
    Jd = csr(s.Jd, s.m_d, s.n_x)
    Ds = sp.diags(s.Ds.vals)
    I = sp.eye(s.m_d)
    K = sp.bmat([[H, None, Jc.T, Jd.T], [None, Ds, None, -I], [Jc, None, None, None], [Jd, -I, None, None]]).tocsr()
    z = np.concatenate([x, ds, y, yd])
    b = np.concatenate([s.rx, s.rs, s.ry, s.ryd])
    rows = np.repeat(np.arange(K.shape[0]), np.diff(K.indptr))
    kz = np.zeros(K.shape[0], dtype=np.longdouble)
    np.add.at(kz, rows, K.data.astype(np.longdouble) * z[K.indices].astype(np.longdouble))
    r = (b.astype(np.longdouble) - kz).astype(np.float64)
    knorm = float(abs(K).sum(axis=1).max())
    eta = float(np.abs(r).max() / (knorm * np.abs(z).max() + np.abs(b).max()))
    sq = np.zeros(K.shape[0])
    np.add.at(sq, rows, (K.data * z[K.indices]) ** 2)
    eps = 2.0 ** -53
    return {"rel_residual_host": float(np.linalg.norm(r) / np.linalg.norm(b)), "backward_error_inf": eta,
            "K_norm_inf": knorm, "z_norm_inf": float(np.abs(z).max()),
            "fp64_storage_floor": float(eps * np.linalg.norm(np.sqrt(sq)) / np.linalg.norm(b))}

STAGES = {
    "formation": ("k_prepare", "k_ruiz_rowmax", "k_ruiz_scale", "k_hgamma"),
    "factorization": ("k_front_small", "k_front_scatter", "k_front_extadd", "k_panel_potrf", "k_panel_trsm",
                      "k_panel_update", "k_piece_inverse", "k_trtri_init", "k_trtri_diag", "k_trtri_update",
                      "k_xpanel_pack"),
    "triangular_solves": ("k_trsv_fwd", "k_trsv_bwd"),
}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-bus", type=int, default=40000)
    ap.add_argument("--gamma", type=float, default=1e6)
    ap.add_argument("--cg-itmax", type=int, default=20000)
    ap.add_argument("--cg-rtol", type=float, default=1e-11)
    ap.add_argument("--refine-max", type=int, default=4)
    ap.add_argument("--profile-cg-its", type=int, default=20, help="CG iterations of the profiled (uncaptured) solve")
    ap.add_argument("--solve-piece", type=int, default=4096,
                    help="most columns of one triangular-solve item (0: whole supernodes; the widest supernode of "
                         "the 80k grid has ~45,000 columns, whose whole inversion costs about as much as the "
                         "factorization)")
    a = ap.parse_args()
    out = {"workload": f"stress_grid{a.n_bus // 1000}k", "n_bus": a.n_bus, "gamma": a.gamma,
           "dx_range": [1e-10, 1e10], "ds_range": [1e-10, 1e10]}
    t = time.perf_counter()
    s = gg.make_system(gg.make_grid(a.n_bus, 0), 1, a.gamma, (1e-10, 1e10), (1e-10, 1e10))
    out.update(n_x=s.n_x, m_c=s.m_c, m_d=s.m_d, generate_s=time.perf_counter() - t)
    t = time.perf_counter()
    plan = Plan(s, solve_piece=a.solve_piece)
    out["plan_s"] = time.perf_counter() - t
    out["solve_piece"] = a.solve_piece
    sz = plan.sizes()
    out.update(nnz_L=sz["nnz_L"], front_arena_doubles=sz["front_arena"], n_supernodes=sz["n_supernodes"])
    sq_c0, sq_c1 = plan.symbolic("sq_c0"), plan.symbolic("sq_c1")
    out["widest_solve_item"] = int((sq_c1 - sq_c0).max())
    out["widest_supernode"] = int(np.diff(plan.symbolic("sn_first")).max())
    # accuracy-mode solve through the graph
    plan.set_accuracy(a.cg_itmax, a.cg_rtol, a.refine_max, 1e-8)
    plan.set_refine_rtol(1e-4)
    t = time.perf_counter()
    st = plan.solve(s)
    out["solve_s"] = time.perf_counter() - t
    info = plan.info()
    out.update(status=st, cg_iterations_total=info["cg_iterations_total"], refine_steps=info["refine_steps"],
               rel_residual_full=info["rel_residual_full"], rel_residual_reference=info["rel_residual"],
               device_bytes=info["device_bytes"], L_stored=info["L_stored"], factor_flops=info["factor_flops"])
    t = time.perf_counter()
    out["accuracy"] = accuracy_report(s, *plan.solution())
    out["accuracy"]["host_check_s"] = time.perf_counter() - t
    # per-stage rates from one uncaptured solve with a bounded CG
    plan.set_accuracy(a.profile_cg_its, a.cg_rtol, 0, 1e-8)
    prof = plan.profile(3)
    stages = {}
    for name, kernels in STAGES.items():
        ms = sum(prof[k][1] for k in kernels if k in prof)
        fl = sum(prof[k][2] for k in kernels if k in prof)
        by = sum(prof[k][3] for k in kernels if k in prof)
        launches = sum(prof[k][0] for k in kernels if k in prof)
        stages[name] = {"launches": int(launches), "ms": ms, "algorithmic_bytes": by, "flops": fl}
    f = stages["factorization"]
    f["algorithmic_bytes"] = 8.0 * float(info["L_stored"])
    for v in stages.values():
        v["GB_s"] = v["algorithmic_bytes"] / (v["ms"] * 1e6) if v["ms"] > 0 else None
        v["TFLOP_s"] = v["flops"] / (v["ms"] * 1e9) if v["ms"] > 0 and v["flops"] > 0 else None
    tri = stages["triangular_solves"]
    tri["pair_ms"] = tri["ms"] / max(1, tri["launches"] // 2)
    out["stages"] = stages
    out["profile"] = {"cg_iterations": a.profile_cg_its, "kernels": {k: list(v) for k, v in prof.items()}}
    print(json.dumps(out), flush=True)
    plan.close()


if __name__ == "__main__":
    main()
