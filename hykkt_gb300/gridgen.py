"""Seeded synthetic power-grid KKT systems (the optimal-power-flow shape HyKKT solves).

The reference ships ACTIVSg200/2000 KKT blocks as Matrix-Market fixtures
(src/mats/a200, src/mats/a2000) and its `hybrid_driver` reads them
(examples/cuSolver_driver_hybrid.cpp:26-96).  The synthetic grids here have the
same block layout and the shapes of the benchmark workloads:

* buses ``N_b``; generators ``G = 0.2 N_b`` at uniform random buses;
  branches ``1.4 N_b`` = a random recursive spanning tree plus random chords
  (no parallel branches);
* variables ``x = [Vm_0, Va_0, ..., Vm_{N_b-1}, Va_{N_b-1}, Pg_0, Qg_0, ...]``
  so ``n_x = 2 N_b + 2 G``;
* ``H`` = branch-weighted bus Laplacian (weights U(0.1, 10)) expanded to the
  (Vm, Va) pair with a per-branch 2x2 coupling block ``[[1, rho], [rho, 1]]``
  (rho U(-0.9, 0.9)), plus a generator diagonal U(0.1, 10), plus ``D_x``
  log-uniform on the whole diagonal (the H block holds H + D_x, as in the
  reference's block_H files);
* ``J_c``: two power-balance rows per bus (P, Q) touching Vm/Va of the bus and
  its neighbours and Pg (P row) or Qg (Q row) of the generators at that bus,
  values N(0, 1);
* ``J_d``: two flow-limit rows per branch (from and to side), four nonzeros at
  the endpoints' Vm/Va, values N(0, 1);
* ``D_s`` diagonal log-uniform; right-hand sides U(-1, 1).

All matrices are returned as 0-based int32/float64 CSR with sorted columns,
``H`` as its full symmetric pattern (the form `HykktSolver::set_H` takes,
src/HykktSolver.cpp:163-168).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np


@dataclasses.dataclass
class CSR:
    n: int
    m: int
    rowptr: np.ndarray  # int32, n+1
    colidx: np.ndarray  # int32, nnz
    vals: np.ndarray  # float64, nnz

    @property
    def nnz(self) -> int:
        return int(self.colidx.shape[0])

    def copy(self) -> "CSR":
        return CSR(self.n, self.m, self.rowptr.copy(), self.colidx.copy(), self.vals.copy())


@dataclasses.dataclass
class KKTSystem:
    H: CSR
    Ds: CSR
    Jc: CSR
    Jd: CSR
    rx: np.ndarray
    rs: np.ndarray
    ry: np.ndarray
    ryd: np.ndarray
    gamma: float

    @property
    def n_x(self) -> int:
        return self.H.n

    @property
    def m_c(self) -> int:
        return self.Jc.n

    @property
    def m_d(self) -> int:
        return self.Jd.n


def coo_to_csr(n: int, m: int, rows, cols, vals) -> CSR:
    """Sorted-column CSR from COO without duplicates (the order `coo_to_csr`
    produces, reference src/input_functions.cpp:121-175)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr)
    return CSR(n, m, rowptr.astype(np.int32), cols.astype(np.int32), vals.copy())


def _log_uniform(rng, lo, hi, size):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size))


@dataclasses.dataclass
class Grid:
    """Structure and the values that stay fixed across interior-point iterations."""
    n_bus: int
    n_gen: int
    branches: np.ndarray  # (n_br, 2) int64
    gen_bus: np.ndarray  # (n_gen,)
    br_w: np.ndarray
    br_rho: np.ndarray
    gen_w: np.ndarray
    Jc: CSR
    Jd: CSR
    Hbase_rows: np.ndarray
    Hbase_cols: np.ndarray
    Hbase_vals: np.ndarray

    @property
    def n_x(self) -> int:
        return 2 * self.n_bus + 2 * self.n_gen


def make_grid(n_bus: int, seed: int, gen_ratio: float = 0.2, branch_ratio: float = 1.4) -> Grid:
    rng = np.random.default_rng(seed)
    n_gen = int(round(gen_ratio * n_bus))
    n_br = int(round(branch_ratio * n_bus))
    # random recursive spanning tree
    parents = np.array([rng.integers(0, b) for b in range(1, n_bus)], dtype=np.int64) if n_bus > 1 else np.zeros(0, np.int64)
    tree = np.stack([np.arange(1, n_bus, dtype=np.int64), parents], axis=1)
    edges = set((int(min(a, b)), int(max(a, b))) for a, b in tree)
    br = [tuple(e) for e in tree.tolist()]
    n_chords = n_br - len(br)
    while n_chords > 0:
        a, b = rng.integers(0, n_bus, 2)
        a, b = int(min(a, b)), int(max(a, b))
        if a == b or (a, b) in edges:
            continue
        edges.add((a, b))
        br.append((a, b))
        n_chords -= 1
    branches = np.array(br, dtype=np.int64).reshape(-1, 2)
    gen_bus = rng.integers(0, n_bus, n_gen).astype(np.int64)
    br_w = rng.uniform(0.1, 10.0, branches.shape[0])
    br_rho = rng.uniform(-0.9, 0.9, branches.shape[0])
    gen_w = rng.uniform(0.1, 10.0, 2 * n_gen)
    n_x = 2 * n_bus + 2 * n_gen

    # H base: Laplacian (x) 2x2 coupling, plus generator diagonal (full symmetric COO)
    rows, cols, vals = [], [], []
    a, b = branches[:, 0], branches[:, 1]
    for (p, q, s) in ((0, 0, 1.0), (1, 1, 1.0), (0, 1, None), (1, 0, None)):
        coup = br_w * (1.0 if s is not None else br_rho)
        # diagonal blocks (a,a), (b,b): +w*B ; off-diagonal (a,b), (b,a): -w*B
        rows += [2 * a + p, 2 * b + p, 2 * a + p, 2 * b + p]
        cols += [2 * a + q, 2 * b + q, 2 * b + q, 2 * a + q]
        vals += [coup, coup, -coup, -coup]
    rows.append(2 * n_bus + np.arange(2 * n_gen))
    cols.append(2 * n_bus + np.arange(2 * n_gen))
    vals.append(gen_w)
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.concatenate(vals)
    # sum duplicates (bus diagonal blocks receive one term per incident branch)
    key = rows * n_x + cols
    uk, inv = np.unique(key, return_inverse=True)
    sv = np.zeros(uk.shape[0])
    np.add.at(sv, inv, vals)
    Hr, Hc = uk // n_x, uk % n_x
    # make sure every diagonal exists (D_x goes there)
    diag = np.arange(n_x)
    have = np.zeros(n_x, dtype=bool)
    have[Hr[Hr == Hc]] = True
    Hr = np.concatenate([Hr, diag[~have]])
    Hc = np.concatenate([Hc, diag[~have]])
    sv = np.concatenate([sv, np.zeros((~have).sum())])

    # J_c: P and Q balance rows per bus
    nbrs = [[i] for i in range(n_bus)]
    for (p, q) in branches.tolist():
        nbrs[p].append(q)
        nbrs[q].append(p)
    gens_at = [[] for _ in range(n_bus)]
    for g, bb in enumerate(gen_bus.tolist()):
        gens_at[bb].append(g)
    jr, jcol = [], []
    for bb in range(n_bus):
        vcols = []
        for nb in nbrs[bb]:
            vcols += [2 * nb, 2 * nb + 1]
        for pq in (0, 1):
            cc = vcols + [2 * n_bus + 2 * g + pq for g in gens_at[bb]]
            jr += [2 * bb + pq] * len(cc)
            jcol += cc
    Jc = coo_to_csr(2 * n_bus, n_x, jr, jcol, rng.standard_normal(len(jr)))

    # J_d: two flow-limit rows per branch
    dr, dc = [], []
    for e, (p, q) in enumerate(branches.tolist()):
        cc = [2 * p, 2 * p + 1, 2 * q, 2 * q + 1]
        for side in (0, 1):
            dr += [2 * e + side] * 4
            dc += cc
    Jd = coo_to_csr(2 * branches.shape[0], n_x, dr, dc, rng.standard_normal(len(dr)))
    return Grid(n_bus, n_gen, branches, gen_bus, br_w, br_rho, gen_w, Jc, Jd, Hr, Hc, sv)


def make_system(grid: Grid, seed: int, gamma: float, dx_range=(1e-8, 1e4), ds_range=(1e-8, 1e8)) -> KKTSystem:
    """Draw one interior-point iterate on a fixed grid: new D_x, D_s and RHS."""
    rng = np.random.default_rng(seed)
    n_x = grid.n_x
    dx = _log_uniform(rng, dx_range[0], dx_range[1], n_x)
    vals = grid.Hbase_vals.copy()
    on_diag = grid.Hbase_rows == grid.Hbase_cols
    vals[on_diag] += dx[grid.Hbase_rows[on_diag]]
    H = coo_to_csr(n_x, n_x, grid.Hbase_rows, grid.Hbase_cols, vals)
    m_d = grid.Jd.n
    ds = _log_uniform(rng, ds_range[0], ds_range[1], m_d)
    Ds = CSR(m_d, m_d, np.arange(m_d + 1, dtype=np.int32), np.arange(m_d, dtype=np.int32), ds)
    rx = rng.uniform(-1, 1, n_x)
    rs = rng.uniform(-1, 1, m_d)
    ry = rng.uniform(-1, 1, grid.Jc.n)
    ryd = rng.uniform(-1, 1, m_d)
    return KKTSystem(H, Ds, grid.Jc.copy(), grid.Jd.copy(), rx, rs, ry, ryd, float(gamma))


# The benchmark workloads (seeded; per-system seed = base seed + index).
WORKLOADS = {
    # single plain solve, 500 buses
    "grid500": dict(n_bus=500, gamma=1e4, dx=(1e-8, 1e4), ds=(1e-8, 1e8), systems=1),
    # 20 same-sparsity interior-point iterates, 10k buses
    "grid10k_seq20": dict(n_bus=10_000, gamma=1e5, dx=(1e-10, 1e8), ds=(1e-10, 1e8), systems=20),
    # conditioning stress test, 80k buses
    "grid80k": dict(n_bus=80_000, gamma=1e6, dx=(1e-10, 1e10), ds=(1e-10, 1e10), systems=1),
}


def workload_systems(name: str, base_seed: int = 0, n_bus: int | None = None, systems: int | None = None):
    w = WORKLOADS[name]
    nb = n_bus if n_bus is not None else w["n_bus"]
    grid = make_grid(nb, base_seed)
    ns = systems if systems is not None else w["systems"]
    return grid, [make_system(grid, base_seed + 1 + i, w["gamma"], w["dx"], w["ds"]) for i in range(ns)]


def write_mm(path: str, A: CSR, symmetric_lower: bool = False) -> None:
    """Matrix-Market coordinate file with a banner and a comment line (read with
    skip=3 by the reference's `read_mm_file_into_coo`, src/input_functions.cpp:16-52)."""
    r = np.repeat(np.arange(A.n), np.diff(A.rowptr))
    c = A.colidx
    v = A.vals
    if symmetric_lower:
        keep = r >= c
        r, c, v = r[keep], c[keep], v[keep]
    kind = "symmetric" if symmetric_lower else "general"
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate real {kind}\n% synthetic grid\n")
        f.write(f"{A.n} {A.m} {r.shape[0]}\n")
        for a, b, x in zip(r.tolist(), c.tolist(), v.tolist()):
            f.write(f"{a + 1} {b + 1} {x:.17g}\n")


def write_rhs(path: str, v: np.ndarray) -> None:
    """Matrix-Market array file with exactly two header lines (the layout
    `read_rhs` expects, src/input_functions.cpp:198-217)."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{v.shape[0]} 1\n")
        for x in v.tolist():
            f.write(f"{x:.17g}\n")


def write_system(dirpath: str, sysm: KKTSystem, tag: str = "00") -> dict:
    """Write one system as the eight hybrid_solver inputs (skip=3)."""
    os.makedirs(dirpath, exist_ok=True)
    names = {}
    for key, A, sym in (("h", sysm.H, True), ("ds", sysm.Ds, False), ("jc", sysm.Jc, False), ("jd", sysm.Jd, False)):
        p = os.path.join(dirpath, f"block_{key}_{tag}.mtx")
        write_mm(p, A, symmetric_lower=sym)
        names[key] = p
    for key, v in (("rx", sysm.rx), ("rs", sysm.rs), ("ry", sysm.ry), ("ryd", sysm.ryd)):
        p = os.path.join(dirpath, f"block_{key}_{tag}.mtx")
        write_rhs(p, v)
        names[key] = p
    return names
