"""Pack the reference's own test fixtures into compact .npz files.

The reference's CTest cases read Matrix-Market files from src/mats/
(examples/CMakeLists.txt:1-86).  The GPU test machine has no copy of the
reference, so this script (run once, where the reference is mounted) stores
the parsed COO triplets and right-hand sides of the fixtures the tests use:

* a200 AC_09, AC_10 (hybrid1 / solver1) and AC_00 (empty J_d)  -- skip 2
* a2000 AC_09, AC_10 (hybrid2 / solver2)                       -- skip 3
* a200_chol H + rhs (cholesky test)                            -- skip 3
* a200_schur Jc, H, rhs (schur_cg test)                        -- skip 3

Parsing uses plain Python with the reference reader's semantics (the
first `skip` lines are consumed and the last of them holds "n m nnz").
Usage:  python tests/golden/make_fixtures.py <reference checkout>/src/mats
"""
from __future__ import annotations

import os
import sys

import numpy as np

OUT = os.path.dirname(os.path.abspath(__file__))


def read_mm(path: str, skip: int):
    with open(path) as f:
        lines = f.read().split("\n")
    n, m, nnz = (int(t) for t in lines[skip - 1].split()[:3])
    r, c, v = [], [], []
    for ln in lines[skip:]:
        t = ln.split()
        if len(t) < 3:
            continue
        r.append(int(t[0]) - 1)
        c.append(int(t[1]) - 1)
        v.append(float(t[2]))
    assert len(r) == nnz, (path, len(r), nnz)
    return n, m, np.array(r, np.int32), np.array(c, np.int32), np.array(v, np.float64)


def read_rhs(path: str):
    with open(path) as f:
        lines = f.read().split("\n")
    vals = [float(t.split()[0]) for t in lines[2:] if t.strip()]
    return np.array(vals, np.float64)


def pack_system(mats: str, folder: str, case: str, tag: str, skip: int) -> dict:
    d = os.path.join(mats, folder)
    f = lambda k: os.path.join(d, f"block_{k}_{case}_AC_{tag}.mtx")
    out = {"skip": np.int32(skip)}
    for key, name in (("H", "H_matrix"), ("Ds", "Dd_matrix"), ("Jc", "J_matrix"), ("Jd", "Jd_matrix")):
        n, m, r, c, v = read_mm(f(name), skip)
        out[f"{key}_shape"] = np.array([n, m], np.int32)
        out[f"{key}_r"], out[f"{key}_c"], out[f"{key}_v"] = r, c, v
    for key, name in (("rx", "rx"), ("rs", "rs"), ("ry", "ry"), ("ryd", "ryd")):
        out[key] = read_rhs(f(name))
    return out


def main(mats: str) -> None:
    for folder, case, tag, skip in (("a200", "ACTIVSg200", "09", 2), ("a200", "ACTIVSg200", "10", 2),
                                    ("a200", "ACTIVSg200", "00", 2), ("a2000", "ACTIVSg2000", "09", 3),
                                    ("a2000", "ACTIVSg2000", "10", 3)):
        np.savez_compressed(os.path.join(OUT, f"{folder}_AC_{tag}.npz"), **pack_system(mats, folder, case, tag, skip))
    n, m, r, c, v = read_mm(os.path.join(mats, "a200_chol", "H_matrix_ACTIVSg200_AC_00.mtx"), 3)
    np.savez_compressed(os.path.join(OUT, "a200_chol.npz"), H_shape=np.array([n, m], np.int32), H_r=r, H_c=c, H_v=v,
                        rhs=read_rhs(os.path.join(mats, "a200_chol", "rhs_chol_ACTIVSg200_AC_00.mtx")))
    d = os.path.join(mats, "a200_schur")
    n, m, r, c, v = read_mm(os.path.join(d, "JC_matrix_ACTIVSg200_AC_00.mtx"), 3)
    hn, hm, hr, hc, hv = read_mm(os.path.join(d, "H_matrix_ACTIVSg200_AC_00.mtx"), 3)
    np.savez_compressed(os.path.join(OUT, "a200_schur.npz"), Jc_shape=np.array([n, m], np.int32), Jc_r=r, Jc_c=c,
                        Jc_v=v, H_shape=np.array([hn, hm], np.int32), H_r=hr, H_c=hc, H_v=hv,
                        rhs=read_rhs(os.path.join(d, "CG_rhs_ACTIVSg200_AC_00.mtx")))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <reference checkout>/src/mats")
    main(sys.argv[1])
