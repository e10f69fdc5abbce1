"""Driver of the reference's own GPU solve path (oracle/_ref/ref_harness).

MEASUREMENT AND TEST INFRASTRUCTURE ONLY: used by bench.py's reference-GPU
arm and by the GPU tests that compare solutions with the reference build.
The harness is built by oracle/ref_build.py from the reference's sources;
when they were not staged on this machine, ``available()`` is False and
callers report the reference build as unavailable.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

from oracle import ref_build

MAGIC = 0x4B4B5442


def available() -> bool:
    if ref_build.built():
        return True
    try:
        return ref_build.build() is not None
    except RuntimeError:
        return False


def why_unavailable() -> str:
    if not ref_build.staged():
        return "the reference's sources were not staged into oracle/_ref/src on this machine"
    try:
        ref_build.build()
    except RuntimeError as e:
        return "the reference build failed: " + str(e).splitlines()[0]
    return ""


def write_systems(path: str, systems) -> None:
    """Pattern of systems[0] once, then every system's values (same sparsity)."""
    s0 = systems[0]
    n_x, m_c, m_d = s0.n_x, s0.m_c, s0.m_d
    with open(path, "wb") as f:
        np.array([MAGIC, n_x, m_c, m_d, s0.H.nnz, s0.Jc.nnz, s0.Jd.nnz, len(systems)], np.int32).tofile(f)
        np.array([s0.gamma], np.float64).tofile(f)
        for a in (s0.H.rowptr, s0.H.colidx, s0.Ds.rowptr, s0.Ds.colidx, s0.Jc.rowptr, s0.Jc.colidx, s0.Jd.rowptr,
                  s0.Jd.colidx):
            np.ascontiguousarray(a, np.int32).tofile(f)
        for s in systems:
            for a in (s.H.vals, s.Ds.vals, s.Jc.vals, s.Jd.vals, s.rx, s.rs, s.ry, s.ryd):
                np.ascontiguousarray(a, np.float64).tofile(f)


def run(systems, itmax: int = 0, dump: bool = False, calls: int | None = None, timeout: float = 3600.0):
    """Run the reference on a same-sparsity sequence: the first execute() on
    system 0 (symbolic + numeric), then one execute() per system.  Returns
    (records, solutions): one dict per call (see oracle/ref_harness.cpp) and,
    with dump, {system: (x, s, y, yd)} of the numeric calls."""
    if not available():
        raise RuntimeError(why_unavailable())
    s0 = systems[0]
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "systems.bin")
        write_systems(path, systems)
        cmd = [ref_build.EXE, path]
        if itmax:
            cmd += ["--itmax", str(int(itmax))]
        if dump:
            cmd += ["--dump", tmp]
        if calls is not None:
            cmd += ["--calls", str(int(calls))]
        capture = os.path.join(tmp, "reference_stdout.txt")
        env = dict(os.environ, HYKKT_REF_CAPTURE=capture)
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, env=env)
        if r.returncode != 0:
            said = open(capture).read()[-2000:] if os.path.exists(capture) else ""
            raise RuntimeError(f"ref_harness exited {r.returncode}: {r.stderr[-1000:]} reference printed: {said}")
        recs = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
        sols = {}
        if dump:
            n_x, m_c, m_d = s0.n_x, s0.m_c, s0.m_d
            for rec in recs:
                if rec["first"]:
                    continue
                k = rec["system"]
                v = np.fromfile(os.path.join(tmp, f"sol_{k}.bin"), np.float64)
                sols[k] = (v[:n_x].copy(), v[n_x:n_x + m_d].copy(), v[n_x + m_d:n_x + m_d + m_c].copy(),
                           v[n_x + m_d + m_c:].copy())
    return recs, sols
