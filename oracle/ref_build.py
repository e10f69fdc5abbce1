"""Build recipe for the reference's own GPU solve path (cuSPARSE/cuSOLVER).

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the reference build is a baseline
to time and to compare solutions with; the product never links or loads it.

Two steps, both writing only under ``oracle/_ref/`` (git-ignored):

* ``stage`` -- where a reference checkout is mounted (``HYKKT_REFERENCE_DIR``,
  default ``/root/reference``), copies its ``src/`` translation units and
  headers unmodified into ``oracle/_ref/src/``, so that the GPU machine, which
  has no checkout, can compile them.  Nothing staged is committed.
* ``build`` -- compiles the staged sources and ``oracle/ref_harness.cpp``
  with nvcc for sm_103a into ``oracle/_ref/ref_harness``.  Three shims make
  the reference build under CUDA 13 without editing its files:
    - ``-DCUSPARSE_MV_ALG_DEFAULT=CUSPARSE_SPMV_ALG_DEFAULT`` (the enum was
      removed; used at src/matrix_vector_ops.cu:86,106);
    - a ``cublas.h`` in ``oracle/_ref/shim/`` that includes ``cublas_v2.h``
      (the reference includes both, which CUDA 13 rejects; it only calls the
      v2 API: src/vector_vector_ops.cpp, src/cusparse_utils.cpp:144-146);
    - the configured ``hykkt_defs.hpp`` (src/hykkt_defs.hpp.in with
      HYKKT_USE_AMD off, the reference's default).
  The reference's cmake build is not used.

Usage: python oracle/ref_build.py [stage|build|all]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
SHIM = os.path.join(OUT, "shim")
OBJ = os.path.join(OUT, "obj")
EXE = os.path.join(OUT, "ref_harness")
HARNESS = os.path.join(HERE, "ref_harness.cpp")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# the library's translation units (src/CMakeLists.txt: HYBRID_SRC, HYBRID_SRC_CUDA)
CPP_UNITS = ["MMatrix.cpp", "input_functions.cpp", "vector_vector_ops.cpp", "cusparse_utils.cpp",
             "matrix_matrix_ops.cpp", "PermClass.cpp", "RuizClass.cpp", "SchurComplementConjugateGradient.cpp",
             "CholeskyClass.cpp", "SpgemmClass.cpp", "HykktSolver.cpp"]
CU_UNITS = ["cuda_memory_utils.cu", "matrix_vector_ops.cu", "permcheck.cu"]
DEFINES = ["-DCUSPARSE_MV_ALG_DEFAULT=CUSPARSE_SPMV_ALG_DEFAULT"]


def reference_dir() -> str:
    return os.environ.get("HYKKT_REFERENCE_DIR", "/root/reference")


def staged() -> bool:
    return all(os.path.exists(os.path.join(SRC, f)) for f in CPP_UNITS + CU_UNITS)


def built() -> bool:
    return os.path.exists(EXE)


def stage(verbose: bool = False) -> bool:
    """Copy the reference's src/ sources (unmodified) into oracle/_ref/src/."""
    ref_src = os.path.join(reference_dir(), "src")
    if not os.path.isdir(ref_src):
        return staged()
    os.makedirs(SRC, exist_ok=True)
    for f in sorted(os.listdir(ref_src)):
        if f.endswith((".cpp", ".cu", ".hpp")):
            d = os.path.join(SRC, f)
            s = os.path.join(ref_src, f)
            if not os.path.exists(d) or os.path.getmtime(s) > os.path.getmtime(d):
                shutil.copy2(s, d)
    if verbose:
        print("staged", SRC)
    return True


def _shims() -> None:
    os.makedirs(SHIM, exist_ok=True)
    files = {
        "cublas.h": "/* CUDA 13 rejects cublas.h together with cublas_v2.h; the reference only uses the v2 API */\n"
                    "#pragma once\n#include <cublas_v2.h>\n",
        "hykkt_defs.hpp": "/* src/hykkt_defs.hpp.in configured with HYKKT_USE_AMD off */\n#pragma once\n",
    }
    for name, text in files.items():
        p = os.path.join(SHIM, name)
        if not os.path.exists(p) or open(p).read() != text:
            with open(p, "w") as f:
                f.write(text)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stdout[-4000:] + r.stderr[-4000:])


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str | None:
    """Compile the staged reference and the harness; None when not staged."""
    if not staged():
        return None
    _shims()
    # objects built on another architecture (this recipe runs on x86 and Arm
    # hosts) are rebuilt from scratch
    stamp = os.path.join(OBJ, "ARCH")
    if os.path.exists(OBJ) and (not os.path.exists(stamp) or open(stamp).read() != platform.machine()):
        shutil.rmtree(OBJ)
        if os.path.exists(EXE):
            os.remove(EXE)
    os.makedirs(OBJ, exist_ok=True)
    with open(stamp, "w") as f:
        f.write(platform.machine())
    inc = ["-I", SHIM, "-I", SRC]
    hdrs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".hpp")]
    jobs, objs = [], []
    for u in CPP_UNITS + CU_UNITS + [HARNESS]:
        s = u if os.path.isabs(u) else os.path.join(SRC, u)
        o = os.path.join(OBJ, os.path.basename(u) + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            # the reference's cmake build sets no build type, so its host code
            # is compiled without optimisation (and relies on that: the int
            # instantiations of src/cuda_memory_utils.cu's templates exist only
            # as out-of-line implicit instantiations); device code gets nvcc's
            # default optimisation either way
            opt = ["-O2"] if u == HARNESS else []
            jobs.append([NVCC, *ARCH, *opt, "-std=c++17", *DEFINES, *inc, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(16, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if _newer(EXE, objs):
        _run([NVCC, *ARCH, "-o", EXE, *objs, "-lcusparse", "-lcusolver", "-lcublas"])
    if verbose:
        print("built", EXE)
    return EXE


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("stage", "all"):
        stage(verbose=True)
    if what in ("build", "all"):
        if build(verbose=True) is None:
            sys.exit("reference sources are not staged (run `stage` where the reference is mounted)")
