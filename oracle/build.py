"""ORACLE build recipe — test infrastructure only.

Compiles
  * oracle/coracle.c           -> oracle/liboracle.so        (the C restatement; always)
  * the reference's own host-compilable helpers, through oracle/ref_shim.cc
                               -> oracle/_ref/libref_helpers.so
    (only where the reference sources are present; they are read in place from
     gpucsl/pc/cuda/helpers/ of the reference checkout, never copied).

Both are plain gcc/g++ invocations; no build system of the reference is run.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("GPUCSL_REFERENCE_ROOT", "/root/reference"))
REF_HELPERS = REF_ROOT / "gpucsl" / "pc" / "cuda" / "helpers"

ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libref_helpers.so"


def _stale(target: Path, *sources: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "coracle.c"
    if force or _stale(ORACLE_SO, src):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
               str(src), "-o", str(ORACLE_SO), "-lm"]
        subprocess.run(cmd, check=True)
    return ORACLE_SO


def build_ref(force: bool = False) -> Path | None:
    """Build the reference-helper shim; returns None when the reference is absent."""
    if not (REF_HELPERS / "math_helpers.cu").exists():
        return None
    shim = HERE / "ref_shim.cc"
    srcs = [shim] + [REF_HELPERS / f for f in ("math_helpers.cu", "set_helpers.cu", "gaussian_helpers.cu")]
    REF_SO.parent.mkdir(exist_ok=True)
    if force or _stale(REF_SO, *srcs):
        cmd = ["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-DGTEST", "-ffp-contract=off",
               f"-I{REF_HELPERS}", str(shim), "-o", str(REF_SO)]
        subprocess.run(cmd, check=True)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
