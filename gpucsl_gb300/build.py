"""Build recipe of libgpucsl_gb300.so: every CUDA source of gpucsl_gb300/csrc is compiled
for sm_103a (one -gencode, in parallel) and linked in-tree into gpucsl_gb300/.

build(debug=True) makes libgpucsl_gb300_debug.so, the same sources with
GCSL_DEBUG_CHECKS=1 (bounds checks that report instead of trapping, permutable work
order): the reference compiles its kernels with -G -lineinfo when is_debug is set
(kernel_management.py:32-33); here is_debug selects this library.  It is built on first
use, as the reference compiles on first use."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgpucsl_gb300.so"
BUILD_DEBUG = PKG / "_build_debug"
LIB_DEBUG = PKG / "libgpucsl_gb300_debug.so"
SOURCES = ["gauss.cu", "capi.cu", "corr.cu", "discrete.cu", "noalloc.cu", "tc_gemm.cu", "corr_tc.cu", "gauss_batch.cu", "orient.cu", "encode.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gpucsl_gb300")
    return cand


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gpucsl_gb300.h"]


def _stale(lib: Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(d.stat().st_mtime > t for d in _deps())


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    lib, bdir = (LIB_DEBUG, BUILD_DEBUG) if debug else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    bdir.mkdir(exist_ok=True)
    nv = nvcc()
    extra = ["-DGCSL_DEBUG_CHECKS=1"] if debug else []

    def compile_one(src: str) -> Path:
        obj = bdir / (Path(src).stem + ".o")
        cmd = [nv, *ARCH, *FLAGS, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
