"""ORACLE build recipe — test infrastructure only.

Compiles
  * oracle/coracle.c           -> oracle/liboracle.so        (the C restatement; always)
  * the reference's own host-compilable helpers, through oracle/ref_shim.cc
                               -> oracle/_ref/libref_helpers.so
    (only where the reference sources are present; they are read in place from
     gpucsl/pc/cuda/helpers/ of the reference checkout, never copied).

  * the reference's own Gaussian level kernels (gpucsl/pc/cuda/gaussian_ci.cu with the
    helpers it includes, read in place) -> oracle/_ref/ref_gauss_p{P}_l{L}.cubin, one
    device-only module per (variables, max_level) shape, as the reference's runtime
    compiler instantiates them (kernel_management.py:199-221, :154-166): the level-0 and
    level-n templates for levels 0..L and compact<P, P>.  The instantiation list is
    written by this recipe; the kernels themselves are the reference's.  Built with
    NDEBUG, so the reference's device asserts compile away.

  * the reference's own discrete kernels (gpucsl/pc/cuda/discrete_ci.cu, read in place)
    -> oracle/_ref/ref_disc_p{P}_n{N}_d{D}_l{L}.cubin per (variables, samples, max_dim,
    max_level) shape.  CUDA 13 rejects the file as it stands: discrete_ci.cu:114
    declares execute_ci_test_for_sepset __global__ and :231 calls it without a launch
    configuration.  The recipe therefore includes the file with __global__ defined as
    __device__ (no source is edited or copied) and launches the reference's kernel
    bodies through extern "C" kernels of its own, one per level plus compact, each a
    single call with the reference's template arguments (kernel_management.py:259-268,
    parallel_ci_tests = 2 from find_execution_specification, :395-397).

The host builds are plain gcc/g++ invocations and the kernels one nvcc call per shape;
no build system of the reference is run.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference checkout: $GPUCSL_REFERENCE_ROOT, else a directory named `reference`
# beside this repository's checkout.  Where neither exists the reference builds are
# skipped (the GPU test box has no checkout; it uses the committed golden fixtures).
REF_ROOT = Path(os.environ.get("GPUCSL_REFERENCE_ROOT") or HERE.parent.parent / "reference")
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


REF_CUDA = REF_ROOT / "gpucsl" / "pc" / "cuda"
# (variables, max_level): the p = 20 workload at max_level 3 and the p = 1000 workload to
# its terminal level 10 (levels 0..10 run).
REF_GPU_SHAPES = ((20, 3), (1000, 10))


def ref_gpu_cubin(p: int, max_level: int) -> Path:
    return HERE / "_ref" / f"ref_gauss_p{p}_l{max_level}.cubin"


def ref_gauss_instantiations(p: int, L: int) -> str:
    """The translation unit compiled for one Gaussian shape: the reference's file and the
    template instances its runtime compiler would request (kernel_management.py:199-221)."""
    sig = "(double *, unsigned short *, int *, double, int *, float *, int)"
    lines = ['#include "gaussian_ci.cu"', f"template __global__ void gaussian_ci_level_0<0, {p}, {L}>{sig};"]
    lines += [f"template __global__ void gaussian_ci_level_n<{l}, {p}, {L}>{sig};" for l in range(1, L + 1)]
    lines.append(f"template __global__ void compact<{p}, {p}u>(unsigned short *, unsigned int *, unsigned int);")
    return "\n".join(lines) + "\n"


def build_ref_gpu(force: bool = False, shapes=REF_GPU_SHAPES) -> list[Path]:
    """Compile the reference's Gaussian CI kernels for sm_103a; [] when the reference
    checkout is absent.  Each module holds gaussian_ci_level_0<0, P, L>,
    gaussian_ci_level_n<l, P, L> for l = 1..L and compact<P, P>."""
    src = REF_CUDA / "gaussian_ci.cu"
    if not src.exists():
        return []
    deps = [src] + [REF_CUDA / "helpers" / f for f in ("gaussian_helpers.cu", "graph_helpers.cu", "set_helpers.cu")]
    out = []
    for p, L in shapes:
        cubin = ref_gpu_cubin(p, L)
        cubin.parent.mkdir(exist_ok=True)
        if force or _stale(cubin, *deps, Path(__file__)):
            inst = cubin.with_suffix(".cu")
            inst.write_text(ref_gauss_instantiations(p, L))
            cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-DNDEBUG",
                   f"-I{REF_CUDA}", f"-I{REF_CUDA / 'helpers'}", str(inst), "-o", str(cubin)]
            subprocess.run(cmd, check=True)
        out.append(cubin)
    return out


# (variables, samples, max_dim, max_level): the p = 200, n = 50000 discrete workload and
# a small case for the parity test; max_dim is the largest observed cardinality.
REF_DISC_SHAPES = ((200, 50000, 5, 3), (24, 4000, 5, 3))
REF_DISC_PARALLEL_TESTS = 2


def ref_disc_cubin(p: int, n: int, max_dim: int, max_level: int) -> Path:
    return HERE / "_ref" / f"ref_disc_p{p}_n{n}_d{max_dim}_l{max_level}.cubin"


def ref_disc_instantiations(p: int, n: int, md: int, L: int) -> str:
    """The translation unit compiled for one discrete shape: the reference's file read
    with __global__ as __device__, and one extern "C" kernel per level (and compact)
    that calls the reference's kernel body with its template arguments."""
    sig = "(uint8_t *d, unsigned short *G, int *Gc, uint8_t *dims, double alpha, uint32_t *wm, int *sep, float *pmax)"
    args = "(d, G, Gc, dims, alpha, wm, sep, pmax)"
    targs = f"{p}, {REF_DISC_PARALLEL_TESTS}, {md}, {n}, {L}"
    lines = ["#include <cstdint>", '#pragma push_macro("__global__")', "#undef __global__",
             "#define __global__ __device__", '#include "discrete_ci.cu"', '#pragma pop_macro("__global__")']
    for l in range(L + 1):
        body = "discrete_ci_level_0" if l == 0 else "discrete_ci_level_n"
        lines.append(f'extern "C" __global__ void ref_disc_level_{l}{sig} {{ {body}<{l}, {targs}>{args}; }}')
    lines.append('extern "C" __global__ void ref_compact(unsigned short *G, unsigned int *Gc, unsigned int di) '
                 f"{{ compact<{p}, {p}u>(G, Gc, di); }}")
    return "\n".join(lines) + "\n"


def build_ref_gpu_discrete(force: bool = False, shapes=REF_DISC_SHAPES) -> list[Path]:
    """Compile the reference's discrete CI kernels for sm_103a; [] when the reference
    checkout is absent.  Exported names: ref_disc_level_{l} for l = 0..L, ref_compact."""
    src = REF_CUDA / "discrete_ci.cu"
    if not src.exists():
        return []
    deps = [src] + [REF_CUDA / "helpers" / f for f in ("discrete_helpers.cu", "graph_helpers.cu", "set_helpers.cu",
                                                          "math_helpers.cu")]
    out = []
    for p, n, md, L in shapes:
        cubin = ref_disc_cubin(p, n, md, L)
        cubin.parent.mkdir(exist_ok=True)
        if force or _stale(cubin, *deps, Path(__file__)):
            inst = cubin.with_suffix(".cu")
            inst.write_text(ref_disc_instantiations(p, n, md, L))
            cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-DNDEBUG",
                   f"-I{REF_CUDA}", f"-I{REF_CUDA / 'helpers'}", str(inst), "-o", str(cubin)]
            subprocess.run(cmd, check=True)
        out.append(cubin)
    return out


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
    print(build_ref_gpu(force="--force" in sys.argv))
    print(build_ref_gpu_discrete(force="--force" in sys.argv))
