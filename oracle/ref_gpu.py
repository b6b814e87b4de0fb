"""ORACLE — test and baseline infrastructure only; never imported by the product.

Runs the reference's own Gaussian and discrete CI kernels (RefGaussianKernels,
RefDiscreteKernels).

Gaussian: runs the reference's own Gaussian CI kernels (gpucsl/pc/cuda/gaussian_ci.cu, compiled
unchanged by oracle/build.py into oracle/_ref/ref_gauss_p{P}_l{L}.cubin) on the current
GPU, driven by a host loop that follows the reference's single-GPU worker
(discover_skeleton_gaussian.py:29-108):

    level 0:   gaussian_ci_level_0 over p(p+1)/2 threads
    level l>0: compact, then max over the compacted row counts read back to the host
               (helpers.py:104-118); stop when max - 1 < l; else gaussian_ci_level_n

with the reference's launch geometry (kernel_management.py:46-67, :167-172) and buffer
initialisation (gaussian_device_manager.py:105-131: compacted = skeleton as int32,
separation sets -1, zmin FLT_MAX).  The module is loaded with the CUDA driver API
(ctypes on libcuda) into the primary context that torch uses, and every launch goes to
torch's current stream.  The reference writes the skeleton deterministically (an edge
is removed iff some test removes it) but its separation sets and zmin depend on thread
timing, so only the skeleton is compared with the oracle.

Discrete: the kernels of gpucsl/pc/cuda/discrete_ci.cu (compiled into
oracle/_ref/ref_disc_p{P}_n{N}_d{D}_l{L}.cubin, each level's kernel body behind an
extern "C" kernel ref_disc_level_{l}) driven as discover_skeleton_discrete.py:24-128
drives them: ordinal-encoded samples column-major as uint8, dims = largest code + 1,
pmax 0, separation sets -1, one working-memory block sized by
find_execution_specification (kernel_management.py:378-465; the memory reduction
factor stays 1 for the shapes built here); level 0 on a (p, p) grid of 32 threads,
level l on a (p, p) grid of (64, 2, 1) threads after compact and the host read of the
largest neighbour count.
"""
from __future__ import annotations

import ctypes as ct
import math
from pathlib import Path

_HERE = Path(__file__).resolve().parent
FLT_MAX = 3.4028234663852886e38


class RefGpuUnavailable(RuntimeError):
    pass


def cubin_path(p: int, max_level: int) -> Path:
    return _HERE / "_ref" / f"ref_gauss_p{p}_l{max_level}.cubin"


_cuda = None


def _driver():
    global _cuda
    if _cuda is None:
        try:
            lib = ct.CDLL("libcuda.so.1")
        except OSError as e:
            raise RefGpuUnavailable(f"libcuda not loadable: {e}") from e
        for name in ("cuModuleGetFunctionCount", "cuModuleEnumerateFunctions", "cuFuncGetName"):
            if not hasattr(lib, name):
                raise RefGpuUnavailable(f"driver lacks {name}")
        lib.cuCtxGetCurrent.argtypes = [ct.POINTER(ct.c_void_p)]
        lib.cuModuleLoadData.argtypes = [ct.POINTER(ct.c_void_p), ct.c_char_p]
        lib.cuModuleUnload.argtypes = [ct.c_void_p]
        lib.cuModuleGetFunction.argtypes = [ct.POINTER(ct.c_void_p), ct.c_void_p, ct.c_char_p]
        lib.cuModuleGetFunctionCount.argtypes = [ct.POINTER(ct.c_uint), ct.c_void_p]
        lib.cuModuleEnumerateFunctions.argtypes = [ct.POINTER(ct.c_void_p), ct.c_uint, ct.c_void_p]
        lib.cuFuncGetName.argtypes = [ct.POINTER(ct.c_char_p), ct.c_void_p]
        lib.cuLaunchKernel.argtypes = [ct.c_void_p, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint,
                                       ct.c_uint, ct.c_uint, ct.c_void_p, ct.POINTER(ct.c_void_p),
                                       ct.POINTER(ct.c_void_p)]
        _cuda = lib
    return _cuda


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"CUDA driver error {rc} in {what}")


def _launch(f, grid, block, args, stream):
    params = (ct.c_void_p * len(args))(*[ct.addressof(a) for a in args])
    gx, gy = grid
    bx, by, bz = block
    _check(_driver().cuLaunchKernel(f, gx, gy, 1, bx, by, bz, 0, ct.c_void_p(stream), params, None),
           "cuLaunchKernel")


def _load_module(path: Path):
    import torch

    torch.cuda.init()
    torch.empty(1, device="cuda")  # the primary context is current on this thread
    cu = _driver()
    ctx = ct.c_void_p()
    _check(cu.cuCtxGetCurrent(ct.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RefGpuUnavailable("no current CUDA context")
    image = path.read_bytes()
    mod = ct.c_void_p()
    _check(cu.cuModuleLoadData(ct.byref(mod), image), "cuModuleLoadData")
    return mod


class RefGaussianKernels:
    """The reference's kernels for one (variables, max_level) shape."""

    def __init__(self, p: int, max_level: int):
        path = cubin_path(p, max_level)
        if not path.exists():
            raise RefGpuUnavailable(f"oracle/_ref/{path.name} is absent: oracle/build.py builds it only where the "
                                    "reference sources are present, and it is not part of the committed tree")
        self.p, self.max_level = p, max_level
        self.mod = _load_module(path)
        cu = _driver()
        count = ct.c_uint()
        _check(cu.cuModuleGetFunctionCount(ct.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (ct.c_void_p * count.value)()
        _check(cu.cuModuleEnumerateFunctions(funcs, count.value, self.mod), "cuModuleEnumerateFunctions")
        by_name = {}
        for f in funcs:
            name = ct.c_char_p()
            _check(cu.cuFuncGetName(ct.byref(name), f), "cuFuncGetName")
            by_name[name.value.decode()] = f
        # Itanium-mangled template names: gaussian_ci_level_n<l, P, L>(...), compact<P, P>(...)
        self.level = {}
        for l in range(max_level + 1):
            stem = "gaussian_ci_level_0" if l == 0 else "gaussian_ci_level_n"
            key = f"_Z{len(stem)}{stem}ILi{l}ELi{p}ELi{max_level}EE"
            hits = [f for n, f in by_name.items() if n.startswith(key)]
            if len(hits) != 1:
                raise RefGpuUnavailable(f"kernel for level {l} not found in {path.name}")
            self.level[l] = hits[0]
        hits = [f for n, f in by_name.items() if n.startswith(f"_Z7compactILi{p}ELj{p}EE")]
        if len(hits) != 1:
            raise RefGpuUnavailable(f"compact<{p}, {p}> not found in {path.name}")
        self.compact = hits[0]

    def __del__(self):
        try:
            if _cuda is not None and self.mod:
                _cuda.cuModuleUnload(self.mod)
        except Exception:
            pass

    def _launch(self, f, grid, block, args, stream):
        _launch(f, grid, (block, 1, 1), args, stream)

    def alloc(self):
        """Device buffers as the reference allocates them for one call."""
        import torch

        p, L = self.p, self.max_level
        return {"G": torch.ones((p, p), dtype=torch.int16, device="cuda"),
                "Gc": torch.ones((p, p), dtype=torch.int32, device="cuda"),
                "sep": torch.full((p * p * max(L, 1),), -1, dtype=torch.int32, device="cuda"),
                "zmin": torch.full((p, p), FLT_MAX, dtype=torch.float32, device="cuda")}

    def reset(self, bufs):
        bufs["G"].fill_(1)
        bufs["sep"].fill_(-1)
        bufs["zmin"].fill_(FLT_MAX)

    def run(self, C, thresholds, bufs) -> int:
        """One skeleton level loop on C (p x p float64, on the device).  Returns the
        number of levels run.  Synchronises once per level >= 1, as the reference does."""
        import torch

        p, L = self.p, self.max_level
        assert C.shape == (p, p) and C.dtype == torch.float64 and C.is_contiguous() and C.is_cuda
        stream = torch.cuda.current_stream().cuda_stream
        G, Gc, sep, zmin = bufs["G"], bufs["Gc"], bufs["sep"], bufs["zmin"]
        ptr = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
        levels = 0
        for level in range(L + 1):
            if level == 0:
                needed = p * (p + 1) // 2
                grid, block = (math.ceil(needed / 1024), 1), min(max(32, needed), 1024)
            else:
                self._launch(self.compact, (math.ceil(p / 512), 1), min(512, p),
                             [ptr(G), ptr(Gc), ct.c_uint(0)], stream)
                if int(Gc[:, 0].max().item()) - 1 < level:
                    break
                grid, block = (p, p), 32
            self._launch(self.level[level], grid, block,
                         [ptr(C), ptr(G), ptr(Gc), ct.c_double(float(thresholds[level])), ptr(sep), ptr(zmin),
                          ct.c_int(0)], stream)
            levels += 1
        return levels


# ------------------------------------------------------------------ discrete
DISC_PARALLEL_TESTS = 2  # find_execution_specification: 2 tests per edge, 1 edge per block


def disc_cubin_path(p: int, n: int, max_dim: int, max_level: int) -> Path:
    return _HERE / "_ref" / f"ref_disc_p{p}_n{n}_d{max_dim}_l{max_level}.cubin"


def disc_working_memory_bytes(p: int, max_dim: int, max_level: int) -> int:
    """find_execution_specification with memory reduction factor 1: the largest over
    levels 1..L of 4 bytes x (contingency + marginal tables) x parallel tests."""
    best = 0
    for level in range(1, max_level + 1):
        ds = max_dim ** level
        storage = ds * max_dim * max_dim + 2 * ds * max_dim + ds
        best = max(best, 4 * storage * (p * p * DISC_PARALLEL_TESTS))
    return best


def ordinal_encode(data):
    """Per column, each value's rank among the column's distinct values (what
    sklearn's OrdinalEncoder gives for integer columns), column-major uint8, and dims."""
    import numpy as np

    n, p = data.shape
    codes = np.empty((p, n), np.uint8)
    for j in range(p):
        _, inv = np.unique(data[:, j], return_inverse=True)
        codes[j] = inv.astype(np.uint8)
    dims = (codes.max(axis=1).astype(np.int64) + 1).astype(np.uint8) if n else np.zeros(p, np.uint8)
    return codes, dims


class RefDiscreteKernels:
    """The reference's discrete kernels for one (variables, samples, max_dim, max_level)
    shape."""

    def __init__(self, p: int, n: int, max_dim: int, max_level: int):
        path = disc_cubin_path(p, n, max_dim, max_level)
        if not path.exists():
            raise RefGpuUnavailable(f"oracle/_ref/{path.name} is absent: oracle/build.py builds it only where the "
                                    "reference sources are present, and it is not part of the committed tree")
        self.p, self.n, self.max_dim, self.max_level = p, n, max_dim, max_level
        self.mod = _load_module(path)
        cu = _driver()
        self.level = {}
        for l in range(max_level + 1):
            f = ct.c_void_p()
            _check(cu.cuModuleGetFunction(ct.byref(f), self.mod, f"ref_disc_level_{l}".encode()), "cuModuleGetFunction")
            self.level[l] = f
        self.compact = ct.c_void_p()
        _check(cu.cuModuleGetFunction(ct.byref(self.compact), self.mod, b"ref_compact"), "cuModuleGetFunction")

    def __del__(self):
        try:
            if _cuda is not None and self.mod:
                _cuda.cuModuleUnload(self.mod)
        except Exception:
            pass

    def alloc(self, codes, dims):
        """Device buffers as discover_skeleton_discrete.py:38-70 allocates them."""
        import numpy as np
        import torch

        p, n, L = self.p, self.n, self.max_level
        if codes.shape != (p, n) or codes.dtype != np.uint8:
            raise ValueError("codes must be (p, n) uint8, column-major samples")
        if int(dims.max()) != self.max_dim:
            raise ValueError(f"largest cardinality {int(dims.max())} != the module's max_dim {self.max_dim}")
        if np.any(codes.max(axis=1) >= dims):
            raise ValueError("a code is not below its column's cardinality")
        return {"data": torch.from_numpy(np.ascontiguousarray(codes)).cuda(),
                "dims": torch.from_numpy(np.ascontiguousarray(dims)).cuda(),
                "G": torch.ones((p, p), dtype=torch.int16, device="cuda"),
                "Gc": torch.ones((p, p), dtype=torch.int32, device="cuda"),
                "sep": torch.full((p * p * max(L, 1),), -1, dtype=torch.int32, device="cuda"),
                "pmax": torch.zeros((p, p), dtype=torch.float32, device="cuda"),
                "wm": torch.empty(disc_working_memory_bytes(p, self.max_dim, L), dtype=torch.uint8, device="cuda")}

    def reset(self, bufs):
        bufs["G"].fill_(1)
        bufs["sep"].fill_(-1)
        bufs["pmax"].zero_()

    def run(self, alpha: float, bufs) -> int:
        """One skeleton level loop; returns the number of levels run."""
        import torch

        p, L = self.p, self.max_level
        stream = torch.cuda.current_stream().cuda_stream
        ptr = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
        levels = 0
        for level in range(L + 1):
            if level == 0:
                grid, block = (p, p), (32, 1, 1)
            else:
                _launch(self.compact, (math.ceil(p / 512), 1), (min(512, p), 1, 1),
                        [ptr(bufs["G"]), ptr(bufs["Gc"]), ct.c_uint(0)], stream)
                if int(bufs["Gc"][:, 0].max().item()) - 1 < level:
                    break
                grid, block = (p, p), (64, DISC_PARALLEL_TESTS, 1)
            _launch(self.level[level], grid, block,
                    [ptr(bufs["data"]), ptr(bufs["G"]), ptr(bufs["Gc"]), ptr(bufs["dims"]), ct.c_double(alpha),
                     ptr(bufs["wm"]), ptr(bufs["sep"]), ptr(bufs["pmax"])], stream)
            levels += 1
        return levels
