"""ORACLE — test and baseline infrastructure only; never imported by the product.

Runs the reference's own Gaussian CI kernels (gpucsl/pc/cuda/gaussian_ci.cu, compiled
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


class RefGaussianKernels:
    """The reference's kernels for one (variables, max_level) shape."""

    def __init__(self, p: int, max_level: int):
        import torch

        path = cubin_path(p, max_level)
        if not path.exists():
            raise RefGpuUnavailable(f"{path.name} not built (the reference checkout was absent at build time)")
        self.p, self.max_level = p, max_level
        torch.cuda.init()
        torch.empty(1, device="cuda")  # the primary context is current on this thread
        cu = _driver()
        ctx = ct.c_void_p()
        _check(cu.cuCtxGetCurrent(ct.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RefGpuUnavailable("no current CUDA context")
        self._image = path.read_bytes()
        self.mod = ct.c_void_p()
        _check(cu.cuModuleLoadData(ct.byref(self.mod), self._image), "cuModuleLoadData")
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
        params = (ct.c_void_p * len(args))(*[ct.addressof(a) for a in args])
        gx, gy = grid
        _check(_driver().cuLaunchKernel(f, gx, gy, 1, block, 1, 1, 0, ct.c_void_p(stream), params, None),
               "cuLaunchKernel")

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
