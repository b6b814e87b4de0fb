"""Device-resident skeleton solvers over the C ABI.

A solver owns every device buffer of one problem shape (workspace, skeleton, pmax,
sepset record pool) so repeated solves reuse them; inputs and outputs stay in device
memory until `to_host` is called.  All work is enqueued on the current torch stream.
"""
from __future__ import annotations

import ctypes as ct
import math
from dataclasses import dataclass

import numpy as np

from . import _lib


def _torch():
    return _lib.require_cuda()


def records_to_dense(rec: np.ndarray, n_ints: int, p: int, max_level: int) -> np.ndarray:
    """Scatter the int32 sepset records [lo, hi, level, S...] into the reference's dense
    (p, p, max_level) layout filled with -1 (discover_skeleton_gaussian.py:166-168), by
    the library's host routine (gcsl_records_to_dense: multi-threaded fill, no GIL)."""
    out = np.empty((p, p, max_level), np.int32)
    rec = np.ascontiguousarray(np.asarray(rec[:n_ints], dtype=np.int32))
    if rec.size < n_ints:
        raise ValueError(f"{n_ints} record ints announced, {rec.size} given (an overflowed record pool?)")
    _lib.check(_lib.lib().gcsl_records_to_dense(rec.ctypes.data if n_ints else None, int(n_ints), int(p),
                                                int(max_level), out.ctypes.data if out.size else None),
               "gcsl_records_to_dense")
    return out


def gaussian_thresholds(n_obs: int, alpha: float) -> list[float]:
    """The 50 Fisher-z thresholds of helpers.py:42-50: |Phi^-1(alpha/2)| / sqrt(n - l - 4)
    for the levels the table covers, 0.0 after."""
    from scipy.stats import norm

    out = [0.0] * 50
    q = norm.ppf(alpha / 2, loc=0, scale=1)
    for i in range(1, min(50, n_obs - 3) - 1):
        out[i - 1] = abs(q / math.sqrt(n_obs - i - 3))
    return out


def correlation(X, out=None, workspace=None, method: str = "tc"):
    """FP64 correlation matrix of device samples X (n x p, float64/float32, row-major).

    method "dfma": FP64 GEMM on the CUDA cores; "tc": exact integer-digit products on
    the tcgen05 tensor cores (same result to about 2^-48 of sum |x_i||x_j|)."""
    torch = _torch()
    if X.dim() != 2:
        raise ValueError("X must be 2-D (samples x variables)")
    if X.dtype not in (torch.float64, torch.float32):
        X = X.to(torch.float64)
    X = X.contiguous()
    n, p = X.shape
    L = _lib.lib()
    if out is None:
        out = torch.empty((p, p), dtype=torch.float64, device=X.device)
    dt = _lib.GCSL_DTYPE_F64 if X.dtype == torch.float64 else _lib.GCSL_DTYPE_F32
    if method == "tc":
        need = int(L.gcsl_corr_tc_workspace_bytes(n, p))
        if workspace is None or workspace.numel() < need:
            workspace = torch.empty(need, dtype=torch.uint8, device=X.device)
        _lib.check(L.gcsl_corr_f64_tc(X.data_ptr(), dt, n, p, p, out.data_ptr(), workspace.data_ptr(),
                                      workspace.numel(), _lib.stream_ptr()), "gcsl_corr_f64_tc")
        return out
    if method != "dfma":
        raise ValueError(f"unknown correlation method {method!r}")
    need = int(L.gcsl_corr_workspace_bytes(n, p))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=X.device)
    _lib.check(L.gcsl_corr_f64(X.data_ptr(), dt, n, p, p, out.data_ptr(), workspace.data_ptr(), workspace.numel(),
                               _lib.stream_ptr()), "gcsl_corr_f64")
    return out


@dataclass
class SolveStats:
    raw: dict

    @property
    def tests(self) -> int:
        return int(sum(self.raw["tests"]))

    @property
    def levels_run(self) -> int:
        return int(self.raw["levels_run"])


class test_precision:
    """Context manager for the precision of the Gaussian level tests on this thread:
    "default", "fp32_first" or "fp64" (gcsl_set_test_precision).  All give the same
    results; "fp64" exists to show it."""

    _modes = {"default": 0, "fp32_first": 1, "fp64": 2}

    def __init__(self, mode: str):
        self.mode = self._modes[mode]

    def __enter__(self):
        _lib.check(_lib.lib().gcsl_set_test_precision(self.mode), "gcsl_set_test_precision")
        return self

    def __exit__(self, *exc):
        _lib.lib().gcsl_set_test_precision(0)
        return False


class debug_work_order:
    """Context manager for the work order of the bounds-checked build on this thread
    (gcsl_debug_set_work_order): seed 0 is the release order, another seed reverses and
    rotates the order in which edges, units and discrete tests are walked.  Results must
    not depend on it."""

    def __init__(self, seed: int):
        self.seed = int(seed)

    def __enter__(self):
        _lib.check(_lib.lib(True).gcsl_debug_set_work_order(self.seed), "gcsl_debug_set_work_order")
        return self

    def __exit__(self, *exc):
        _lib.lib(True).gcsl_debug_set_work_order(0)
        return False


class GaussianSolver:
    """Gaussian PC-stable skeleton of p variables up to max_level on one device.  With
    debug=True the solves run the bounds-checked build of the kernels (is_debug)."""

    def __init__(self, p: int, max_level: int, device=None, dense_sepsets: bool = False, record_cap: int | None = None,
                 debug: bool = False):
        torch = _torch()
        self.p, self.max_level = int(p), int(max_level)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.debug = bool(debug)
        L = _lib.lib(self.debug)
        ws = int(L.gcsl_gauss_workspace_bytes(self.p, self.max_level))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
        self.G = torch.empty((self.p, self.p), dtype=torch.int16, device=self.device)
        self.pmax = torch.empty((self.p, self.p), dtype=torch.float64, device=self.device)
        if record_cap is None:
            record_cap = max(1024, self.p * 64)
        self.rec = torch.empty(int(record_cap), dtype=torch.int32, device=self.device)
        self.sep_dense = None
        if dense_sepsets and self.max_level > 0:
            self.sep_dense = torch.empty((self.p, self.p, self.max_level), dtype=torch.int32, device=self.device)
        self.stats = _lib.GcslStats()
        self._thr = None

    def run(self, C, num_observations: int, thresholds, sync: bool = True) -> SolveStats | None:
        """Enqueue one solve on the current stream.  With sync=True (default) the call
        waits for it, grows the record pool if it overflowed, and returns the stats."""
        torch = _torch()
        L = _lib.lib(self.debug)
        thr = (ct.c_double * len(thresholds))(*[float(t) for t in thresholds])
        self._thr = thr
        if self.sep_dense is not None:
            self.sep_dense.fill_(-1)
        while True:
            st = self.stats if sync else None
            rc = L.gcsl_gauss_skeleton(
                C.data_ptr(), self.p, int(num_observations), thr, len(thresholds), self.max_level,
                self.G.data_ptr(), _lib.ptr(self.sep_dense), self.rec.data_ptr(), self.rec.numel(),
                self.pmax.data_ptr(), ct.byref(st) if st is not None else None,
                self.workspace.data_ptr(), self.workspace.numel(), _lib.stream_ptr())
            if rc == _lib.GCSL_ERR_CAPACITY and sync:
                need = int(self.stats.n_records)
                self.rec = torch.empty(max(need, 2 * self.rec.numel()), dtype=torch.int32, device=self.device)
                if self.sep_dense is not None:
                    self.sep_dense.fill_(-1)
                continue
            _lib.check(rc, "gcsl_gauss_skeleton")
            return SolveStats(self.stats.as_dict()) if sync else None

    def to_host(self):
        """(skeleton uint16 p x p, sepsets int32 (p, p, max_level), pmax float64 p x p)."""
        n_ints = int(self.stats.n_records)
        rec = self.rec[:n_ints].cpu().numpy() if n_ints else np.zeros(0, np.int32)
        G = self.G.cpu().numpy().view(np.uint16)
        pmax = self.pmax.cpu().numpy()
        sep = records_to_dense(rec, n_ints, self.p, self.max_level)
        return G, sep, pmax


class DiscreteSolver:
    """Discrete (chi-squared) PC-stable skeleton on one device."""

    def __init__(self, p: int, n: int, max_level: int, max_dim: int, device=None, record_cap: int | None = None,
                 debug: bool = False):
        torch = _torch()
        self.p, self.n, self.max_level, self.max_dim = int(p), int(n), int(max_level), int(max_dim)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.ld = (self.n + 15) // 16 * 16
        self.debug = bool(debug)
        L = _lib.lib(self.debug)
        ws = int(L.gcsl_disc_workspace_bytes(self.p, self.n, self.max_level, self.max_dim))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
        self.data = torch.zeros((self.p, self.ld), dtype=torch.uint8, device=self.device)
        self.dims = torch.empty(self.p, dtype=torch.uint8, device=self.device)
        self.G = torch.empty((self.p, self.p), dtype=torch.int16, device=self.device)
        self.pmax = torch.empty((self.p, self.p), dtype=torch.float64, device=self.device)
        if record_cap is None:
            record_cap = max(1024, self.p * 64)
        self.rec = torch.empty(int(record_cap), dtype=torch.int32, device=self.device)
        self.stats = _lib.GcslStats()

    def load(self, codes_colmajor: np.ndarray | None = None, dims: np.ndarray | None = None, codes_dev=None,
             dims_dev=None):
        """Upload (p, n) uint8 codes (column-major samples) and (p,) cardinalities."""
        torch = _torch()
        if codes_dev is not None:
            self.data[:, :self.n].copy_(codes_dev, non_blocking=True)
        else:
            self.data[:, :self.n].copy_(torch.from_numpy(np.ascontiguousarray(codes_colmajor)), non_blocking=False)
        if dims_dev is not None:
            self.dims.copy_(dims_dev)
        else:
            self.dims.copy_(torch.from_numpy(np.ascontiguousarray(dims, dtype=np.uint8)))

    def run(self, alpha: float, sync: bool = True) -> SolveStats | None:
        torch = _torch()
        L = _lib.lib(self.debug)
        while True:
            st = self.stats if sync else None
            rc = L.gcsl_disc_skeleton(
                self.data.data_ptr(), self.ld, self.n, self.p, self.dims.data_ptr(), self.max_dim, float(alpha),
                self.max_level, self.G.data_ptr(), None, self.rec.data_ptr(), self.rec.numel(),
                self.pmax.data_ptr(), ct.byref(st) if st is not None else None,
                self.workspace.data_ptr(), self.workspace.numel(), _lib.stream_ptr())
            if rc == _lib.GCSL_ERR_CAPACITY and sync:
                need = int(self.stats.n_records)
                self.rec = torch.empty(max(need, 2 * self.rec.numel()), dtype=torch.int32, device=self.device)
                continue
            _lib.check(rc, "gcsl_disc_skeleton")
            return SolveStats(self.stats.as_dict()) if sync else None

    def to_host(self):
        n_ints = int(self.stats.n_records)
        rec = self.rec[:n_ints].cpu().numpy() if n_ints else np.zeros(0, np.int32)
        G = self.G.cpu().numpy().view(np.uint16)
        pmax = self.pmax.cpu().numpy()
        sep = records_to_dense(rec, n_ints, self.p, self.max_level)
        return G, sep, pmax


def ordinal_encode_device(X, ld: int | None = None):
    """Device ordinal encoding (gcsl_ordinal_encode) of an (n, p) integer-valued device
    tensor (int32, int64, uint8, or float64 holding integers): returns (codes (p, ld)
    uint8 column-major device tensor, ld = n rounded up to 16 by default, dims (p,) uint8
    device tensor).  Raises GcslError (unsupported) for a column with more than 255
    distinct values or a value range of 4096 or more."""
    torch = _torch()
    if X.dim() != 2:
        raise ValueError("X must be 2-D (samples x variables)")
    dt = {torch.int32: _lib.GCSL_DTYPE_I32, torch.int64: _lib.GCSL_DTYPE_I64, torch.uint8: _lib.GCSL_DTYPE_U8,
          torch.float64: _lib.GCSL_DTYPE_F64}.get(X.dtype)
    if dt is None:
        raise ValueError(f"unsupported dtype {X.dtype}")
    X = X.contiguous()
    n, p = X.shape
    ld = (n + 15) // 16 * 16 if ld is None else int(ld)
    codes = torch.zeros((p, ld), dtype=torch.uint8, device=X.device)
    dims = torch.empty(p, dtype=torch.uint8, device=X.device)
    L = _lib.lib()
    ws = torch.empty(int(L.gcsl_encode_workspace_bytes(p)), dtype=torch.uint8, device=X.device)
    _lib.check(L.gcsl_ordinal_encode(X.data_ptr(), dt, n, p, p, codes.data_ptr(), ld, dims.data_ptr(), ws.data_ptr(),
                                     ws.numel(), _lib.stream_ptr()), "gcsl_ordinal_encode")
    return codes, dims


def ordinal_encode(data: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Per-column codes 0..k-1 over the observed values in sorted order, and k per column
    (the OrdinalEncoder + max+1 of discover_skeleton_discrete.py:38-39, 49).
    Returns (codes (p, n) uint8 column-major, dims (p,) uint8)."""
    data = np.asarray(data)
    n, p = data.shape
    codes = np.empty((p, n), np.uint8)
    dims = np.empty(p, np.uint8)
    if data.dtype.kind in "ui" and n > 0 and data.min() >= 0 and data.max() <= 255:
        # small non-negative integers: the observed values by a presence table per column
        for v in range(p):
            col = data[:, v].astype(np.intp)
            present = np.bincount(col, minlength=256) > 0
            rank = np.cumsum(present) - 1
            codes[v] = rank[col].astype(np.uint8)
            dims[v] = max(int(present.sum()), 1)
        return codes, dims
    for v in range(p):
        uniq, inv = np.unique(data[:, v], return_inverse=True)
        if uniq.size > 255:
            raise ValueError(f"variable {v} has {uniq.size} distinct values; at most 255 are supported")
        codes[v] = inv.astype(np.uint8)
        dims[v] = max(int(inv.max()) + 1 if inv.size else 1, 1)
    return codes, dims
