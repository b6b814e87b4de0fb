"""Batches of independent Gaussian skeletons on one device.

`GaussianBatch` solves many problems of different sizes together: one batched
tensor-core correlation (the exact digit-product path, one launch per stage for all
instances) and one batched level loop (one launch per kernel and level for all
instances).  Neither enqueues a host read, so both are captured into one CUDA graph
that later solves replay.  The per-level lane-group width of the test kernel is tuned
on the first solves (`autotune`).

Precision "f64" gives, per instance, exactly the results of the single-problem path;
"split" computes the correlation over five of the seven integer digits (15 of the 28
digit-pair products, with a bound eps on its distance to the seven-digit result), tests
in FP32 with an FP64 re-test inside the guard band, both carrying error bounds that
include eps, and solves again with the exact correlation the few instances whose tests
could not be decided on the split one: skeleton and sepsets identical to "f64", pmax
within the FP32 error of z*.  After a split run, C of an instance holds the split
correlation unless that instance was solved again (`InstanceResult.exact_rerun`).
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np

from . import _lib
from .engine import gaussian_thresholds, records_to_dense


@dataclass
class InstanceResult:
    status: int
    levels_run: int
    n_records: int
    tests: int
    retests: int
    exact_rerun: int = 0


class GaussianBatch:
    """Gaussian PC-stable skeletons of `len(ps)` instances (p_k variables, n_k samples)
    at significance `alpha` up to `max_level` (<= 12), solved together on one device."""

    LANE_CHOICES = (32, 8)

    def __init__(self, ps, ns, alpha: float, max_level: int, precision: str = "f64", record_cap=None,
                 device=None):
        torch = _lib.require_cuda()
        if precision not in ("f64", "split"):
            raise ValueError("precision must be 'f64' or 'split'")
        if not 0 <= int(max_level) <= _lib.GCSL_BATCH_MAX_LEVEL:
            raise ValueError(f"max_level must be in [0, {_lib.GCSL_BATCH_MAX_LEVEL}]")
        self.ps = [int(p) for p in ps]
        self.ns = [int(n) for n in ns]
        if len(self.ps) != len(self.ns) or not self.ps:
            raise ValueError("ps and ns must be non-empty and of equal length")
        self.count = len(self.ps)
        self.alpha = float(alpha)
        self.max_level = int(max_level)
        self.precision = precision
        self.split = precision == "split"
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        L = _lib.lib()
        self.corr_plan = None
        self.corr_ws = None
        # outputs and inputs of every instance live in a few flat buffers (views per instance)
        pp = [p * p for p in self.ps]
        off = np.concatenate([[0], np.cumsum(pp)]).astype(np.int64)
        tot = int(off[-1])
        self._C = torch.empty(tot, dtype=torch.float64, device=self.device)
        self._C32 = torch.empty(tot, dtype=torch.float32, device=self.device) if self.split else None
        self._cerr = torch.zeros(self.count, dtype=torch.float64, device=self.device) if self.split else None
        self._G = torch.empty(tot, dtype=torch.int16, device=self.device)
        self._pmax = torch.empty(tot, dtype=torch.float64, device=self.device)
        self.C = [self._C[off[k]:off[k + 1]].view(p, p) for k, p in enumerate(self.ps)]
        self.C32 = [self._C32[off[k]:off[k + 1]].view(p, p) for k, p in enumerate(self.ps)] if self.split else None
        self.G = [self._G[off[k]:off[k + 1]].view(p, p) for k, p in enumerate(self.ps)]
        self.pmax = [self._pmax[off[k]:off[k + 1]].view(p, p) for k, p in enumerate(self.ps)]
        caps = [max(1024, p * 64) if record_cap is None else int(record_cap) for p in self.ps]
        self._alloc_records(caps)
        # host thresholds (kept alive: the instance table points at them)
        self._thr = [(ct.c_double * 50)(*gaussian_thresholds(n, self.alpha)) for n in self.ns]
        if self.split:
            self._lo = [(ct.c_double * 50)(*gaussian_thresholds(n, 1.1 * self.alpha)) for n in self.ns]
            self._hi = [(ct.c_double * 50)(*gaussian_thresholds(n, 0.9 * self.alpha)) for n in self.ns]
        p_arr = (ct.c_int32 * self.count)(*self.ps)
        ws = int(L.gcsl_gauss_batch_workspace_bytes(p_arr, self.count))
        if ws == 0:
            raise ValueError("unsupported instance sizes")
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
        self.plan = _lib.BatchPlan()
        self.graph = None
        self.lanes = {l: 32 for l in range(1, self.max_level + 1)}
        self._prepare()

    # ----------------------------------------------------------- setup
    def _alloc_records(self, caps):
        torch = _lib.require_cuda()
        self.rec_caps = [int(c) for c in caps]
        roff = np.concatenate([[0], np.cumsum(self.rec_caps)]).astype(np.int64)
        self._rec = torch.empty(int(roff[-1]), dtype=torch.int32, device=self.device)
        self.rec = [self._rec[roff[k]:roff[k + 1]] for k in range(self.count)]

    def _instances(self):
        arr = (_lib.GaussInstance * self.count)()
        for k in range(self.count):
            I = arr[k]
            I.C = self.C[k].data_ptr()
            I.C32 = self.C32[k].data_ptr() if self.split else None
            I.p = self.ps[k]
            I.n_obs = self.ns[k]
            I.thresholds = self._thr[k]
            I.n_thresholds = 50
            if self.split:
                I.band_lo = self._lo[k]
                I.band_hi = self._hi[k]
            I.G = self.G[k].data_ptr()
            I.pmax = self.pmax[k].data_ptr()
            I.rec_pool = self.rec[k].data_ptr()
            I.rec_cap = self.rec_caps[k]
            # the split correlation's bound (set only while samples are bound: given
            # correlations are taken as exact)
            I.c_err = (self._cerr.data_ptr() + 8 * k) if (self.split and self.corr_plan is not None) else None
        return arr

    def _prepare(self):
        L = _lib.lib()
        self._inst = self._instances()
        _lib.check(L.gcsl_gauss_batch_prepare(self._inst, self.count, self.max_level,
                                              _lib.GCSL_PREC_SPLIT if self.split else _lib.GCSL_PREC_F64,
                                              self.workspace.data_ptr(), self.workspace.numel(),
                                              ct.byref(self.plan), _lib.stream_ptr()), "gcsl_gauss_batch_prepare")
        for l, lanes in self.lanes.items():
            _lib.check(L.gcsl_gauss_batch_set_lanes(ct.byref(self.plan), l, lanes), "gcsl_gauss_batch_set_lanes")
        self.graph = None

    def bind_samples(self, Xs):
        """Attach device sample matrices (n_k x p_k, row-major, float64 or float32; one
        dtype for all) whose correlations `run` computes first.  The tensors must stay
        alive and in place while the batch is used."""
        torch = _lib.require_cuda()
        L = _lib.lib()
        if len(Xs) != self.count:
            raise ValueError("one sample matrix per instance")
        dt = Xs[0].dtype
        for k, X in enumerate(Xs):
            if X.dim() != 2 or tuple(X.shape) != (self.ns[k], self.ps[k]) or X.dtype != dt or not X.is_contiguous():
                raise ValueError(f"instance {k}: expected a contiguous ({self.ns[k]}, {self.ps[k]}) tensor of {dt}")
        if dt not in (torch.float64, torch.float32):
            raise ValueError("samples must be float64 or float32")
        self._X = list(Xs)
        n = (ct.c_int64 * self.count)(*self.ns)
        p = (ct.c_int32 * self.count)(*self.ps)
        need = int(L.gcsl_corr_tc_batch_workspace_bytes(n, p, self.count))
        if self.corr_ws is None or self.corr_ws.numel() < need:
            self.corr_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        Xp = (ct.c_void_p * self.count)(*[X.data_ptr() for X in Xs])
        ld = (ct.c_int64 * self.count)(*self.ps)
        Cp = (ct.c_void_p * self.count)(*[c.data_ptr() for c in self.C])
        C32p = (ct.c_void_p * self.count)(*[c.data_ptr() for c in self.C32]) if self.split else None
        self.corr_plan = _lib.BatchPlan()
        _lib.check(L.gcsl_corr_tc_batch_prepare(Xp, _lib.GCSL_DTYPE_F64 if dt == torch.float64 else _lib.GCSL_DTYPE_F32,
                                                n, p, ld, Cp, C32p, self.count, self.corr_ws.data_ptr(),
                                                self.corr_ws.numel(), ct.byref(self.corr_plan), _lib.stream_ptr()),
                   "gcsl_corr_tc_batch_prepare")
        if self.split:
            self._prepare()  # the instances now carry the split correlation's bound
        self.graph = None

    def set_correlations(self, Cs):
        """Use given FP64 correlation matrices instead of samples (copied in)."""
        if len(Cs) != self.count:
            raise ValueError("one correlation matrix per instance")
        for k, C in enumerate(Cs):
            self.C[k].copy_(C)
            if self.split:
                self.C32[k].copy_(C.to(self.C32[k].dtype))
        had_samples = self.corr_plan is not None
        self.corr_plan = None
        if self.split and had_samples:
            self._prepare()  # given correlations are exact: no bound
        self.graph = None

    # ------------------------------------------------------------- runs
    def enqueue_correlation(self):
        """The correlation stage alone (split: the five-digit product with its bound)."""
        L = _lib.lib()
        s = _lib.stream_ptr()
        if self.corr_plan is None:
            return
        if self.split:
            _lib.check(L.gcsl_corr_tc_batch_run_split(ct.byref(self.corr_plan), self._cerr.data_ptr(), s),
                       "gcsl_corr_tc_batch_run_split")
        else:
            _lib.check(L.gcsl_corr_tc_batch_run(ct.byref(self.corr_plan), s), "gcsl_corr_tc_batch_run")

    def enqueue_levels(self):
        """The level loop alone (split with samples: first pass, the exact correlation of
        the flagged instances, their exact re-solve)."""
        L = _lib.lib()
        s = _lib.stream_ptr()
        _lib.check(L.gcsl_gauss_batch_run(ct.byref(self.plan), s), "gcsl_gauss_batch_run")
        if self.split and self.corr_plan is not None:
            flags = L.gcsl_gauss_batch_flags(ct.byref(self.plan))
            _lib.check(L.gcsl_corr_tc_batch_run_flagged(ct.byref(self.corr_plan), flags, s),
                       "gcsl_corr_tc_batch_run_flagged")
            _lib.check(L.gcsl_gauss_batch_rerun(ct.byref(self.plan), s), "gcsl_gauss_batch_rerun")

    def enqueue(self):
        """Enqueue correlation (when samples are bound) and the level loop, no sync."""
        self.enqueue_correlation()
        self.enqueue_levels()

    def capture(self):
        """Capture `enqueue` into a CUDA graph replayed by `run(graph=True)`."""
        torch = _lib.require_cuda()
        self.enqueue()  # warm: lazy attributes, module loading
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            g.capture_begin()
            self.enqueue()
            g.capture_end()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = g
        return g

    def run(self, graph: bool = True, sync: bool = True):
        """One solve of the whole batch.  With sync, grows overflowing record pools (and
        solves again) and returns the per-instance results."""
        while True:
            if graph:
                if self.graph is None:
                    self.capture()
                self.graph.replay()
            else:
                self.enqueue()
            if not sync:
                return None
            res = self.collect()
            over = [k for k, r in enumerate(res) if r.n_records > self.rec_caps[k]]
            if not over:
                return res
            caps = list(self.rec_caps)
            for k in over:
                caps[k] = max(2 * caps[k], res[k].n_records)
            self._alloc_records(caps)
            self._prepare()

    def collect(self) -> list[InstanceResult]:
        L = _lib.lib()
        rc = L.gcsl_gauss_batch_collect(ct.byref(self.plan), self._inst, self.count, _lib.stream_ptr())
        res = [InstanceResult(int(I.status), int(I.levels_run), int(I.n_records), int(I.tests), int(I.retests),
                              int(I.exact_rerun)) for I in self._inst]
        if rc not in (_lib.GCSL_OK, _lib.GCSL_ERR_CAPACITY):
            _lib.check(rc, "gcsl_gauss_batch_collect")
        return res

    def to_host(self, k: int):
        """(skeleton uint16, sepsets int32 (p, p, max_level), pmax float64) of instance k."""
        p = self.ps[k]
        n_ints = int(self._inst[k].n_records)
        if n_ints > self.rec_caps[k]:
            raise RuntimeError(f"instance {k}: its sepset records ({n_ints} ints) overflowed the record pool "
                               f"({self.rec_caps[k]} ints); run(sync=True) grows the pools and solves again")
        rec = self.rec[k][:n_ints].cpu().numpy() if n_ints else np.zeros(0, np.int32)
        G = self.G[k].cpu().numpy().view(np.uint16)
        pmax = self.pmax[k].cpu().numpy()
        return G, records_to_dense(rec, n_ints, p, self.max_level), pmax

    # ---------------------------------------------------------- autotuner
    def _time(self, reps: int) -> float:
        torch = _lib.require_cuda()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            self.enqueue()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    def autotune(self, reps: int = 3) -> dict:
        """Per level, the lane-group width of the test kernel (32 lanes per edge, or 8
        for levels <= 4) that gives the fastest whole-batch solve, by coordinate descent
        over the levels.  Results never depend on the choice."""
        L = _lib.lib()
        self.enqueue()
        best = self._time(reps)
        for l in range(1, min(self.max_level, 4) + 1):
            for lanes in self.LANE_CHOICES:
                if lanes == self.lanes[l]:
                    continue
                old = self.lanes[l]
                _lib.check(L.gcsl_gauss_batch_set_lanes(ct.byref(self.plan), l, lanes), "set_lanes")
                t = self._time(reps)
                if t < best:
                    best, self.lanes[l] = t, lanes
                else:
                    _lib.check(L.gcsl_gauss_batch_set_lanes(ct.byref(self.plan), l, old), "set_lanes")
        self.graph = None
        return dict(self.lanes)
