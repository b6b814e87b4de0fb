"""Serving skeleton requests with continuous batching and memory-budget admission.

Requests (Gaussian: FP32 samples; discrete: ordinal codes and cardinalities) arrive at
arbitrary times.  A request is admitted once the device memory it needs fits in the
budget next to the requests in flight (first come, first served: a large request at
the head waits rather than being overtaken).  Workers own one CUDA stream each:

* the Gaussian workers (two by default) each take every admitted Gaussian request that
  is waiting when they become free and solve them as one `GaussianBatch` (batched
  tensor-core correlation + batched level loop), so requests that arrive while a batch
  runs join the next one; one or two waiting requests go through the single-problem
  path instead, whose solve is shorter than a batch's setup;
* the discrete workers (three by default) each take the next admitted discrete request
  and solve it through `DiscreteSolver`, so discrete solves overlap on the device.

Latency is measured from a request's arrival to the moment its results are on the
host.  `serve_plain` serves the same trace one request at a time through the plain
single-problem API, for comparison.  Results of a request do not depend on what it was
batched with (each instance of a batch keeps its own state).
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import _lib
from .engine import DiscreteSolver, GaussianSolver, correlation, gaussian_thresholds


@dataclass
class Request:
    rid: int
    kind: str                 # "gaussian" | "discrete"
    p: int
    n: int
    alpha: float
    max_level: int
    arrival: float            # seconds after the start of the trace
    samples: object = None    # gaussian: pinned host float32 tensor (n, p)
    codes: object = None      # discrete: pinned host uint8 tensor (p, n), column-major samples
    dims: np.ndarray | None = None


@dataclass
class Response:
    rid: int
    kind: str
    skeleton: np.ndarray
    sepsets: np.ndarray
    pmax: np.ndarray
    arrival: float
    admitted: float
    done: float
    batch: int = 1            # instances solved together with it (itself included)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def gaussian_footprint(p: int, n: int, max_level: int) -> int:
    """Device bytes of one Gaussian request in a batch: samples (FP32), correlation
    workspace (7 BF16 digit planes + int64 partials), C, skeleton, pmax, the level-loop
    slice and a record pool."""
    p_pad = (p + 127) // 128 * 128
    n_pad = (n + 31) // 32 * 32
    return (4 * n * p + 14 * p_pad * n_pad + 16 * p_pad * p_pad + 8 * p * p + 2 * p * p + 8 * p * p
            + (4 + 8 + 8 + 2) * p * p + 4 * max(1024, 64 * p) + 4096)


def discrete_footprint(p: int, n: int, max_level: int, max_dim: int) -> int:
    """Device bytes of one discrete request: codes, skeleton, pmax, workspace, records."""
    L = _lib.lib()
    ld = (n + 15) // 16 * 16
    return (p * ld + 2 * p * p + 8 * p * p + int(L.gcsl_disc_workspace_bytes(p, n, max_level, max_dim))
            + 4 * max(1024, 64 * p) + 4096)


def footprint(req: Request) -> int:
    if req.kind == "gaussian":
        return gaussian_footprint(req.p, req.n, req.max_level)
    return discrete_footprint(req.p, req.n, req.max_level, int(req.dims.max()))


class _Admission:
    """FIFO admission against a byte budget (thread-safe)."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.used = 0
        self.lock = threading.Lock()

    def try_admit(self, nbytes: int) -> bool:
        with self.lock:
            if self.used + nbytes > self.budget and self.used > 0:
                return False
            self.used += nbytes  # a request larger than the whole budget runs alone
            return True

    def release(self, nbytes: int):
        with self.lock:
            self.used -= nbytes


class SkeletonServer:
    """Continuous-batching server for one device."""

    def __init__(self, budget_bytes: float = 120e9, max_batch: int = 256, precision: str = "f64",
                 discrete_workers: int = 3, gaussian_workers: int = 2, solo_max: int = 2):
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)
        self.precision = precision
        # Gaussian workers: each takes every waiting request it can batch; up to solo_max
        # requests are solved one by one through the single-problem path (its solve is
        # shorter than a batch's setup), more form one GaussianBatch
        self.gaussian_workers = max(1, int(gaussian_workers))
        self.solo_max = int(solo_max)
        # discrete solves of different requests overlap on the device: each worker owns a
        # stream, and one solve's host reads between levels leave the GPU to the others
        self.discrete_workers = max(1, int(discrete_workers))

    # ----------------------------------------------------------- workers
    def _guard(self, fn, errors, stop, *args):
        try:
            fn(*args)
        except BaseException as e:  # surfaced by serve()
            errors.append(e)
            stop[0] = True

    def _gaussian_worker(self, q, cv, stop, adm, out, t0, clock):
        torch = _lib.require_cuda()
        from .batch import GaussianBatch

        stream = torch.cuda.Stream()
        while True:
            with cv:
                while not q and not stop[0]:
                    cv.wait(0.001)
                if not q and stop[0]:
                    return
                # the head request and every waiting request with its alpha and level cap
                key = (q[0][0].alpha, q[0][0].max_level)
                batch, rest = [], deque()
                while q:
                    item = q.popleft()
                    if (item[0].alpha, item[0].max_level) == key and len(batch) < self.max_batch:
                        batch.append(item)
                    else:
                        rest.append(item)
                q.extend(rest)
            if len(batch) <= self.solo_max:
                for r, adm_t, nbytes in batch:
                    with torch.cuda.stream(stream):
                        X = r.samples.to("cuda", non_blocking=True)
                        s = GaussianSolver(r.p, r.max_level)
                        s.run(correlation(X), r.n, gaussian_thresholds(r.n, r.alpha))
                        G, sep, pm = s.to_host()
                    out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0, 1))
                    adm.release(nbytes)
                    del s, X
                continue
            with torch.cuda.stream(stream):
                Xs = [r.samples.to("cuda", non_blocking=True) for r, _, _ in batch]
                b = GaussianBatch([r.p for r, _, _ in batch], [r.n for r, _, _ in batch], key[0], key[1],
                                  self.precision)
                b.bind_samples(Xs)
                b.run(graph=False)
                res = [b.to_host(k) for k in range(len(batch))]
            done = clock() - t0
            for k, (r, adm_t, nbytes) in enumerate(batch):
                G, sep, pm = res[k]
                out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, done, len(batch)))
                adm.release(nbytes)
            del b, Xs

    def _discrete_worker(self, q, cv, stop, adm, out, t0, clock):
        torch = _lib.require_cuda()
        stream = torch.cuda.Stream()
        while True:
            with cv:
                while not q and not stop[0]:
                    cv.wait(0.001)
                if not q and stop[0]:
                    return
                r, adm_t, nbytes = q.popleft()
            with torch.cuda.stream(stream):
                ds = DiscreteSolver(r.p, r.n, r.max_level, int(r.dims.max()))
                codes = r.codes.to("cuda", non_blocking=True)
                dims = torch.from_numpy(np.ascontiguousarray(r.dims, dtype=np.uint8)).to("cuda", non_blocking=True)
                ds.load(codes_dev=codes, dims_dev=dims)
                ds.run(r.alpha)
                G, sep, pm = ds.to_host()
            out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0))
            adm.release(nbytes)
            del ds, codes

    # -------------------------------------------------------------- serve
    def serve(self, trace: list[Request], clock=time.perf_counter) -> list[Response]:
        """Serve `trace` (arrival times relative to the call) and return one response per
        request, in completion order."""
        adm = _Admission(self.budget)
        qg, qd = deque(), deque()
        cvg, cvd = threading.Condition(), threading.Condition()
        stop = [False]
        errors: list[BaseException] = []
        out: list[Response] = []
        t0 = clock()
        wgs = [threading.Thread(target=self._guard, args=(self._gaussian_worker, errors, stop, qg, cvg, stop, adm,
                                                          out, t0, clock), daemon=True)
               for _ in range(self.gaussian_workers)]
        wds = [threading.Thread(target=self._guard, args=(self._discrete_worker, errors, stop, qd, cvd, stop, adm,
                                                          out, t0, clock), daemon=True)
               for _ in range(self.discrete_workers)]
        for w in wgs + wds:
            w.start()
        pending = deque(sorted(trace, key=lambda r: r.arrival))
        waiting: deque = deque()  # arrived, not admitted (FIFO)
        try:
            while pending or waiting:
                if errors:
                    break
                now = clock() - t0
                while pending and pending[0].arrival <= now:
                    waiting.append(pending.popleft())
                while waiting:
                    r = waiting[0]
                    nbytes = footprint(r)
                    if not adm.try_admit(nbytes):
                        break
                    waiting.popleft()
                    item = (r, clock() - t0, nbytes)
                    if r.kind == "gaussian":
                        with cvg:
                            qg.append(item)
                            cvg.notify()
                    else:
                        with cvd:
                            qd.append(item)
                            cvd.notify()
                if pending and not waiting:
                    time.sleep(max(0.0, min(0.0005, pending[0].arrival - (clock() - t0))))
                elif waiting:
                    time.sleep(0.0002)
        finally:
            stop[0] = True
            with cvg:
                cvg.notify_all()
            with cvd:
                cvd.notify_all()
            for w in wgs + wds:
                w.join()
        if errors:
            raise errors[0]
        return out


def serve_plain(trace: list[Request], clock=time.perf_counter) -> list[Response]:
    """The same trace through the plain single-problem API, one request at a time in
    arrival order (a request waits for its arrival and for the previous one)."""
    torch = _lib.require_cuda()
    out: list[Response] = []
    t0 = clock()
    for r in sorted(trace, key=lambda r: r.arrival):
        while clock() - t0 < r.arrival:
            time.sleep(max(0.0, min(0.0005, r.arrival - (clock() - t0))))
        start = clock() - t0
        if r.kind == "gaussian":
            X = r.samples.to("cuda", non_blocking=True)
            C = correlation(X)
            s = GaussianSolver(r.p, r.max_level)
            s.run(C, r.n, gaussian_thresholds(r.n, r.alpha))
            G, sep, pm = s.to_host()
        else:
            ds = DiscreteSolver(r.p, r.n, r.max_level, int(r.dims.max()))
            codes = r.codes.to("cuda", non_blocking=True)
            dims = torch.from_numpy(np.ascontiguousarray(r.dims, dtype=np.uint8)).to("cuda")
            ds.load(codes_dev=codes, dims_dev=dims)
            ds.run(r.alpha)
            G, sep, pm = ds.to_host()
        out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, start, clock() - t0))
    return out


def latency_summary(resp: list[Response]) -> dict:
    lat = np.array([r.latency for r in resp])
    span = max(r.done for r in resp) - min(r.arrival for r in resp)
    return {"p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
            "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
            "mean_ms": round(1e3 * float(lat.mean()), 3),
            "skeletons_per_s": round(len(resp) / span, 2) if span > 0 else None,
            "mean_batch": round(float(np.mean([r.batch for r in resp])), 2)}
