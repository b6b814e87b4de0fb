"""Serving skeleton requests with continuous batching at level granularity.

Requests (Gaussian: FP32 samples; discrete: ordinal codes and cardinalities) arrive at
arbitrary times.  A request is admitted once the device memory it needs fits in the
budget next to the requests in flight (first come, first served: a large request at
the head waits rather than being overtaken).

* Gaussian requests go to one engine thread that owns two CUDA streams.  On the
  correlation stream an admitted request's samples are copied in and its correlation is
  computed at once.  On the level stream the engine advances, tick by tick, every
  request in flight by one level: first those past their last level get the pmax
  write-back and their results copied into pinned host memory, with an event that
  hands them to the finishing threads as soon as it passes; then the requests in
  progress run their next level; then requests whose correlation is done start (state
  reset, level 0 and level 1).  The requests due for the same levels form one batched
  plan per tick (gcsl_gauss_batch_prepare_staged / gcsl_gauss_batch_step); each request
  keeps its solve state in its own device slice across ticks, so a request that arrives
  while others are in flight joins at the next tick and a finished one leaves at once.
  No host read happens between the levels of a request.
* Gaussian requests with more than `solo_p` (400) variables, which fill the GPU on their
  own, and requests deeper than the batched kernels' 12 levels go to two single-problem
  workers (one stream each) instead.
* Discrete requests go to worker threads, one stream each, which solve them
  concurrently through the single-problem path.
* Finished requests are turned into the reference's output arrays (dense sepsets by the
  library's host routine, outside the GIL) by a pool of finishing threads.
* Without a backlog the batching is skipped: while nothing is in flight concurrently
  and at most `exclusive_backlog` (8) requests wait, the request at the head of the
  queue is solved alone on the whole device through the single-problem path, by the
  dispatching thread on its current stream, exactly as the plain path does, and the
  next one waits for it (`overlap_host=True` finishes such a request's host part on a
  finishing thread while the next one is solved).
  Once more requests wait (or concurrent work is still in flight), every waiting request
  goes to the concurrent engines above.  Sharing the device only pays when requests
  queue up; at low load it only slows each request down.

Latency is measured from a request's arrival to the moment its results are on the
host.  `serve_plain` serves the same trace one request at a time through the plain
single-problem API, for comparison.  Results of a request do not depend on what it was
batched with (each instance keeps its own state).
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes as ct
import sys
import threading
import time
from collections import deque
from dataclasses import dataclass, replace

import numpy as np

from . import _lib
from .engine import DiscreteSolver, GaussianSolver, correlation, gaussian_thresholds, records_to_dense


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
    stages: dict | None = None  # Gaussian engine: seconds of its milestones after the trace start
    path: str = "plain"       # server: "exclusive", "batched", "solo" or "discrete"

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


class _Flow:
    """Requests in flight on the concurrent engines (thread-safe).  Every completion
    wakes the dispatcher, which otherwise sleeps until the next arrival (no polling
    thread competes for the interpreter lock)."""

    def __init__(self):
        self.concurrent = 0
        self.events = 0
        self.cv = threading.Condition()

    def state(self) -> tuple[int, int]:
        with self.cv:
            return self.concurrent, self.events

    def started(self):
        with self.cv:
            self.concurrent += 1

    def finished(self):
        with self.cv:
            self.concurrent -= 1
            self.events += 1
            self.cv.notify_all()

    def wait(self, seen: int, timeout: float):
        """Sleeps up to `timeout` seconds unless a request finished since `seen`."""
        with self.cv:
            if self.events == seen and timeout > 0:
                self.cv.wait(timeout)


class _PinnedPool:
    """Reusable pinned host buffers for result copies, by power-of-two size class and
    shared by every server of the process.  Page-locking fresh host memory takes
    milliseconds and can hold up the device, so each finished request borrows a staging
    buffer, its results are copied out of it on a finishing thread, and it goes back."""

    def __init__(self):
        self.free: dict[int, list] = {}
        self.lock = threading.Lock()

    def get(self, nbytes: int):
        torch = _lib.require_cuda()
        cap = max(1 << 16, 1 << (max(int(nbytes), 1) - 1).bit_length())
        with self.lock:
            lst = self.free.get(cap)
            if lst:
                return lst.pop()
        return torch.empty(cap, dtype=torch.uint8, pin_memory=True)

    def put(self, buf):
        with self.lock:
            self.free.setdefault(buf.numel(), []).append(buf)


_PINNED = _PinnedPool()

_STREAMS: dict = {}
_STREAMS_LOCK = threading.Lock()


def _stream(role: str, index: int = 0, priority: int = 0):
    """The process's stream for a server role on the current device, created once.
    PyTorch's caching allocator keeps a pool per stream, so a server that made fresh
    streams per call would find none of the device buffers cached by earlier calls (or by
    a warm-up) and pay a device allocation for every request size it meets again."""
    torch = _lib.require_cuda()
    key = (torch.cuda.current_device(), role, index)
    with _STREAMS_LOCK:
        st = _STREAMS.get(key)
        if st is None:
            st = _STREAMS[key] = torch.cuda.Stream(priority=priority)
        return st


class _Tick:
    """One tick of the Gaussian engine in flight: its completion event, what must stay
    alive until the stream has passed it, and the requests it finishes with the event
    recorded right after their results were copied out (the tick's first work)."""
    __slots__ = ("event", "keep", "finishing", "fin_event")

    def __init__(self, event, keep, finishing, fin_event):
        self.event, self.keep, self.finishing, self.fin_event = event, keep, finishing, fin_event


class _GaussJob:
    """A Gaussian request in the engine: its device buffers and where it stands."""
    __slots__ = ("r", "adm_t", "nbytes", "X", "cws", "C", "G", "pmax", "rec", "state", "thr", "inst", "corr_ev",
                 "next_level", "status", "host", "batch", "stages")


class SkeletonServer:
    """Continuous-batching server for one device (see the module docstring)."""

    MAX_LEVEL = 12  # the batched level kernels' range; deeper requests take the single-problem path

    def __init__(self, budget_bytes: float = 120e9, discrete_workers: int = 3, finishing_threads: int = 4,
                 max_inflight_ticks: int = 2, solo_p: int = 400, solo_workers: int = 2,
                 discrete_blocks_per_sm: int = 1, exclusive_backlog: int = 8, switch_interval: float = 5e-4,
                 overlap_host: bool = False):
        self.budget = int(budget_bytes)
        # requests solved alone: inline, as the plain path does (True: their host part --
        # copies out, dense sepsets -- runs on a finishing thread while the next request is
        # solved; measured no better at p99, the copies and the scatter then compete with
        # the next solve for the host)
        self.overlap_host = bool(overlap_host)
        # waiting requests up to which the head of the queue is solved alone (negative:
        # never, every request goes to the concurrent engines)
        self.exclusive_backlog = int(exclusive_backlog)
        # the engine thread steps levels in short slices of Python; with the interpreter's
        # default 5 ms switch interval a busy finishing or worker thread holds it off for
        # whole milliseconds per tick
        self.switch_interval = float(switch_interval)
        # Gaussian requests with more variables than solo_p fill the GPU on their own: they
        # gain nothing from sharing a plan, and the single-problem path (FP32-first tests,
        # chunked walks) solves them faster than the batched FP64 level kernels
        self.solo_p = int(solo_p)
        self.solo_workers = max(1, int(solo_workers))
        self.discrete_blocks_per_sm = max(0, int(discrete_blocks_per_sm))
        # discrete solves of different requests overlap on the device: each worker owns a
        # stream, and one solve's host reads between levels leave the GPU to the others
        self.discrete_workers = max(1, int(discrete_workers))
        self.finishing_threads = max(1, int(finishing_threads))
        self.max_inflight = max(1, int(max_inflight_ticks))

    # ----------------------------------------------------------- workers
    def _guard(self, fn, errors, stop, *args):
        try:
            fn(*args)
        except BaseException as e:  # surfaced by serve()
            errors.append(e)
            stop[0] = True

    # -- Gaussian engine -------------------------------------------------
    def _start(self, item, torch, corr_stream):
        """Allocate a request's buffers and enqueue its samples and correlation."""
        L = _lib.lib()
        r, adm_t, nbytes = item
        j = _GaussJob()
        j.r, j.adm_t, j.nbytes = r, adm_t, nbytes
        p, n = r.p, r.n
        with torch.cuda.stream(corr_stream):
            j.X = r.samples.to("cuda", non_blocking=True)
            j.cws = torch.empty(int(L.gcsl_corr_tc_workspace_bytes(n, p)), dtype=torch.uint8, device="cuda")
            j.C = torch.empty((p, p), dtype=torch.float64, device="cuda")
            _lib.check(L.gcsl_corr_f64_tc(j.X.data_ptr(), _lib.GCSL_DTYPE_F32, n, p, p, j.C.data_ptr(),
                                          j.cws.data_ptr(), j.cws.numel(), _lib.stream_ptr(corr_stream)),
                       "gcsl_corr_f64_tc")
            j.corr_ev = torch.cuda.Event()
            j.corr_ev.record(corr_stream)
            j.G = torch.empty((p, p), dtype=torch.int16, device="cuda")
            j.pmax = torch.empty((p, p), dtype=torch.float64, device="cuda")
            j.rec = torch.empty(max(1024, 64 * p), dtype=torch.int32, device="cuda")
            j.state = torch.empty(int(L.gcsl_gauss_state_bytes(p)), dtype=torch.uint8, device="cuda")
        j.thr = (ct.c_double * 50)(*gaussian_thresholds(n, r.alpha))
        I = _lib.GaussInstance()
        I.C, I.p, I.n_obs = j.C.data_ptr(), p, n
        I.thresholds, I.n_thresholds = j.thr, 50
        I.G, I.pmax = j.G.data_ptr(), j.pmax.data_ptr()
        I.rec_pool, I.rec_cap = j.rec.data_ptr(), j.rec.numel()
        I.state = j.state.data_ptr()
        j.inst = I
        j.next_level = 0
        j.host = None
        j.stages = {}
        return j

    def _enqueue_group(self, torch, jobs, first, last, finish, stream, keep):
        """One batched plan over `jobs` (all due for levels first..last), stepped on
        `stream`; returns the pinned status array [done, last level, status, records]."""
        L = _lib.lib()
        k = len(jobs)
        arr = (_lib.GaussInstance * k)(*[j.inst for j in jobs])
        tb = int(L.gcsl_gauss_batch_table_bytes(k))
        ws = torch.empty(tb, dtype=torch.uint8, device="cuda")
        stage = torch.empty(tb, dtype=torch.uint8, pin_memory=True)
        status = torch.zeros(4 * k, dtype=torch.int32, pin_memory=True)
        plan = _lib.BatchPlan()
        sp = _lib.stream_ptr(stream)
        _lib.check(L.gcsl_gauss_batch_prepare_staged(arr, k, max(j.r.max_level for j in jobs), _lib.GCSL_PREC_F64,
                                                     ws.data_ptr(), tb, stage.data_ptr(), tb, ct.byref(plan), sp),
                   "gcsl_gauss_batch_prepare_staged")
        _lib.check(L.gcsl_gauss_batch_step(ct.byref(plan), first, last, 1 if finish else 0, status.data_ptr(), sp),
                   "gcsl_gauss_batch_step")
        keep += [arr, ws, stage, status, plan]
        return status

    def _gaussian_engine(self, q, cv, stop, adm, out, t0, clock, finisher, solo_q, solo_cv):
        torch = _lib.require_cuda()
        # the engine's many short kernels take precedence over the long discrete ones; the
        # correlations of successive requests alternate between two streams (they overlap)
        corr_streams = [_stream("corr", i, priority=-1) for i in range(2)]
        n_started = 0
        level_stream = _stream("levels", priority=-1)
        starting: list[_GaussJob] = []    # correlation enqueued, levels not started
        active: list[_GaussJob] = []      # levels in progress
        inflight: deque[_Tick] = deque()
        while True:
            with cv:
                while not q and not starting and not active and not inflight and not stop[0]:
                    cv.wait(0.05)  # woken by every enqueue and by stop
                if stop[0] and not (q or starting or active or inflight):
                    return
                new = list(q)
                q.clear()
            for item in new:
                if item[0].max_level > self.MAX_LEVEL or item[0].p > self.solo_p:
                    with solo_cv:
                        solo_q.append(item)
                        solo_cv.notify()
                    continue
                j = self._start(item, torch, corr_streams[n_started % len(corr_streams)])
                n_started += 1
                j.stages["corr_enqueued"] = clock() - t0
                starting.append(j)
            # hand finished requests to the finishing threads as soon as their copies are
            # done, and retire the ticks the stream has passed (without waiting)
            for t in inflight:
                if t.finishing and t.fin_event.query():
                    for j in t.finishing:
                        j.stages["finish_done_seen"] = clock() - t0
                        finisher.submit(self._finish_gaussian, j, out, adm, t0, clock)
                    t.finishing = []
            while inflight and not inflight[0].finishing and inflight[0].event.query():
                inflight.popleft()
            ready = [j for j in starting if j.corr_ev.query()]
            for j in ready:
                j.stages.setdefault("corr_done_seen", clock() - t0)
            starting = [j for j in starting if j not in ready]
            # a plan's instances share their level cap: groups by (next level, cap)
            groups, starts = {}, {}
            for j in active:
                groups.setdefault((j.next_level, j.r.max_level), []).append(j)
            for j in ready:
                starts.setdefault(j.r.max_level, []).append(j)
            keep, finishing = [], []
            if (ready or active) and len(inflight) >= self.max_inflight:
                # the level stream is busy: keep the correlation-finished requests for the
                # next tick and come back for new arrivals
                starting = ready + starting
                ready = []
                time.sleep(0.0001)
                continue
            if ready or active:
                # a tick's order: the requests past their last level first (pmax, results
                # copied out, an event), so their host part starts without waiting for the
                # rest of the tick; then the levels of the requests in progress, oldest
                # levels first; then the first levels of the requests whose correlation
                # is done
                fin_ev = None
                for lv, cap in sorted(groups):
                    js = groups[(lv, cap)]
                    if lv <= cap:
                        continue
                    st = self._enqueue_group(torch, js, lv, lv - 1, True, level_stream, keep)
                    with torch.cuda.stream(level_stream):
                        for i, j in enumerate(js):
                            j.status = (st, i)
                            # staging layout: pmax (8 p^2 bytes), records, G (2 p^2): every
                            # part starts at a multiple of its element size
                            pp, nr = j.r.p * j.r.p, j.rec.numel()
                            buf = _PINNED.get(8 * pp + 4 * nr + 2 * pp)
                            j.host = buf
                            buf[:8 * pp].view(torch.float64).copy_(j.pmax.view(-1), non_blocking=True)
                            buf[8 * pp:8 * pp + 4 * nr].view(torch.int32).copy_(j.rec, non_blocking=True)
                            buf[8 * pp + 4 * nr:10 * pp + 4 * nr].view(torch.int16).copy_(
                                j.G.view(-1), non_blocking=True)
                    for j in js:
                        j.stages["finish_enqueued"] = clock() - t0
                    finishing += js
                if finishing:
                    fin_ev = torch.cuda.Event()
                    fin_ev.record(level_stream)
                for lv, cap in sorted(groups):
                    if lv > cap:
                        continue
                    js = groups[(lv, cap)]
                    self._enqueue_group(torch, js, lv, lv, False, level_stream, keep)
                    for j in js:
                        j.next_level = lv + 1
                for j in ready:
                    level_stream.wait_event(j.corr_ev)  # completed already: orders the stream after it
                for cap, js in starts.items():  # start: state reset, level 0 and level 1
                    self._enqueue_group(torch, js, 0, min(1, cap), False, level_stream, keep)
                    for j in js:
                        j.next_level, j.batch = 2, len(js)
                        j.cws = j.X = None  # the correlation is done with them
                active = [j for j in active if j not in finishing] + ready
                ev = torch.cuda.Event()
                ev.record(level_stream)
                inflight.append(_Tick(ev, keep, finishing, fin_ev))
            if not ready and not active and (starting or inflight):
                time.sleep(0.0002)  # correlations or the last ticks running: nothing to step yet

    def _finish_gaussian(self, j, out, adm, t0, clock):
        st, i = j.status
        done, last, status, n_rec = (int(x) for x in st[4 * i:4 * i + 4].tolist())
        r = j.r
        if status != _lib.GCSL_OK or n_rec > j.rec.numel():
            # record pool too small (or an error): solve this request alone through the
            # single-problem path, which grows its pool
            G, sep, pm = self._solve_alone(r, j.C)
        else:
            pp, nr = r.p * r.p, j.rec.numel()
            h = j.host.numpy()
            pm = h[:8 * pp].view(np.float64).reshape(r.p, r.p).copy()
            sep = records_to_dense(h[8 * pp:8 * pp + 4 * n_rec].view(np.int32), n_rec, r.p, r.max_level)
            G = h[8 * pp + 4 * nr:10 * pp + 4 * nr].view(np.uint16).reshape(r.p, r.p).copy()
        if j.host is not None:
            _PINNED.put(j.host)
            j.host = None
        out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, j.adm_t, clock() - t0, j.batch, j.stages,
                            "batched"))
        adm.release(j.nbytes)
        self._flow.finished()

    @staticmethod
    def _solve_alone(r, C):
        s = GaussianSolver(r.p, r.max_level)
        s.run(C, r.n, gaussian_thresholds(r.n, r.alpha))
        return s.to_host()

    def _solo_worker(self, q, cv, stop, adm, out, t0, clock, idx):
        """Gaussian requests beyond the batched kernels' level range or above solo_p
        variables, one at a time per worker (each worker owns a stream)."""
        torch = _lib.require_cuda()
        stream = _stream("solo", idx, priority=-1)
        while True:
            with cv:
                while not q and not stop[0]:
                    cv.wait(0.05)  # woken by every enqueue and by stop
                if not q and stop[0]:
                    return
                r, adm_t, nbytes = q.popleft()
            with torch.cuda.stream(stream):
                X = r.samples.to("cuda", non_blocking=True)
                G, sep, pm = self._solve_alone(r, correlation(X))
            out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0, path="solo"))
            adm.release(nbytes)
            self._flow.finished()

    def _discrete_worker(self, q, cv, stop, adm, out, t0, clock, idx):
        torch = _lib.require_cuda()
        stream = _stream("discrete", idx)
        # a discrete level kernel strides over all its tests with resident blocks; at one
        # block per SM it leaves room on every SM for the Gaussian solves next to it
        _lib.check(_lib.lib().gcsl_set_blocks_per_sm_cap(self.discrete_blocks_per_sm), "gcsl_set_blocks_per_sm_cap")
        while True:
            with cv:
                while not q and not stop[0]:
                    cv.wait(0.05)  # woken by every enqueue and by stop
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
            out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0, path="discrete"))
            adm.release(nbytes)
            self._flow.finished()
            del ds, codes

    # -------------------------------------------------------------- serve
    def warmup(self, requests: list[Request]):
        """Serves every request once through the concurrent engines and once alone (all
        arriving at once), so that the device buffers of every size the requests need are
        cached on each stream the server uses."""
        trace = [replace(r, arrival=0.0) for r in requests]
        saved = self.exclusive_backlog
        try:
            self.exclusive_backlog = -1
            self.serve(trace)
            self.exclusive_backlog = len(trace) + 1
            self.serve(trace)
        finally:
            self.exclusive_backlog = saved

    def serve(self, trace: list[Request], clock=time.perf_counter) -> list[Response]:
        """Serve `trace` (arrival times relative to the call) and return one response per
        request, in completion order."""
        adm = _Admission(self.budget)
        self._flow = flow = _Flow()
        qg, qd, qs = deque(), deque(), deque()
        cvg, cvd, cvs = threading.Condition(), threading.Condition(), threading.Condition()
        stop = [False]
        errors: list[BaseException] = []
        out: list[Response] = []
        finisher = cf.ThreadPoolExecutor(max_workers=self.finishing_threads)
        t0 = clock()

        def fin_guard(fn, *a):
            try:
                fn(*a)
            except BaseException as e:  # surfaced by serve()
                errors.append(e)
                stop[0] = True

        class _Fin:
            def submit(self_, fn, *a):
                return finisher.submit(fin_guard, fn, *a)

        # requests solved alone whose host part is still pending: at most two per
        # finishing thread, so the host work cannot fall behind without bound
        host_slots = threading.BoundedSemaphore(2 * self.finishing_threads)

        def finish_alone(r, fin, adm_t):
            try:
                G, sep, pm = fin()
                out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0, path="exclusive"))
            except BaseException as e:  # surfaced by serve()
                errors.append(e)
                stop[0] = True
            finally:
                host_slots.release()

        wg = threading.Thread(target=self._guard, args=(self._gaussian_engine, errors, stop, qg, cvg, stop, adm, out,
                                                        t0, clock, _Fin(), qs, cvs), daemon=True)
        wss = [threading.Thread(target=self._guard, args=(self._solo_worker, errors, stop, qs, cvs, stop, adm, out,
                                                          t0, clock, i), daemon=True)
               for i in range(self.solo_workers)]
        wds = [threading.Thread(target=self._guard, args=(self._discrete_worker, errors, stop, qd, cvd, stop, adm,
                                                          out, t0, clock, i), daemon=True)
               for i in range(self.discrete_workers)]
        workers = [wg] + wss + wds
        # the engines' threads (and the short switch interval they need) exist only from
        # the first request that goes to them: while every request is solved alone, no
        # other thread of the server shares the interpreter with the solving one
        old_switch = sys.getswitchinterval()
        started = [False]

        def start_engines():
            if not started[0]:
                started[0] = True
                sys.setswitchinterval(self.switch_interval)
                for w in workers:
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
                concurrent, seen = flow.state()
                if waiting and concurrent == 0 and len(waiting) <= self.exclusive_backlog:
                    # no backlog and nothing in flight: the head is solved alone, here, on
                    # this thread's current stream (what the plain path does); arrivals
                    # meanwhile queue up behind it
                    # the host part (copies out, dense sepsets) of each such request is
                    # finished on a finishing thread while the next one is solved
                    r = waiting.popleft()
                    adm_t = clock() - t0
                    if self.overlap_host:
                        host_slots.acquire()
                        fin = start_plain(r)
                        finisher.submit(finish_alone, r, fin, adm_t)
                    else:
                        G, sep, pm = solve_plain(r)
                        out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, adm_t, clock() - t0,
                                            path="exclusive"))
                    continue
                elif waiting:
                    start_engines()
                    while waiting:
                        r = waiting[0]
                        nbytes = footprint(r)
                        if not adm.try_admit(nbytes):
                            break
                        waiting.popleft()
                        flow.started()
                        item = (r, clock() - t0, nbytes)
                        q, cv = (qg, cvg) if r.kind == "gaussian" else (qd, cvd)
                        with cv:
                            q.append(item)
                            cv.notify()
                # sleep until the next arrival, or until a request finishes when some wait
                # (for budget); while every request has been solved alone, in the plain
                # path's short slices
                until_next = pending[0].arrival - (clock() - t0) if pending else 0.05
                if not started[0] and not waiting:
                    time.sleep(max(0.0, min(0.0005, until_next)))
                else:
                    flow.wait(seen, min(until_next, 0.05) if waiting else until_next)
        finally:
            stop[0] = True
            for cv in (cvg, cvd, cvs):
                with cv:
                    cv.notify_all()
            if started[0]:
                for w in workers:
                    w.join()
            finisher.shutdown(wait=True)
            sys.setswitchinterval(old_switch)
        if errors:
            raise errors[0]
        return out


def solve_plain(r: Request):
    """One request through the plain single-problem API on the current stream:
    (skeleton, sepsets, pmax) on the host."""
    torch = _lib.require_cuda()
    if r.kind == "gaussian":
        X = r.samples.to("cuda", non_blocking=True)
        C = correlation(X)
        s = GaussianSolver(r.p, r.max_level)
        s.run(C, r.n, gaussian_thresholds(r.n, r.alpha))
        return s.to_host()
    ds = DiscreteSolver(r.p, r.n, r.max_level, int(r.dims.max()))
    codes = r.codes.to("cuda", non_blocking=True)
    dims = torch.from_numpy(np.ascontiguousarray(r.dims, dtype=np.uint8)).to("cuda", non_blocking=True)
    ds.load(codes_dev=codes, dims_dev=dims)
    ds.run(r.alpha)
    return ds.to_host()


def start_plain(r: Request):
    """The device part of `solve_plain` on the current stream: the solve, then copies of
    its results into a pinned staging buffer.  Returns a function that finishes the
    request on the host (waits for the copies; skeleton, dense sepsets and pmax as
    `solve_plain` returns them), so that a caller can run it on another thread while the
    next request's solve proceeds."""
    torch = _lib.require_cuda()
    if r.kind == "gaussian":
        X = r.samples.to("cuda", non_blocking=True)
        s = GaussianSolver(r.p, r.max_level)
        s.run(correlation(X), r.n, gaussian_thresholds(r.n, r.alpha))
    else:
        s = DiscreteSolver(r.p, r.n, r.max_level, int(r.dims.max()))
        codes = r.codes.to("cuda", non_blocking=True)
        dims = torch.from_numpy(np.ascontiguousarray(r.dims, dtype=np.uint8)).to("cuda", non_blocking=True)
        s.load(codes_dev=codes, dims_dev=dims)
        s.run(r.alpha)
    p, n_rec = r.p, int(s.stats.n_records)
    pp = p * p
    # staging layout: pmax (8 p^2 bytes), records, G (2 p^2): every part starts at a
    # multiple of its element size
    buf = _PINNED.get(8 * pp + 4 * n_rec + 2 * pp)
    buf[:8 * pp].view(torch.float64).copy_(s.pmax.view(-1), non_blocking=True)
    if n_rec:
        buf[8 * pp:8 * pp + 4 * n_rec].view(torch.int32).copy_(s.rec[:n_rec], non_blocking=True)
    buf[8 * pp + 4 * n_rec:10 * pp + 4 * n_rec].view(torch.int16).copy_(s.G.view(-1), non_blocking=True)
    done = torch.cuda.Event()
    done.record()

    def finish():
        done.synchronize()
        h = buf.numpy()
        pm = h[:8 * pp].view(np.float64).reshape(p, p).copy()
        sep = records_to_dense(h[8 * pp:8 * pp + 4 * n_rec].view(np.int32), n_rec, p, r.max_level)
        G = h[8 * pp + 4 * n_rec:10 * pp + 4 * n_rec].view(np.uint16).reshape(p, p).copy()
        _PINNED.put(buf)
        return G, sep, pm

    finish.solver = s  # the device buffers stay alive until the copies have run
    return finish


def serve_plain(trace: list[Request], clock=time.perf_counter) -> list[Response]:
    """The same trace through the plain single-problem API, one request at a time in
    arrival order (a request waits for its arrival and for the previous one)."""
    out: list[Response] = []
    t0 = clock()
    for r in sorted(trace, key=lambda r: r.arrival):
        while clock() - t0 < r.arrival:
            time.sleep(max(0.0, min(0.0005, r.arrival - (clock() - t0))))
        start = clock() - t0
        G, sep, pm = solve_plain(r)
        out.append(Response(r.rid, r.kind, G, sep, pm, r.arrival, start, clock() - t0))
    return out


def latency_summary(resp: list[Response]) -> dict:
    """p50 / p99 / mean latency and throughput of a set of responses, overall and per kind."""
    def summ(rs):
        lat = np.array([r.latency for r in rs])
        span = max(r.done for r in rs) - min(r.arrival for r in rs)
        return {"count": len(rs), "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
                "mean_ms": round(1e3 * float(lat.mean()), 3),
                "skeletons_per_s": round(len(rs) / span, 2) if span > 0 else None,
                "mean_batch": round(float(np.mean([r.batch for r in rs])), 2)}

    out = summ(resp)
    paths: dict[str, int] = {}
    for r in resp:
        paths[r.path] = paths.get(r.path, 0) + 1
    out["paths"] = paths
    for kind in ("gaussian", "discrete"):
        rs = [r for r in resp if r.kind == kind]
        if rs:
            out[kind] = {k: v for k, v in summ(rs).items() if k in ("count", "p50_ms", "p99_ms", "mean_ms")}
    return out
