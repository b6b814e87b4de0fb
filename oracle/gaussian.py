"""ORACLE — test infrastructure only.

FP64 NumPy restatement of the reference's Gaussian PC-stable skeleton
(hpi-epic/gpucsl), vectorised per level over conditional-independence tests:

  thresholds           gpucsl/pc/helpers.py:42-50   (tau_l = |Phi^-1(alpha/2)| / sqrt(n - l - 4))
  correlation matrix   gpucsl/pc/helpers.py:58-59   (np.corrcoef, rowvar=False)
  level 0              gpucsl/pc/cuda/gaussian_ci.cu:18-51
  compaction           gpucsl/pc/cuda/helpers/graph_helpers.cu:35-56
  level l              gpucsl/pc/cuda/gaussian_ci.cu:66-120
  CI test (Alg. 7)     gpucsl/pc/cuda/helpers/gaussian_helpers.cu:56-262
  set unranking        gpucsl/pc/cuda/helpers/set_helpers.cu:25-71
  edge removal         gpucsl/pc/cuda/helpers/graph_helpers.cu:81-101
  level loop           gpucsl/pc/discover_skeleton_gaussian.py:60-108
  zmin -> pmax         gpucsl/pc/helpers.py:62-101

The CI test follows the reference's operation order exactly (M2^T M2, Cholesky,
Gauss-Jordan inverse without pivoting, four products, H = M0 - M1 M2+ M1^T) as
loops over matrix indices, vectorised over the batch of tests.

Canonical rules where the reference is non-deterministic:
  * keys: a test of edge {i, j} is (rank, dir); dir = 0 when v_i = min(i, j).  Tests
    of an edge are taken in increasing key order (both directions in lock-step by
    rank), up to and including the first test that removes the edge;
  * the sepset is that first remover's set (a set the reference's CAS race can emit);
  * z*_ij (FP64) is the minimum Z over those tests at every level where {i, j} was
    adjacent at level start; NaN statistics neither remove nor count toward z*;
  * pmax_ij = 2 * norm.sf(sqrt(n - 3) * z*_ij) for i < j, -1 on and below the diagonal.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from math import sqrt

import numpy as np
from scipy.stats import norm

N_THRESHOLDS = 50


def thresholds(num_observations: int, alpha: float) -> list[float]:
    """helpers.py:42-50 restated: entry l-1 is |q|/sqrt(n - l - 3), i.e. tau_l = |q|/sqrt(n-l-4)."""
    out = [0.0] * N_THRESHOLDS
    q = norm.ppf(alpha / 2, loc=0, scale=1)
    for i in range(1, min(N_THRESHOLDS, num_observations - 3) - 1):
        out[i - 1] = abs(q / sqrt(num_observations - i - 3))
    return out


def corrcoef(data: np.ndarray) -> np.ndarray:
    return np.corrcoef(data, rowvar=False)


def fisher_z_level0(r: np.ndarray) -> np.ndarray:
    """gaussian_ci.cu:36-37: Z = |0.5 * log|(1 + r) / (1 - r)||."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.abs(0.5 * np.log(np.abs((1.0 + r) / (1.0 - r))))


# ---------------------------------------------------------------- Alg. 7, batched
def _mm(A, B, d1, d2, d3):
    """R[i][j] = sum_k A[i][k] B[k][j], accumulated from 0.0 in k order (gaussian_helpers.cu:16-25)."""
    R = np.zeros((A.shape[0], d1, d3))
    for i in range(d1):
        for j in range(d3):
            acc = np.zeros(A.shape[0])
            for k in range(d2):
                acc = acc + A[:, i, k] * B[:, k, j]
            R[:, i, j] = acc
    return R


def _mm_t1(A, B, d1, d2, d3):
    """A^T B with A stored d2 x d1 (gaussian_helpers.cu:29-39)."""
    R = np.zeros((A.shape[0], d1, d3))
    for i in range(d1):
        for j in range(d3):
            acc = np.zeros(A.shape[0])
            for k in range(d2):
                acc = acc + A[:, k, i] * B[:, k, j]
            R[:, i, j] = acc
    return R


def _mm_t2(A, B, d1, d2, d3):
    """A B^T with B stored d3 x d2 (gaussian_helpers.cu:43-53)."""
    R = np.zeros((A.shape[0], d1, d3))
    for i in range(d1):
        for j in range(d3):
            acc = np.zeros(A.shape[0])
            for k in range(d2):
                acc = acc + A[:, i, k] * B[:, j, k]
            R[:, i, j] = acc
    return R


def cholesky_batched(A: np.ndarray) -> np.ndarray:
    """gaussian_helpers.cu:183-199 (lower factor; 1/L_jj * (A_ij - sum) off the diagonal)."""
    b, n, _ = A.shape
    L = np.zeros_like(A)
    with np.errstate(all="ignore"):
        for i in range(n):
            for j in range(i + 1):
                s = np.zeros(b)
                for k in range(j):
                    s = s + L[:, i, k] * L[:, j, k]
                if i == j:
                    L[:, i, j] = np.sqrt(A[:, i, i] - s)
                else:
                    L[:, i, j] = (1.0 / L[:, j, j]) * (A[:, i, j] - s)
    return L


def inverse_gauss_jordan_batched(M: np.ndarray) -> np.ndarray:
    """gaussian_helpers.cu:123-151: Gauss-Jordan without pivoting; M is consumed."""
    M = M.copy()
    b, n, _ = M.shape
    inv = np.broadcast_to(np.eye(n), (b, n, n)).copy()
    with np.errstate(all="ignore"):
        for i in range(n):
            piv = M[:, i, i].copy()
            for j in range(n):
                inv[:, i, j] = inv[:, i, j] / piv
                M[:, i, j] = M[:, i, j] / piv
            for j in range(n):
                if j == i:
                    continue
                f = M[:, j, i].copy()
                for k in range(n):
                    inv[:, j, k] = inv[:, j, k] - inv[:, i, k] * f
                    M[:, j, k] = M[:, j, k] - M[:, i, k] * f
    return inv


def m2_inv_batched(M2: np.ndarray) -> np.ndarray:
    """cuPC Alg. 7 as in gaussian_helpers.cu:201-218."""
    l = M2.shape[1]
    with np.errstate(all="ignore"):
        T = _mm_t1(M2, M2, l, l, l)
        L = cholesky_batched(T)
        T = _mm_t1(L, L, l, l, l)
        R = inverse_gauss_jordan_batched(T)
        T = _mm(L, R, l, l, l)
        T2 = _mm(T, R, l, l, l)
        T = _mm_t2(T2, L, l, l, l)
        return _mm_t2(T, M2, l, l, l)


def gaussian_ci_z(C: np.ndarray, vi: np.ndarray, vj: np.ndarray, S: np.ndarray) -> np.ndarray:
    """Z of a batch of tests (gaussian_helpers.cu:240-262, 78-89, 220-227).
    vi, vj: (b,), S: (b, l) variable ids."""
    b, l = S.shape
    M1 = np.empty((b, 2, l))
    M1[:, 0, :] = C[vi[:, None], S]
    M1[:, 1, :] = C[vj[:, None], S]
    M2 = C[S[:, :, None], S[:, None, :]]
    M2i = m2_inv_batched(M2)
    with np.errstate(all="ignore"):
        temp = _mm_t2(M2i, M1, l, l, 2)
        H = _mm(M1, temp, 2, l, 2)
        h00 = 1.0 - H[:, 0, 0]
        h01 = C[vi, vj] - H[:, 0, 1]
        h11 = 1.0 - H[:, 1, 1]
        rho = h01 / (np.sqrt(np.abs(h00)) * np.sqrt(np.abs(h11)))
        return np.abs(0.5 * (np.log(np.abs(1.0 + rho)) - np.log(np.abs(1.0 - rho))))


def gaussian_ci_z_cholesky(C, vi, vj, S):
    """Same statistic through a direct Cholesky of M2 (Schur complement).  Used only to
    bound the algorithmic difference between Alg. 7 and a Cholesky formulation."""
    b, l = S.shape
    M2 = C[S[:, :, None], S[:, None, :]]
    ci = C[vi[:, None], S]
    cj = C[vj[:, None], S]
    with np.errstate(all="ignore"):
        L = np.linalg.cholesky(M2)
        a = np.linalg.solve(L, ci[..., None])[..., 0]
        bb = np.linalg.solve(L, cj[..., None])[..., 0]
        h00 = 1.0 - (a * a).sum(1)
        h11 = 1.0 - (bb * bb).sum(1)
        h01 = C[vi, vj] - (a * bb).sum(1)
        rho = h01 / (np.sqrt(np.abs(h00)) * np.sqrt(np.abs(h11)))
        return np.abs(0.5 * (np.log(np.abs(1.0 + rho)) - np.log(np.abs(1.0 - rho))))


# ------------------------------------------------------------------ combinatorics
def binom_table(kmax: int, lmax: int) -> np.ndarray:
    """T[n, k] = C(n, k) for 0 <= n <= kmax, 0 <= k <= lmax (int64, saturating)."""
    T = np.zeros((kmax + 1, lmax + 1), dtype=object)
    for nn in range(kmax + 1):
        for k in range(lmax + 1):
            if k == 0:
                T[nn, k] = 1
            elif nn == 0:
                T[nn, k] = 0
            else:
                T[nn, k] = T[nn - 1, k - 1] + T[nn - 1, k]
    cap = (1 << 62)
    return np.array([[min(int(x), cap) for x in row] for row in T], dtype=np.int64)


def unrank_batched(K: np.ndarray, rank: np.ndarray, l: int, BT: np.ndarray) -> np.ndarray:
    """Lexicographic unranking (set_helpers.cu:25-49), vectorised: returns 1-based positions (b, l)."""
    b = K.shape[0]
    pos = np.zeros((b, l), np.int64)
    r = rank.astype(np.int64).copy()
    x = np.zeros(b, np.int64)
    for c in range(l):
        x = x + 1
        while True:
            idx = K - x
            cnt = np.where(idx >= 0, BT[np.clip(idx, 0, BT.shape[0] - 1), l - c - 1], 0)
            move = r >= cnt
            if not move.any():
                break
            r = np.where(move, r - cnt, r)
            x = np.where(move, x + 1, x)
        pos[:, c] = x
    return pos


def resolve_batched(adj: np.ndarray, vi: np.ndarray, vj: np.ndarray, pos: np.ndarray) -> np.ndarray:
    """set_helpers.cu:51-57: position q -> nbrs[q-1], or nbrs[q] when nbrs[q-1] >= v_j."""
    idx = pos - 1
    cand = adj[vi[:, None], 1 + idx]
    idx = idx + (cand >= vj[:, None])
    return adj[vi[:, None], 1 + idx].astype(np.int64)


def compact(G: np.ndarray) -> np.ndarray:
    """graph_helpers.cu:35-56 (fresh zeros behind the neighbour list)."""
    p = G.shape[0]
    adj = np.zeros((p, p), np.int32)
    for r in range(p):
        nb = np.nonzero((G[r] != 0) & (np.arange(p) != r))[0]
        adj[r, 0] = nb.size
        adj[r, 1:1 + nb.size] = nb
    return adj


# ------------------------------------------------------------------- skeleton
@dataclass
class LevelStats:
    level: int
    edges: int = 0                 # edges alive at level start (undirected)
    tests_canonical: int = 0       # tests up to and including the first remover per edge
    tests_full: int = 0            # full test space sum_(directions) C(d_i - 1, l)
    removed: int = 0
    min_margin: float = float("inf")  # min |Z - tau| / tau over canonical tests


@dataclass
class GaussianResult:
    skeleton: np.ndarray
    sepsets: np.ndarray
    pmax: np.ndarray
    zmin: np.ndarray
    levels: list = field(default_factory=list)

    @property
    def tests_canonical(self) -> int:
        return sum(s.tests_canonical for s in self.levels)


def _walk_level(C, adj, deg, ei, ej, level, tau, BT, chunk, z_fn):
    """Level `level` for the edges (ei, ej) against the level-start lists `adj`: every
    edge independent of the others (PC-stable).  Returns (zlev per edge, [(edge index,
    sepset)] of removed edges, canonical tests, full tests, smallest decision margin)."""
    K0 = deg[ei] - 1
    K1 = deg[ej] - 1
    R0 = np.where(K0 >= level, BT[np.clip(K0, 0, None), level], 0)
    R1 = np.where(K1 >= level, BT[np.clip(K1, 0, None), level], 0)
    T = R0 + R1
    tests_full = int(T.sum())
    tests_canonical = 0
    min_margin = float("inf")
    removed = []
    Rmin = np.minimum(R0, R1)
    longer_dir = np.where(R0 > R1, 0, 1)
    active = np.nonzero(T > 0)[0]
    zlev = np.full(ei.size, np.inf)
    base = 0
    while active.size:
        m = np.broadcast_to(base + np.arange(chunk)[None, :], (active.size, chunk))
        e = np.broadcast_to(active[:, None], m.shape)
        valid = m < T[e]
        ev, mv = e[valid], m[valid]
        inter = mv < 2 * Rmin[ev]
        rank = np.where(inter, mv >> 1, mv - Rmin[ev])
        dirn = np.where(inter, mv & 1, longer_dir[ev])
        vi = np.where(dirn == 0, ei[ev], ej[ev])
        vj = np.where(dirn == 0, ej[ev], ei[ev])
        K = deg[vi] - 1
        pos = unrank_batched(K, rank, level, BT)
        S = resolve_batched(adj, vi, vj, pos)
        Z = z_fn(C, vi, vj, S)
        with np.errstate(invalid="ignore"):
            rem = Z < tau
            marg = np.abs(Z - tau) / tau if tau > 0 else np.full(Z.shape, np.inf)
        # scatter back to (a, chunk)
        Zg = np.full(m.shape, np.nan)
        Zg[valid] = Z
        remg = np.zeros(m.shape, bool)
        remg[valid] = rem
        Mg = np.full(m.shape, np.inf)
        Mg[valid] = marg
        Sg = np.full(m.shape + (level,), -1, np.int64)
        Sg[valid] = S
        has = remg.any(1)
        first = np.where(has, remg.argmax(1), chunk)
        upto = np.arange(chunk)[None, :] <= first[:, None]
        take = upto & valid
        zt = np.where(take & ~np.isnan(Zg), Zg, np.inf)
        zlev[active] = np.minimum(zlev[active], zt.min(1))
        tests_canonical += int(take.sum())
        mm = np.where(take, Mg, np.inf).min(1)
        min_margin = min(min_margin, float(mm.min(initial=np.inf)))
        for a_idx in np.nonzero(has)[0]:
            removed.append((int(active[a_idx]), Sg[a_idx, first[a_idx]].copy()))
        done = has | (base + chunk >= T[active])
        active = active[~done]
        base += chunk
    return zlev, removed, tests_canonical, tests_full, min_margin


# Worker side of the process pool: the solve's C and the level's lists are shared memory
# blocks that the parent fills; a task attaches them by name and detaches before it
# returns (its results are fresh arrays).
def _pool_level(args):
    from multiprocessing import shared_memory

    c_name, adj_name, p, deg, ei, ej, level, tau, BT, chunk, z_fn = args
    c_shm = shared_memory.SharedMemory(name=c_name)
    adj_shm = shared_memory.SharedMemory(name=adj_name)
    try:
        C = np.ndarray((p, p), np.float64, buffer=c_shm.buf)
        adj = np.ndarray((p, p), np.int32, buffer=adj_shm.buf)
        out = _walk_level(C, adj, deg, ei, ej, level, tau, BT, chunk, z_fn)
        del C, adj
        return out
    finally:
        c_shm.close()
        adj_shm.close()


_POOLS = {}


def _pool(workers):
    """One process pool per worker count for the process's lifetime (started with spawn,
    so it is safe in a process that uses a GPU)."""
    if workers not in _POOLS:
        import multiprocessing as mp
        import os

        # one BLAS thread per worker process (the workers are the parallelism)
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        os.environ.update({k: "1" for k in keys})
        try:
            _POOLS[workers] = mp.get_context("spawn").Pool(workers)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    return _POOLS[workers]


def skeleton(C: np.ndarray, num_observations: int, alpha: float, max_level: int,
             thr: list | None = None, chunk: int = 64, z_fn=gaussian_ci_z, workers: int = 0) -> GaussianResult:
    """Gaussian PC-stable skeleton on correlation matrix C (FP64).  workers > 1 splits each
    level's edges over that many processes (started with spawn); the result is the same."""
    C = np.ascontiguousarray(C, dtype=np.float64)
    p = C.shape[0]
    if thr is None:
        thr = thresholds(num_observations, alpha)
    G = np.ones((p, p), np.uint16)
    sepsets = np.full((p, p, max_level), -1, np.int32)
    zmin = np.full((p, p), np.inf)
    stats = []

    # level 0 (gaussian_ci.cu:18-51): r = C[min * p + max]
    iu, ju = np.triu_indices(p, 1)
    z0 = fisher_z_level0(C[iu, ju])
    tau0 = thr[0]
    keep = ~(z0 < tau0)
    G[iu, ju] = keep
    G[ju, iu] = keep
    np.fill_diagonal(G, 0)
    zmin[iu, ju] = np.where(np.isnan(z0), np.inf, z0)
    st0 = LevelStats(0, edges=iu.size, tests_canonical=iu.size, tests_full=iu.size,
                     removed=int((~keep).sum()))
    with np.errstate(invalid="ignore"):
        if iu.size:
            st0.min_margin = float(np.nanmin(np.abs(z0 - tau0)) / tau0) if tau0 > 0 else float("inf")
    stats.append(st0)

    pool = c_shm = adj_shm = None
    if workers > 1 and max_level >= 1 and p > 1:
        from multiprocessing import shared_memory

        pool = _pool(workers)
        c_shm = shared_memory.SharedMemory(create=True, size=C.nbytes)
        np.ndarray(C.shape, np.float64, buffer=c_shm.buf)[:] = C
    try:
        for level in range(1, max_level + 1):
            adj = compact(G)
            deg = adj[:, 0].astype(np.int64)
            if deg.max(initial=0) - 1 < level:
                break
            if level >= len(thr):
                raise IndexError(f"no Fisher-z threshold for level {level}")
            tau = thr[level]
            st = LevelStats(level)
            ei, ej = np.nonzero(np.triu(G, 1))
            st.edges = ei.size
            BT = binom_table(int(max(deg.max(), 1)), level)
            if pool is None:
                parts = [(np.arange(ei.size), _walk_level(C, adj, deg, ei, ej, level, tau, BT, chunk, z_fn))]
            else:
                # a fresh block per level: workers may still hold the previous level's
                from multiprocessing import shared_memory

                if adj_shm is not None:
                    adj_shm.close()
                    adj_shm.unlink()
                adj_shm = shared_memory.SharedMemory(create=True, size=p * p * 4)
                np.ndarray((p, p), np.int32, buffer=adj_shm.buf)[:] = adj
                # contiguous slices of about equal test counts
                K0, K1 = deg[ei] - 1, deg[ej] - 1
                w = (np.where(K0 >= level, BT[np.clip(K0, 0, None), level], 0)
                     + np.where(K1 >= level, BT[np.clip(K1, 0, None), level], 0) + 1).astype(np.float64)
                cuts = np.searchsorted(np.cumsum(w), np.linspace(0, w.sum(), 4 * workers + 1)[1:-1])
                idx = [x for x in np.split(np.arange(ei.size), cuts) if x.size]
                outs = pool.map(_pool_level, [(c_shm.name, adj_shm.name, p, deg, ei[x], ej[x], level, tau, BT,
                                               chunk, z_fn) for x in idx])
                parts = list(zip(idx, outs))
            zlev = np.full(ei.size, np.inf)
            for x, (zl, removed, tc, tf, mm) in parts:
                zlev[x] = zl
                st.tests_canonical += tc
                st.tests_full += tf
                st.min_margin = min(st.min_margin, mm)
                for a, s in removed:
                    lo, hi = int(ei[x[a]]), int(ej[x[a]])
                    G[lo, hi] = 0
                    G[hi, lo] = 0
                    sepsets[lo, hi, :level] = s
                    sepsets[hi, lo, :level] = s
                    st.removed += 1
            zmin[ei, ej] = np.minimum(zmin[ei, ej], zlev)
            stats.append(st)
    finally:
        for shm in (c_shm, adj_shm):
            if shm is not None:
                shm.close()
                shm.unlink()

    pmax = pmax_from_zmin(zmin, num_observations)
    return GaussianResult(G, sepsets, pmax, zmin, stats)


def pmax_from_zmin(zmin: np.ndarray, num_observations: int) -> np.ndarray:
    """helpers.py:85-101 on FP64 z*: 2 * sf(sqrt(n-3) z), lower triangle and diagonal -1."""
    pm = 2.0 * norm.sf(np.abs(np.sqrt(num_observations - 3) * zmin))
    pm[np.tril_indices(zmin.shape[0])] = -1
    return pm


def executed_tests(res: GaussianResult) -> int:
    return res.tests_canonical
