"""Seeded synthetic workloads with the shapes of the skeleton-discovery benchmarks.

The reference's datasets (coolingData, NCI-60, alarm, link, ...) are downloaded by its
scripts and are not available offline; these generators stand in for them with the
same kinds of inputs:

* linear-Gaussian DAG data: a random topological order, each forward pair an edge with
  probability deg / (p - 1), weights +-U[0.1, 1] with a random sign, N(0, 1) noise,
  X_v = sum_parents w * X_u + eps_v;
* discrete Bayesian-network data: an Erdos-Renyi DAG with the same edge law, at most
  `max_in_degree` parents per node (extra parents dropped), per-variable cardinality
  uniform in [card_lo, card_hi], conditional probability rows drawn from Dirichlet(1),
  ancestral sampling, uint8 codes.

All draws come from numpy.random.default_rng(seed) (PCG64).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class GaussianWorkload:
    data: np.ndarray          # (n, p) float64 or float32, C order
    dag: np.ndarray           # (p, p) uint8, dag[u, v] = 1 for u -> v
    weights: np.ndarray       # (p, p) float64
    seed: int


def random_dag(rng: np.random.Generator, p: int, expected_degree: float) -> np.ndarray:
    """Adjacency of an ER DAG over a random topological order (dag[u, v] = 1 for u -> v)."""
    order = rng.permutation(p)
    prob = 0.0 if p < 2 else min(1.0, expected_degree / (p - 1))
    upper = np.triu(rng.random((p, p)) < prob, 1)
    dag = np.zeros((p, p), np.uint8)
    # position a -> position b (a < b) becomes order[a] -> order[b]
    dag[np.ix_(order, order)] = upper.astype(np.uint8)
    return dag


def gaussian_dag_data(p: int, n: int, expected_degree: float, seed: int,
                      dtype=np.float64) -> GaussianWorkload:
    rng = np.random.default_rng(seed)
    order = rng.permutation(p)
    prob = 0.0 if p < 2 else min(1.0, expected_degree / (p - 1))
    upper = np.triu(rng.random((p, p)) < prob, 1)
    w = rng.uniform(0.1, 1.0, size=(p, p)) * rng.choice([-1.0, 1.0], size=(p, p))
    W = np.where(upper, w, 0.0)
    X = rng.standard_normal((n, p))
    # positions in topological order: column b of the position-space sample depends on a < b
    Z = np.empty((n, p))
    for b in range(p):
        parents = np.nonzero(W[:, b])[0]
        Z[:, b] = X[:, b] + (Z[:, parents] @ W[parents, b] if parents.size else 0.0)
    data = np.empty((n, p))
    data[:, order] = Z
    dag = np.zeros((p, p), np.uint8)
    dag[np.ix_(order, order)] = upper.astype(np.uint8)
    weights = np.zeros((p, p))
    weights[np.ix_(order, order)] = W
    return GaussianWorkload(np.ascontiguousarray(data.astype(dtype)), dag, weights, seed)


@dataclass
class DiscreteWorkload:
    data: np.ndarray          # (n, p) uint8, C order
    dag: np.ndarray
    cardinality: np.ndarray   # (p,) nominal cardinalities
    seed: int


def discrete_bn_data(p: int, n: int, expected_degree: float, seed: int, max_in_degree: int = 3,
                     card_lo: int = 2, card_hi: int = 5) -> DiscreteWorkload:
    rng = np.random.default_rng(seed)
    order = rng.permutation(p)
    prob = 0.0 if p < 2 else min(1.0, expected_degree / (p - 1))
    upper = np.triu(rng.random((p, p)) < prob, 1)
    card = rng.integers(card_lo, card_hi + 1, size=p)
    Z = np.zeros((p, n), np.int64)  # one contiguous row per topological position
    kept = np.zeros((p, p), bool)
    card_pos = card[order]
    for b in range(p):
        parents = np.nonzero(upper[:, b])[0]
        if parents.size > max_in_degree:
            parents = np.sort(rng.choice(parents, size=max_in_degree, replace=False))
        kept[parents, b] = True
        k = int(card_pos[b])
        n_cfg = int(np.prod(card_pos[parents])) if parents.size else 1
        cpt = rng.dirichlet(np.ones(k), size=n_cfg)            # (n_cfg, k)
        cfg = np.zeros(n, np.int64)
        mult = 1
        for u in parents:
            cfg += Z[u] * mult
            mult *= int(card_pos[u])
        cdf = np.cumsum(cpt, axis=1)[cfg]
        u01 = rng.random(n)[:, None]
        Z[b] = np.minimum((u01 > cdf).sum(1), k - 1)
    data = np.empty((n, p), np.uint8)
    data[:, order] = Z.T.astype(np.uint8)
    dag = np.zeros((p, p), np.uint8)
    dag[np.ix_(order, order)] = kept.astype(np.uint8)
    return DiscreteWorkload(np.ascontiguousarray(data), dag, card, seed)


def gaussian_dag_data_device(p: int, n: int, expected_degree: float, seed: int, device="cuda"):
    """gaussian_dag_data's law with the samples drawn on the device: the order, DAG and
    weights come from numpy.random.default_rng(seed) as above, the N(0, 1) noise from a
    torch generator seeded with `seed`, and X = E (I - W)^-1 in topological positions
    (FP64), with (I - W)^-1 = (I + W)(I + W^2)(I + W^4)... for the nilpotent W (matrix
    products only).  Returns an (n, p) float64 device tensor."""
    import torch

    rng = np.random.default_rng(seed)
    order = rng.permutation(p)
    prob = 0.0 if p < 2 else min(1.0, expected_degree / (p - 1))
    upper = np.triu(rng.random((p, p)) < prob, 1)
    w = rng.uniform(0.1, 1.0, size=(p, p)) * rng.choice([-1.0, 1.0], size=(p, p))
    W = torch.from_numpy(np.where(upper, w, 0.0)).to(device)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    E = torch.randn((n, p), generator=gen, dtype=torch.float64, device=device)
    S = torch.eye(p, dtype=torch.float64, device=device)
    P = W.clone()
    for _ in range(max(1, int(np.ceil(np.log2(max(p, 2)))))):
        S = S + S @ P  # S (I + P): the sum of W^k, k < 2^(round + 1)
        P = P @ P
    Z = E @ S
    X = torch.empty_like(Z)
    X[:, torch.from_numpy(order).to(device)] = Z
    return X.contiguous()


def discrete_bn_data_device(p: int, n: int, expected_degree: float, seed: int, max_in_degree: int = 3,
                            card_lo: int = 2, card_hi: int = 5, device="cuda"):
    """discrete_bn_data's law with the samples drawn on the device: order, DAG, parents,
    cardinalities and CPT rows come from numpy.random.default_rng(seed) as there, the
    uniforms of the ancestral sampling from a torch generator seeded with `seed`.
    Returns an (n, p) uint8 device tensor of codes 0..card-1 (not yet ordinal-encoded:
    a value that no sample takes leaves a gap)."""
    import torch

    rng = np.random.default_rng(seed)
    order = rng.permutation(p)
    prob = 0.0 if p < 2 else min(1.0, expected_degree / (p - 1))
    upper = np.triu(rng.random((p, p)) < prob, 1)
    card = rng.integers(card_lo, card_hi + 1, size=p)
    card_pos = card[order]
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    Z = torch.empty((p, n), dtype=torch.int64, device=device)
    for b in range(p):
        parents = np.nonzero(upper[:, b])[0]
        if parents.size > max_in_degree:
            parents = np.sort(rng.choice(parents, size=max_in_degree, replace=False))
        k = int(card_pos[b])
        n_cfg = int(np.prod(card_pos[parents])) if parents.size else 1
        cdf = torch.from_numpy(np.cumsum(rng.dirichlet(np.ones(k), size=n_cfg), axis=1)).to(device)
        cfg = torch.zeros(n, dtype=torch.int64, device=device)
        mult = 1
        for u in parents:
            cfg += Z[u] * mult
            mult *= int(card_pos[u])
        u01 = torch.rand((n, 1), generator=gen, dtype=torch.float64, device=device)
        Z[b] = torch.clamp((u01 > cdf[cfg]).sum(1), max=k - 1)
    data = torch.empty((n, p), dtype=torch.uint8, device=device)
    data[:, torch.from_numpy(order).to(device)] = Z.t().to(torch.uint8)
    return data.contiguous()


def batch_instance_sizes(count: int, base_seed: int = 1000, p_range=(50, 400), n_range=(500, 20000),
                         deg_range=(2.0, 4.0)):
    """Sizes of a batch of uneven Gaussian instances: instance k draws p ~ U{p_range},
    n ~ U{n_range}, expected degree ~ U[deg_range] from default_rng(base_seed + k), and
    its data use seed base_seed + k.  Returns a list of (p, n, deg, seed)."""
    out = []
    for k in range(count):
        rng = np.random.default_rng(base_seed + k)
        p = int(rng.integers(p_range[0], p_range[1] + 1))
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        deg = float(rng.uniform(deg_range[0], deg_range[1]))
        out.append((p, n, deg, base_seed + k))
    return out


def serving_sizes(count: int, seed: int = 7, gaussian_share: float = 0.7, g_p=(20, 2000), g_n=(1000, 50000),
                  d_p=(20, 300), d_n=(10000, 100000)):
    """(kind, p, n) of the requests serving_requests draws with the same arguments, without
    their payloads: request k draws from default_rng(seed * 100003 + k)."""
    out = []
    for k in range(count):
        rng = np.random.default_rng(seed * 100003 + k)
        if rng.random() < gaussian_share:
            p = int(round(np.exp(rng.uniform(np.log(g_p[0]), np.log(g_p[1])))))
            n = int(rng.integers(g_n[0], g_n[1] + 1))
            out.append(("gaussian", p, n))
        else:
            p = int(rng.integers(d_p[0], d_p[1] + 1))
            n = int(rng.integers(d_n[0], d_n[1] + 1))
            out.append(("discrete", p, n))
    return out


def serving_requests(count: int, seed: int = 7, gaussian_share: float = 0.7, max_level: int = 3,
                     g_p=(20, 2000), g_n=(1000, 50000), d_p=(20, 300), d_n=(10000, 100000), d_card=(2, 6),
                     discrete_on_device: bool = True, only=None):
    """A mix of skeleton requests with their payloads in pinned host memory: Gaussian
    (share `gaussian_share`): p log-uniform in g_p, n uniform in g_n, FP32 samples of a
    degree-3 DAG, alpha 0.01; discrete: p uniform in d_p, n uniform in d_n, cardinality
    uniform in d_card, degree 2, alpha 0.05, codes ordinal-encoded.  Each request draws
    its sizes from default_rng(seed * 100003 + k) and its data from seed * 100003 + k
    (discrete samples drawn on the device and encoded there unless discrete_on_device is
    False).  `only` (indices) materialises a subset; rid stays the index.  Arrival times
    are left at 0 (see poisson_arrivals)."""
    import torch

    from .engine import ordinal_encode, ordinal_encode_device
    from .serve import Request

    sizes = serving_sizes(count, seed, gaussian_share, g_p, g_n, d_p, d_n)
    keep = range(count) if only is None else sorted(set(int(k) for k in only))
    out = []
    for k in keep:
        kind, p, n = sizes[k]
        s_k = seed * 100003 + k
        if kind == "gaussian":
            X = gaussian_dag_data_device(p, n, 3.0, s_k).float().cpu().pin_memory()
            out.append(Request(k, "gaussian", p, n, 0.01, max_level, 0.0, samples=X))
        else:
            if discrete_on_device:
                raw = discrete_bn_data_device(p, n, 2, s_k, card_lo=d_card[0], card_hi=d_card[1])
                cd, dd = ordinal_encode_device(raw)
                codes_t = cd[:, :n].cpu().pin_memory()
                dims = dd.cpu().numpy()
            else:
                d = discrete_bn_data(p, n, 2, s_k, card_lo=d_card[0], card_hi=d_card[1])
                codes, dims = ordinal_encode(d.data)
                codes_t = torch.from_numpy(codes).pin_memory()
            out.append(Request(k, "discrete", p, n, 0.05, max_level, 0.0, codes=codes_t, dims=dims))
    return out


def poisson_times(count: int, rate: float, seed: int = 11) -> np.ndarray:
    """Arrival times of `count` requests at `rate` per second (exponential gaps from
    default_rng(seed))."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=count))


def poisson_arrivals(requests, rate: float, seed: int = 11, count: int | None = None):
    """Copies of `requests` with Poisson arrival times at `rate` per second: request with
    rid k gets the k-th time of poisson_times(count, rate, seed) (count defaults to the
    number of requests), so a subset of a trace keeps its arrival times; the payloads
    are shared."""
    from dataclasses import replace

    total = len(requests) if count is None else int(count)
    t = poisson_times(max(total, max((r.rid for r in requests), default=-1) + 1), rate, seed)
    return [replace(r, arrival=float(t[r.rid])) for r in requests]
