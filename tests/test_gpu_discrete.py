"""Discrete skeleton parity: GPU (C ABI) vs the C oracle on seeded Bayesian-network data.

Bar: skeleton and contingency counts bit-exact (the counts enter the statistic
unchanged, so identical statistics prove identical counts), sepsets identical, pmax
within 1e-9 relative of the oracle's FP64 evaluation."""
import ctypes as ct

import numpy as np
import pytest

from gpucsl_gb300.synthetic import discrete_bn_data
from oracle import cbind

pytestmark = pytest.mark.gpu


def oracle_discrete(codes, dims, alpha, L, threads=0):
    p, n = codes.shape
    G = np.zeros((p, p), np.uint16)
    sep = np.full((p, p, L), -1, np.int32)
    pmax = np.zeros((p, p))
    st = cbind.OrcStats()
    cbind.lib().orc_discrete_skeleton(cbind.ptr(codes), n, n, p, cbind.ptr(dims), alpha, L, cbind.ptr(G),
                                      cbind.ptr(sep) if L > 0 else None, cbind.ptr(pmax), threads, ct.byref(st))
    pmax[np.tril_indices(p)] = -1
    return G, sep, pmax, st


def run_gpu(codes, dims, alpha, L):
    from gpucsl_gb300 import engine

    p, n = codes.shape
    s = engine.DiscreteSolver(p, n, L, int(dims.max()))
    s.load(codes, dims)
    st = s.run(alpha)
    G, sep, pmax = s.to_host()
    return G, sep, pmax, st


def assert_parity(got, ref):
    G, sep, pmax, st = got
    Gr, sepr, pmaxr, str_ = ref
    assert (G == Gr).all(), int((G != Gr).sum())
    assert (sep == sepr).all()
    iu = np.triu_indices(G.shape[0], 1)
    a, b = pmax[iu], pmaxr[iu]
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    assert ((rel <= 1e-9) | (np.abs(a - b) <= 1e-300)).all(), float(rel.max())
    assert (pmax[np.tril_indices(G.shape[0])] == -1).all()
    assert st.raw["levels_run"] == str_.levels_run
    for l in range(str_.levels_run):
        assert st.raw["tests"][l] == str_.tests[l], l
        if l > 0:
            assert st.raw["removed"][l] == str_.removed[l], l


@pytest.mark.parametrize("seed,p,n,deg,L,card", [
    (3, 20, 2000, 2, 3, (2, 5)),
    (4, 30, 5001, 3, 3, (2, 6)),
    (6, 12, 777, 4, 5, (2, 3)),
])
def test_discrete_parity(cuda, seed, p, n, deg, L, card):
    w = discrete_bn_data(p, n, deg, seed, card_lo=card[0], card_hi=card[1])
    from gpucsl_gb300.engine import ordinal_encode

    codes, dims = ordinal_encode(w.data)
    assert_parity(run_gpu(codes, dims, 0.05, L), oracle_discrete(codes, dims, 0.05, L))


def test_discrete_parity_at_scale(cuda):
    """p = 200, n = 50000, cardinality 2..5, alpha 0.05, max_level 3."""
    w = discrete_bn_data(200, 50000, 2, 3)
    from gpucsl_gb300.engine import ordinal_encode

    codes, dims = ordinal_encode(w.data)
    assert_parity(run_gpu(codes, dims, 0.05, 3), oracle_discrete(codes, dims, 0.05, 3))


def test_discrete_edge_cases(cuda):
    from gpucsl_gb300.engine import ordinal_encode

    rng = np.random.default_rng(1)
    # constant column (one observed value), binary columns, duplicate columns
    n = 3000
    X = np.stack([rng.integers(0, 2, n), np.full(n, 7), rng.integers(0, 4, n), rng.integers(0, 3, n)], 1)
    X = np.concatenate([X, X[:, :1]], 1)
    codes, dims = ordinal_encode(X)
    assert dims.tolist()[1] == 1
    assert_parity(run_gpu(codes, dims, 0.05, 3), oracle_discrete(codes, dims, 0.05, 3))


def test_concurrent_solves_of_different_table_sizes(cuda):
    """Solves on several host threads whose levels need different shared-memory tables
    (cardinality 2 vs up to 5, levels up to 3) give the results of solving them one by one:
    no launch of one thread depends on a limit another thread set."""
    import threading

    import torch

    probs = [discrete_bn_data(40, 4000, 2, 11, card_lo=2, card_hi=2), discrete_bn_data(60, 6000, 3, 12)]
    from gpucsl_gb300 import engine

    alone = []
    for d in probs:
        codes, dims = engine.ordinal_encode(d.data)
        alone.append(run_gpu(codes, dims, 0.05, 3)[:3])
    results = {}
    errors = []

    def worker(k):
        try:
            stream = torch.cuda.Stream()
            codes, dims = engine.ordinal_encode(probs[k % 2].data)
            out = []
            with torch.cuda.stream(stream):
                for _ in range(4):
                    out.append(run_gpu(codes, dims, 0.05, 3)[:3])
            results[k] = out
        except BaseException as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[0]
    for k, outs in results.items():
        for G, sep, pm in outs:
            G0, sep0, pm0 = alone[k % 2]
            assert np.array_equal(G, G0) and np.array_equal(sep, sep0) and np.array_equal(pm, pm0)
