"""Parity of the batched and serving paths at the shapes of their benchmark workloads.

* Batched (512 uneven instances, p ~ U{50..400}, n ~ U{500..20000}, alpha 0.01, levels
  <= 4): 32 instances of that generator, chosen deterministically and including the
  largest p, the largest n and the smallest p (a single 128-row tile), solved as one
  batch in FP64 and in split precision.  FP64: skeleton and sepsets bit-exact against
  the oracle, canonical test counts identical, pmax within 1e-9 relative.  Split: the
  same skeleton, sepsets and test counts as FP64, and pmax within the split path's
  stated bound (1e-4 absolute; 1e-2 relative where the FP64 value is at least 1e-6).
* Serving (Poisson mix, 70 % Gaussian with FP32 samples, 30 % discrete, levels <= 3):
  requests of that generator with the largest draws forced in (Gaussian p = 2000,
  n = 50000; discrete p = 300, n = 100000, cardinality up to 6); every response of the
  continuous-batching server equals the plain single-request path's, bit for bit.
"""
import numpy as np
import pytest

from oracle import gaussian as og

pytestmark = pytest.mark.gpu

ALPHA, MAXL = 0.01, 4
SPLIT_PMAX_ABS, SPLIT_PMAX_REL = 1e-4, 1e-2


def batch_pick(sizes, count=32):
    ps = np.array([s[0] for s in sizes])
    ns = np.array([s[1] for s in sizes])
    must = [int(ps.argmax()), int(ns.argmax()), int(ps.argmin())]
    rest = [int(k) for k in np.linspace(0, len(sizes) - 1, count) if int(k) not in must]
    out = list(dict.fromkeys(must + rest))[:count]
    return out


@pytest.fixture(scope="module")
def cfg4(cuda):
    from gpucsl_gb300.batch import GaussianBatch
    from gpucsl_gb300.synthetic import batch_instance_sizes, gaussian_dag_data_device

    torch = cuda
    sizes = batch_instance_sizes(512)
    idx = batch_pick(sizes)
    chosen = [sizes[k] for k in idx]
    assert max(s[0] for s in chosen) == max(s[0] for s in sizes)
    assert max(s[1] for s in chosen) == max(s[1] for s in sizes)
    assert min(s[0] for s in chosen) <= 64
    Xs = [gaussian_dag_data_device(p, n, d, seed) for (p, n, d, seed) in chosen]
    ps, ns = [s[0] for s in chosen], [s[1] for s in chosen]
    out = {}
    for prec in ("f64", "split"):
        b = GaussianBatch(ps, ns, ALPHA, MAXL, prec)
        b.bind_samples(Xs)
        res = b.run(graph=True)
        out[prec] = (b, res)
    torch.cuda.synchronize()
    return chosen, out


def test_cfg4_f64_batch_equals_oracle(cfg4):
    chosen, out = cfg4
    b, res = out["f64"]
    for k, (p, n, _, seed) in enumerate(chosen):
        assert res[k].status == 0, (seed, res[k].status)
        G, sep, pmax = b.to_host(k)
        ref = og.skeleton(b.C[k].cpu().numpy(), n, ALPHA, MAXL)
        assert (G == ref.skeleton).all(), seed
        assert (sep == ref.sepsets).all(), seed
        assert res[k].tests == ref.tests_canonical, (seed, res[k].tests, ref.tests_canonical)
        iu = np.triu_indices(p, 1)
        rel = np.abs(pmax[iu] - ref.pmax[iu]) / np.maximum(np.abs(ref.pmax[iu]), 1e-300)
        assert (rel <= 1e-9).all(), (seed, float(rel.max()))


def test_cfg4_split_batch_keeps_every_decision(cfg4):
    chosen, out = cfg4
    b64, r64 = out["f64"]
    b32, r32 = out["split"]
    worst_abs = worst_rel = 0.0
    for k, (p, n, _, seed) in enumerate(chosen):
        assert r32[k].status == 0, (seed, r32[k].status)
        G, sep, pmax = b64.to_host(k)
        G2, sep2, pmax2 = b32.to_host(k)
        assert (G == G2).all(), seed
        assert (sep == sep2).all(), seed
        assert r32[k].tests == r64[k].tests, (seed, r32[k].tests, r64[k].tests)
        iu = np.triu_indices(p, 1)
        d = np.abs(pmax[iu] - pmax2[iu])
        worst_abs = max(worst_abs, float(d.max()))
        big = pmax[iu] >= 1e-6
        if big.any():
            worst_rel = max(worst_rel, float((d[big] / pmax[iu][big]).max()))
    assert worst_abs <= SPLIT_PMAX_ABS, worst_abs
    assert worst_rel <= SPLIT_PMAX_REL, worst_rel


@pytest.fixture(scope="module")
def cfg5_requests(cuda):
    """Requests of the serving generator plus its largest draws."""
    import torch

    from gpucsl_gb300.engine import ordinal_encode
    from gpucsl_gb300.serve import Request
    from gpucsl_gb300.synthetic import discrete_bn_data, gaussian_dag_data_device, serving_requests

    reqs = serving_requests(10, seed=19)
    k = len(reqs)
    Xg = gaussian_dag_data_device(2000, 50000, 3.0, 9001).float().cpu().pin_memory()
    reqs.append(Request(k, "gaussian", 2000, 50000, 0.01, 3, 0.0, samples=Xg))
    d = discrete_bn_data(300, 100000, 2, 9002, card_lo=2, card_hi=6)
    codes, dims = ordinal_encode(d.data)
    reqs.append(Request(k + 1, "discrete", 300, 100000, 0.05, 3, 0.0, codes=torch.from_numpy(codes).pin_memory(),
                        dims=dims))
    assert int(dims.max()) == 6
    return reqs


def test_cfg5_shapes_served_equal_plain(cfg5_requests):
    from gpucsl_gb300.serve import SkeletonServer, serve_plain
    from gpucsl_gb300.synthetic import poisson_arrivals

    trace = poisson_arrivals(cfg5_requests, rate=200.0, seed=5)
    plain = {r.rid: r for r in serve_plain(trace)}
    served = SkeletonServer(budget_bytes=120e9, exclusive_backlog=-1).serve(trace)
    assert len(served) == len(trace)
    for r in served:
        q = plain[r.rid]
        assert r.kind == q.kind
        assert np.array_equal(r.skeleton, q.skeleton), r.rid
        assert np.array_equal(r.sepsets, q.sepsets), r.rid
        assert np.array_equal(r.pmax, q.pmax), r.rid
