"""Continuous-batching server: every response equals the plain single-problem result of
the same request (alone and in the mix), under a generous and a one-request budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def requests(cuda):
    from gpucsl_gb300.synthetic import serving_requests

    return serving_requests(12, seed=3, g_p=(10, 150), g_n=(500, 3000), d_p=(8, 30), d_n=(2000, 6000))


def by_rid(resp):
    return {r.rid: r for r in resp}


def assert_same(a, b):
    assert a.kind == b.kind
    assert np.array_equal(a.skeleton, b.skeleton), a.rid
    assert np.array_equal(a.sepsets, b.sepsets), a.rid
    assert np.array_equal(a.pmax, b.pmax), a.rid


def test_batched_serving_equals_plain(requests):
    from gpucsl_gb300.serve import SkeletonServer, serve_plain
    from gpucsl_gb300.synthetic import poisson_arrivals

    trace = poisson_arrivals(requests, rate=400.0)
    plain = by_rid(serve_plain(trace))
    # exclusive_backlog=-1: every request goes to the concurrent engines
    served = SkeletonServer(budget_bytes=120e9, exclusive_backlog=-1).serve(trace)
    assert len(served) == len(trace)
    assert max(r.batch for r in served) >= 1
    assert "exclusive" not in {r.path for r in served}
    for r in served:
        assert_same(r, plain[r.rid])
        assert r.done >= r.admitted >= r.arrival - 1e-9


def test_exclusive_without_backlog_then_batching(requests):
    from dataclasses import replace

    from gpucsl_gb300.serve import SkeletonServer, serve_plain

    # the first request arrives alone (solved exclusively); the rest arrive together
    # later, a backlog beyond exclusive_backlog, and go to the concurrent engines
    trace = [replace(r, arrival=0.0 if i == 0 else 0.25) for i, r in enumerate(requests)]
    plain = by_rid(serve_plain(trace))
    # inline host part (default) and host part on a finishing thread
    for overlap in (False, True):
        served = SkeletonServer(budget_bytes=120e9, exclusive_backlog=2, overlap_host=overlap).serve(trace)
        assert len(served) == len(trace)
        paths = {r.rid: r.path for r in served}
        assert paths[trace[0].rid] == "exclusive"
        assert "batched" in paths.values()
        for r in served:
            assert_same(r, plain[r.rid])


def test_all_at_once_batches_every_gaussian_request(requests):
    from gpucsl_gb300.serve import SkeletonServer, serve_plain
    from gpucsl_gb300.synthetic import poisson_arrivals

    trace = poisson_arrivals(requests, rate=1e9)  # everything arrives at once
    served = SkeletonServer(budget_bytes=120e9).serve(trace)
    g = [r for r in served if r.kind == "gaussian"]
    assert g and max(r.batch for r in g) > 1
    plain = by_rid(serve_plain(trace))
    for r in served:
        assert_same(r, plain[r.rid])


def test_tiny_budget_serialises_and_keeps_results(requests):
    from gpucsl_gb300.serve import SkeletonServer, serve_plain
    from gpucsl_gb300.synthetic import poisson_arrivals

    trace = poisson_arrivals(requests, rate=1e9)
    served = SkeletonServer(budget_bytes=1).serve(trace)
    assert all(r.batch == 1 for r in served)
    plain = by_rid(serve_plain(trace))
    for r in served:
        assert_same(r, plain[r.rid])
