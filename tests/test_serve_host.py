"""Host logic of the server (no GPU): admission accounting, footprints, arrivals."""
import numpy as np

from gpucsl_gb300.serve import _Admission, gaussian_footprint, latency_summary, Response


def test_admission_is_fifo_budgeted():
    a = _Admission(100)
    assert a.try_admit(60)
    assert not a.try_admit(50)      # would exceed the budget next to the first
    assert a.try_admit(40)
    a.release(60)
    assert a.try_admit(50)
    a.release(40)
    a.release(50)
    assert a.used == 0
    assert a.try_admit(10_000)      # larger than the budget: admitted alone
    assert not a.try_admit(1)


def test_gaussian_footprint_grows_with_size():
    small = gaussian_footprint(20, 1000, 3)
    big = gaussian_footprint(2000, 50000, 3)
    assert 0 < small < big
    # samples + 7 BF16 digit planes dominate: at least 18 bytes per sample value
    assert big >= 18 * 2000 * 50000


def test_poisson_arrivals_rate():
    from gpucsl_gb300.synthetic import poisson_arrivals
    from gpucsl_gb300.serve import Request

    reqs = [Request(k, "gaussian", 10, 100, 0.01, 3, 0.0) for k in range(4000)]
    tr = poisson_arrivals(reqs, rate=50.0, seed=1)
    t = np.array([r.arrival for r in tr])
    assert (np.diff(t) > 0).all()
    assert abs(len(t) / t[-1] - 50.0) < 5.0


def test_latency_summary():
    z = np.zeros((2, 2))
    resp = [Response(k, "gaussian", z, z, z, 0.1 * k, 0.1 * k, 0.1 * k + 0.05) for k in range(100)]
    s = latency_summary(resp)
    assert abs(s["p50_ms"] - 50.0) < 1e-6 and abs(s["p99_ms"] - 50.0) < 1e-6
