"""Host side of the drop-in API, CPU only: argument checks (the reference's
pc_validations.py), the threshold table (helpers.py:42-50), the pmax post-processing
(helpers.py:85-101), the start graph, the timing wrapper and the record-pool scatter into
the reference's dense sepset layout."""
import logging
import math

import numpy as np
import pytest
from scipy.stats import norm

from gpucsl_gb300 import engine
from gpucsl_gb300.pc import helpers, pc_validations as v


def test_determine_max_level():
    data = np.zeros((100, 7))
    assert v.determine_max_level(None, data) == 5
    assert v.determine_max_level(3, data) == 3
    assert v.determine_max_level(0, data) == 0


def test_determine_max_level_clamps_with_a_warning(caplog):
    with caplog.at_level(logging.WARNING):
        assert v.determine_max_level(40, np.zeros((10, 4))) == 2
    assert "biggest possible level is 2" in caplog.text


def test_determine_max_level_of_one_variable_is_an_error():
    with pytest.raises(v.GpucslError):
        v.determine_max_level(None, np.zeros((10, 1)))


@pytest.mark.parametrize("alpha", [-0.01, 1.01])
def test_alpha_out_of_range(alpha):
    with pytest.raises(v.GpucslError):
        v.validate_alpha(alpha)


@pytest.mark.parametrize("alpha", [0.0, 0.05, 1.0])
def test_alpha_in_range(alpha):
    v.validate_alpha(alpha)


def test_devices():
    v.validate_given_devices([0], None)
    v.validate_given_devices([0], 0)
    with pytest.raises(v.GpucslError):
        v.validate_given_devices([0, 1], None)
    with pytest.raises(v.GpucslError):
        v.validate_given_devices([0], 1)


@pytest.mark.parametrize("n,alpha", [(1000, 0.05), (10000, 0.01), (30, 0.05), (5, 0.05)])
def test_thresholds(n, alpha):
    t = helpers.get_gaussian_thresholds(np.zeros((n, 3)), alpha)
    assert len(t) == 50
    q = abs(norm.ppf(alpha / 2))
    covered = max(min(50, n - 3) - 2, 0)
    for l in range(50):
        if l < covered:
            assert t[l] == pytest.approx(q / math.sqrt(n - l - 4), rel=1e-15)
        else:
            assert t[l] == 0.0


def test_pmax_transform_and_postprocess():
    z = np.array([[0.0, 0.1, 0.5], [0.1, 0.0, 2.0], [0.5, 2.0, 0.0]])
    pm = helpers.transform_to_pmax(z, 103)
    assert pm[0, 1] == pytest.approx(2 * norm.sf(10 * 0.1), rel=1e-14)
    assert pm[1, 2] == pytest.approx(2 * norm.sf(10 * 2.0), rel=1e-14)
    out = helpers.postprocess_pmax(pm.copy())
    assert (out[np.tril_indices(3)] == -1).all()
    assert out[0, 2] == pm[0, 2]


def test_start_graph_and_timed():
    G = helpers.init_pc_graph(np.zeros((4, 6)))
    assert G.shape == (6, 6) and G.dtype == np.uint16 and (G == 1).all()
    r = helpers.timed(lambda a, b=1: a + b)(2, b=3)
    assert isinstance(r, helpers.TimedReturn) and r.result == 5 and r.runtime >= 0.0
    assert helpers.get_max_neighbor_count(np.array([[2, 1, 3], [0, 0, 0], [3, 0, 1]])) == 3


def test_records_to_dense():
    # records [lo, hi, level, S...]: (1, 4) at level 2 by {0, 2}; (0, 3) at level 1 by {2};
    # a record above max_level is dropped
    rec = np.array([1, 4, 2, 0, 2, 0, 3, 1, 2, 2, 3, 3, 0, 1, 4, 99], np.int32)
    out = engine.records_to_dense(rec, 15, 5, 2)
    assert out.shape == (5, 5, 2)
    assert out[1, 4].tolist() == [0, 2] and out[4, 1].tolist() == [0, 2]
    assert out[0, 3].tolist() == [2, -1] and out[3, 0].tolist() == [2, -1]
    assert (out[2, 3] == -1).all()
    assert int((out >= 0).sum()) == 6
    # more record ints announced than given (an overflowed pool): refused, never read past
    with pytest.raises(ValueError):
        engine.records_to_dense(rec[:9], 15, 5, 2)


def _dense_by_loop(rec, n_ints, p, max_level):
    out = np.full((p, p, max_level), -1, np.int32)
    k = 0
    while k < n_ints:
        lo, hi, lev = int(rec[k]), int(rec[k + 1]), int(rec[k + 2])
        if lev <= max_level:
            out[lo, hi, :lev] = rec[k + 3:k + 3 + lev]
            out[hi, lo, :lev] = rec[k + 3:k + 3 + lev]
        k += 3 + lev
    return out


def test_records_to_dense_matches_a_record_by_record_walk():
    """The vectorised scatter (record offsets by pointer doubling) equals a walk over the
    records one by one, on random pools of mixed levels, some above max_level."""
    rng = np.random.default_rng(5)
    for trial in range(20):
        p, L = int(rng.integers(2, 60)), int(rng.integers(1, 6))
        recs = []
        pairs = [(a, b) for a in range(p) for b in range(a + 1, p)]
        for k in rng.permutation(len(pairs))[:int(rng.integers(0, 300))]:  # one record per pair
            lev = int(rng.integers(1, L + 3))
            lo, hi = pairs[k]
            recs += [lo, hi, lev] + rng.integers(0, p, lev).tolist()
        rec = np.array(recs + [7, 7, 7], np.int32)  # trailing words past n_ints are ignored
        n = len(recs)
        assert np.array_equal(engine.records_to_dense(rec, n, p, L), _dense_by_loop(rec, n, p, L)), trial
