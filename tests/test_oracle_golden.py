"""Pin the oracle (CPU restatement) against the reference's own golden vectors and
against the reference's helpers' outputs recorded in tests/golden/reference_helpers.json.
CPU only."""
import ctypes as ct
import itertools
from math import comb

import numpy as np
import pytest

import golden_data as gd
from oracle import cbind
from oracle import gaussian as og


def test_binomial_golden():
    for n, k, v in gd.BINOMIAL_GOLDEN:
        assert cbind.binomial(n, k) == v


def test_binomial_reference_grid():
    for n, k, v in gd.reference_helpers()["binomial"]:
        assert cbind.binomial(n, k) == v, (n, k)


def test_pchisq_golden():
    for x, df, expect in gd.PCHISQ_GOLDEN:
        assert gd.float_eq(cbind.pchisq(x, df), expect), (x, df)


def test_pchisq_matches_reference_bit_for_bit():
    # same algorithm, same operation order, both compiled without FP contraction
    for xh, df, vh in gd.reference_helpers()["pchisq"]:
        x, v = gd.h2f(xh), gd.h2f(vh)
        got = cbind.pchisq(x, df)
        assert got == v or abs(got - v) <= 1e-15 * abs(v), (x, df, got, v)


def test_poz_matches_reference():
    for zh, vh in gd.reference_helpers()["poz"]:
        assert cbind.poz(gd.h2f(zh)) == gd.h2f(vh)


def test_unrank_golden_3_of_5():
    for r, expect in enumerate(gd.UNRANK_3_OF_5):
        assert list(cbind.unrank(5, 3, r)) == expect
    BT = og.binom_table(5, 3)
    pos = og.unrank_batched(np.full(10, 5), np.arange(10), 3, BT)
    assert pos.tolist() == gd.UNRANK_3_OF_5


def test_unrank_matches_reference_and_itertools():
    for K, L, r, expect in gd.reference_helpers()["unrank"]:
        assert list(cbind.unrank(K, L, r)) == expect
    for K in range(1, 11):
        for L in range(1, min(K, 5) + 1):
            combos = list(itertools.combinations(range(1, K + 1), L))
            BT = og.binom_table(K, L)
            pos = og.unrank_batched(np.full(len(combos), K), np.arange(len(combos)), L, BT)
            assert [tuple(x) for x in pos.tolist()] == combos


def test_compact_golden():
    assert (cbind.compact(gd.COMPACT_IN) == gd.COMPACT_OUT).all()
    assert (og.compact(gd.COMPACT_IN) == gd.COMPACT_OUT).all()
    full = np.ones((6, 6), np.uint16)
    assert (cbind.compact(full) == gd.COMPACT_FULL_OUT).all()


def test_alg7_known_answers():
    # tests/test_cuda_gaussian_helpers.py:248-299
    a = np.array([[1, 2, 3], [5, 2, 2], [1, 6, 1]], np.float64)
    assert np.allclose(og.m2_inv_batched(a[None])[0], np.linalg.pinv(a))
    b = np.array([[5, 3, 4], [3, 4, 5], [6, 3, 2]], np.float64)
    assert np.allclose(og.inverse_gauss_jordan_batched(b[None])[0], np.linalg.inv(b))
    c = np.array([[4.2, 12.3, -16.4], [12.3, 37.3, -43.3], [-16.4, -43.5, 98.6]], np.float64)
    assert np.allclose(og.cholesky_batched(c[None])[0], np.linalg.cholesky(c))


def test_m2_inv_matches_reference():
    for case in gd.reference_helpers()["m2_inv"]:
        L = case["level"]
        M = np.array([gd.h2f(x) for x in case["M"]]).reshape(L, L)
        ref = np.array([gd.h2f(x) for x in case["inv"]]).reshape(L, L)
        got = og.m2_inv_batched(M[None])[0]
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-13)


def test_gaussian_ci_z_matches_reference():
    g = gd.reference_helpers()
    p = g["gaussian_ci_test"]["p"]
    mats = [np.array([gd.h2f(x) for x in m]).reshape(p, p) for m in g["corr_matrices"]]
    worst = 0.0
    for t in g["gaussian_ci_test"]["tests"]:
        C = mats[t["case"]]
        S = np.array([t["S"]], np.int64)
        z = og.gaussian_ci_z(C, np.array([t["vi"]]), np.array([t["vj"]]), S)[0]
        zc = og.gaussian_ci_z_cholesky(C, np.array([t["vi"]]), np.array([t["vj"]]), S)[0]
        ref = gd.h2f(t["z"])
        worst = max(worst, abs(z - ref) / max(abs(ref), 1e-300))
        assert abs(z - ref) <= 1e-12 * max(1.0, abs(ref)), (t, z, ref)
        assert abs(zc - ref) <= 1e-9 * max(1.0, abs(ref)), (t, zc, ref)
    assert worst < 1e-12


def test_contingency_level0_crosstab():
    # tests/test_cuda_discrete_helpers.py:20-41
    a = np.array([0, 1, 2, 3, 4, 5, 1, 2, 3, 4, 5, 6], np.uint8)
    b = np.array([0, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0], np.uint8)
    data = np.stack([a, b])  # column-major: 2 columns of 12
    dims = np.array([7, 2], np.uint8)
    counts = np.zeros(14, np.uint32)
    cbind.lib().orc_contingency(cbind.ptr(data), 12, 12, cbind.ptr(dims), 0, 1, None, 0, cbind.ptr(counts))
    expect = np.zeros((7, 2), np.uint32)
    for x, y in zip(a, b):
        expect[x, y] += 1
    assert (counts.reshape(7, 2) == expect).all()


def test_contingency_level_n_layout():
    data, expected = gd.level_n_contingency_case()
    col = np.ascontiguousarray(data.T.astype(np.uint8))
    dims = np.full(4, 5, np.uint8)
    S = np.array([0, 1], np.int32)
    counts = np.zeros(5 ** 4, np.uint32)
    cbind.lib().orc_contingency(cbind.ptr(col), 100, 100, cbind.ptr(dims), 2, 3, cbind.ptr(S), 2,
                                cbind.ptr(counts))
    assert (counts == expected.ravel()).all()


def test_chi2_formula():
    N, chi = gd.chi2_formula_case()
    tab = np.ascontiguousarray(N.astype(np.uint32))
    got = cbind.lib().orc_chi2_level_n(cbind.ptr(tab), 5, 5, 5)
    assert abs(got - chi) <= 1e-10


def test_thresholds_formula():
    thr = og.thresholds(1000, 0.05)
    from scipy.stats import norm

    q = abs(norm.ppf(0.025))
    assert thr[0] == pytest.approx(q / np.sqrt(1000 - 4), rel=1e-15)
    assert thr[3] == pytest.approx(q / np.sqrt(1000 - 7), rel=1e-15)
    assert thr[47] > 0 and thr[48] == 0.0 and thr[49] == 0.0  # range(1, 49) fills 0..47
    small = og.thresholds(10, 0.05)  # min(50, 7) - 1 = 6 -> entries 0..4
    assert all(v > 0 for v in small[:5]) and all(v == 0 for v in small[5:])


def test_ref_lib_pins_when_available():
    R = cbind.ref_lib()
    if R is None:
        pytest.skip("reference sources not present on this machine")
    rng = np.random.default_rng(5)
    for _ in range(2000):
        x = float(rng.uniform(0, 300))
        df = int(rng.integers(0, 400))
        assert cbind.pchisq(x, df) == R.ref_pchisq(x, df)
    buf = (ct.c_int * 6)()
    for K in range(6, 15):
        for L in range(1, 5):
            for r in range(0, comb(K, L), 7):
                R.ref_sepset_indices(L, K, r, ct.addressof(buf))
                assert list(cbind.unrank(K, L, r)) == [buf[i] for i in range(L)]


def test_oracle_process_pool_matches_serial():
    """The oracle's level loop split over spawned processes gives the serial answer:
    same skeleton, sepsets, pmax and per-level test counts."""
    from gpucsl_gb300.synthetic import gaussian_dag_data

    C = og.corrcoef(gaussian_dag_data(60, 800, 3.0, seed=5).data)
    a = og.skeleton(C, 800, 0.05, 4)
    b = og.skeleton(C, 800, 0.05, 4, workers=2)
    assert np.array_equal(a.skeleton, b.skeleton)
    assert np.array_equal(a.sepsets, b.sepsets)
    assert np.array_equal(a.pmax, b.pmax)
    assert [s.tests_canonical for s in a.levels] == [s.tests_canonical for s in b.levels]


def test_reference_kernel_host_sizing():
    """Host-side sizing of the reference-kernel baseline: the discrete working memory is
    find_execution_specification's figure (4 bytes x (D^l D^2 + 2 D^l D + D^l) x p x p x 2
    parallel tests, largest over levels), and the ordinal codes are per-column ranks of
    the distinct values with dims = largest code + 1 (a constant column has dims 1)."""
    from oracle import ref_gpu

    assert ref_gpu.disc_working_memory_bytes(200, 5, 3) == 4 * (125 * 25 + 2 * 125 * 5 + 125) * 200 * 200 * 2
    assert ref_gpu.disc_working_memory_bytes(24, 5, 1) == 4 * (5 * 25 + 2 * 5 * 5 + 5) * 24 * 24 * 2
    X = np.array([[7, 3, 9], [2, 3, 9], [7, 3, 4], [5, 3, 9]], dtype=np.uint8)
    codes, dims = ref_gpu.ordinal_encode(X)
    assert codes.shape == (3, 4) and codes.dtype == np.uint8
    assert codes[0].tolist() == [2, 0, 2, 1] and codes[1].tolist() == [0, 0, 0, 0] and codes[2].tolist() == [1, 1, 0, 1]
    assert dims.tolist() == [3, 1, 2]


def test_reference_kernel_instantiation_lists():
    """The translation units oracle/build.py compiles for the reference's kernels: every
    level 0..L instantiated once, with the names oracle/ref_gpu.py looks up."""
    from oracle import build as ob

    g = ob.ref_gauss_instantiations(1000, 10)
    assert g.startswith('#include "gaussian_ci.cu"')
    assert g.count("gaussian_ci_level_0<0, 1000, 10>") == 1
    for l in range(1, 11):
        assert g.count(f"gaussian_ci_level_n<{l}, 1000, 10>") == 1
    assert "gaussian_ci_level_n<11," not in g and "compact<1000, 1000u>" in g
    d = ob.ref_disc_instantiations(200, 50000, 5, 3)
    assert "#define __global__ __device__" in d and '#include "discrete_ci.cu"' in d
    for l in range(4):
        assert d.count(f'extern "C" __global__ void ref_disc_level_{l}(') == 1
        body = "discrete_ci_level_0" if l == 0 else "discrete_ci_level_n"
        assert f"{body}<{l}, 200, 2, 5, 50000, 3>" in d
    assert 'extern "C" __global__ void ref_compact(' in d
