"""The bounds-checked build (is_debug) on the GPU.

The reference compiles its kernels with -G -lineinfo when is_debug is set
(kernel_management.py:32-33); here is_debug selects libgpucsl_gb300_debug.so, the same
kernels with every derived index checked before use (a failed check returns
GCSL_ERR_DEBUG_CHECK with the failing site instead of trapping) and a permutable work
order.  The tests run tiny cases exhaustively (p <= 8, every level) against the oracle
with no check firing, and show that permuting the order in which warps and blocks take
their work (edges, units of chunked edges, discrete tests) changes no result: run twice
and under shuffled orders, the outputs equal the release build's bit for bit."""
import ctypes as ct

import numpy as np
import pytest

from gpucsl_gb300.synthetic import discrete_bn_data, gaussian_dag_data
from oracle import cbind
from oracle import gaussian as og

pytestmark = pytest.mark.gpu


def gauss_solve(torch, C, n, alpha, max_level, debug):
    from gpucsl_gb300 import engine

    s = engine.GaussianSolver(C.shape[0], max_level, debug=debug)
    st = s.run(torch.from_numpy(np.ascontiguousarray(C)).cuda(), n, og.thresholds(n, alpha))
    return (*s.to_host(), st)


def disc_solve(codes, dims, n, alpha, max_level, debug):
    from gpucsl_gb300 import engine

    p = codes.shape[0]
    s = engine.DiscreteSolver(p, n, max_level, int(dims.max()), debug=debug)
    s.load(codes, dims)
    st = s.run(alpha)
    return (*s.to_host(), st)


def test_debug_build_small_gaussian_cases_every_level(cuda):
    for seed in range(16):
        p, n = 3 + seed % 6, 300
        w = gaussian_dag_data(p, n, 2.0 + 0.5 * (seed % 3), 500 + seed)
        C = og.corrcoef(w.data)
        ref = og.skeleton(C, n, 0.05, p - 2)
        G, sep, pmax, st = gauss_solve(cuda, C, n, 0.05, p - 2, debug=True)
        assert st.raw["status"] == 0 and st.raw["debug_site"] == 0, (seed, st.raw["status"], st.raw["debug_site"])
        assert (G == ref.skeleton).all() and (sep == ref.sepsets).all(), seed
        assert st.tests == ref.tests_canonical, seed
        iu = np.triu_indices(p, 1)
        rel = np.abs(pmax[iu] - ref.pmax[iu]) / np.maximum(np.abs(ref.pmax[iu]), 1e-300)
        assert (rel <= 1e-9).all(), (seed, float(rel.max()))


def test_debug_build_small_discrete_cases_every_level(cuda):
    from gpucsl_gb300 import engine

    for seed in range(12):
        p, n = 3 + seed % 6, 500
        d = discrete_bn_data(p, n, 2, 700 + seed)
        codes, dims = engine.ordinal_encode(d.data)
        L = max(p - 2, 0)
        G, sep, pmax, st = disc_solve(codes, dims, n, 0.05, L, debug=True)
        assert st.raw["status"] == 0 and st.raw["debug_site"] == 0, (seed, st.raw["status"], st.raw["debug_site"])
        Go = np.zeros((p, p), np.uint16)
        sepo = np.full((p, p, L), -1, np.int32)
        pmo = np.zeros((p, p))
        ost = cbind.OrcStats()
        cbind.lib().orc_discrete_skeleton(cbind.ptr(codes), n, n, p, cbind.ptr(dims), 0.05, L, cbind.ptr(Go),
                                          cbind.ptr(sepo), cbind.ptr(pmo), 1, ct.byref(ost))
        pmo[np.tril_indices(p)] = -1
        assert (G == Go).all() and (sep == sepo).all(), seed
        assert np.allclose(pmax, pmo, rtol=1e-9, atol=0), seed


def test_shuffled_work_order_changes_nothing(cuda):
    """Release build once; debug build twice in the release order and under two shuffled
    orders: identical skeleton, sepsets, pmax and test counts (Gaussian with chunked
    edges, and discrete)."""
    from gpucsl_gb300 import engine

    w = gaussian_dag_data(150, 3000, 4, 31)
    C = og.corrcoef(w.data)
    base = gauss_solve(cuda, C, 3000, 0.05, 148, debug=False)
    for seed in (0, 0, 1, 12345):
        with engine.debug_work_order(seed):
            got = gauss_solve(cuda, C, 3000, 0.05, 148, debug=True)
        assert got[3].raw["status"] == 0, seed
        for a, b in zip(got[:3], base[:3]):
            assert np.array_equal(a, b), seed
        assert got[3].raw["tests"] == base[3].raw["tests"], seed

    d = discrete_bn_data(40, 5000, 2, 33)
    codes, dims = engine.ordinal_encode(d.data)
    base = disc_solve(codes, dims, 5000, 0.05, 3, debug=False)
    for seed in (0, 7, 99991):
        with engine.debug_work_order(seed):
            got = disc_solve(codes, dims, 5000, 0.05, 3, debug=True)
        assert got[3].raw["status"] == 0, seed
        for a, b in zip(got[:3], base[:3]):
            assert np.array_equal(a, b), seed


def test_public_api_is_debug_selects_the_checked_build(cuda):
    from gpucsl_gb300.pc.discover_skeleton_gaussian import discover_skeleton_gpu_gaussian

    w = gaussian_dag_data(40, 2000, 3, 35)
    skel = np.ones((40, 40), np.uint16)
    a = discover_skeleton_gpu_gaussian(skel, w.data, None, 0.05, 6, 40, 2000, is_debug=True).result
    b = discover_skeleton_gpu_gaussian(skel, w.data, None, 0.05, 6, 40, 2000, is_debug=False).result
    assert np.array_equal(a.skeleton, b.skeleton)
    assert np.array_equal(a.seperation_sets, b.seperation_sets)
    assert np.array_equal(a.pmax, b.pmax)
