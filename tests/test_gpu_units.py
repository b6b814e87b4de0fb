"""Single-kernel parity on the GPU, mirroring the reference's CUDA unit tests
(tests/test_cuda_graph_helpers.py, test_cuda_set_helpers.py, test_cuda_discrete_helpers.py,
tests/cuda/helper_test.cc), through the C ABI."""
import ctypes as ct

import numpy as np
import pytest

import golden_data as gd
from oracle import cbind

pytestmark = pytest.mark.gpu


def _L():
    from gpucsl_gb300 import _lib

    return _lib


def test_compact_golden(cuda):
    torch = cuda
    lib = _L()
    G = torch.from_numpy(gd.COMPACT_IN.astype(np.int16)).cuda()
    adj = torch.zeros((6, 6), dtype=torch.int32, device="cuda")
    lib.check(lib.lib().gcsl_compact(G.data_ptr(), 6, adj.data_ptr(), lib.stream_ptr()), "compact")
    assert (adj.cpu().numpy() == gd.COMPACT_OUT).all()
    G = torch.ones((6, 6), dtype=torch.int16, device="cuda")
    adj.zero_()
    lib.check(lib.lib().gcsl_compact(G.data_ptr(), 6, adj.data_ptr(), lib.stream_ptr()), "compact")
    assert (adj.cpu().numpy() == gd.COMPACT_FULL_OUT).all()


def test_compact_random_large_matches_oracle(cuda):
    torch = cuda
    lib = _L()
    rng = np.random.default_rng(7)
    p = 1500
    G = (rng.random((p, p)) < 0.3).astype(np.uint16)
    adj = torch.full((p, p), -7, dtype=torch.int32, device="cuda")
    lib.check(lib.lib().gcsl_compact(torch.from_numpy(G.view(np.int16)).cuda().data_ptr(), p, adj.data_ptr(),
                                     lib.stream_ptr()), "compact")
    got = adj.cpu().numpy()
    ref = cbind.compact(G)
    deg = ref[:, 0]
    assert (got[:, 0] == deg).all()
    for r in range(p):
        assert (got[r, 1:1 + deg[r]] == ref[r, 1:1 + deg[r]]).all()


def test_unrank_golden_and_reference(cuda):
    torch = cuda
    lib = _L()
    out = torch.zeros(10 * 3, dtype=torch.int32, device="cuda")
    lib.check(lib.lib().gcsl_unrank(5, 3, 10, out.data_ptr(), lib.stream_ptr()), "unrank")
    assert out.view(10, 3).cpu().numpy().tolist() == gd.UNRANK_3_OF_5
    by = {}
    for K, L, r, expect in gd.reference_helpers()["unrank"]:
        by.setdefault((K, L), {})[r] = expect
    for (K, L), ranks in by.items():
        n = len(ranks)
        out = torch.zeros(n * L, dtype=torch.int32, device="cuda")
        lib.check(lib.lib().gcsl_unrank(K, L, n, out.data_ptr(), lib.stream_ptr()), "unrank")
        got = out.view(n, L).cpu().numpy()
        for r in range(n):
            assert got[r].tolist() == ranks[r]


def test_unrank_large_k_matches_oracle(cuda):
    torch = cuda
    lib = _L()
    for K, L in [(146, 1), (146, 2), (60, 3), (30, 5), (24, 8), (20, 12)]:
        from math import comb

        total = comb(K, L)
        ranks = np.unique(np.concatenate([np.arange(min(total, 300)), np.linspace(0, total - 1, 300).astype(np.int64)]))
        n = int(ranks.max()) + 1
        n = min(n, 200000)
        out = torch.zeros(n * L, dtype=torch.int32, device="cuda")
        lib.check(lib.lib().gcsl_unrank(K, L, n, out.data_ptr(), lib.stream_ptr()), "unrank")
        got = out.view(n, L).cpu().numpy()
        for r in ranks[ranks < n]:
            assert got[r].tolist() == list(cbind.unrank(K, L, int(r))), (K, L, r)


def test_pchisq_matches_reference_values(cuda):
    torch = cuda
    lib = _L()
    rows = gd.reference_helpers()["pchisq"]
    x = torch.tensor([gd.h2f(r[0]) for r in rows], dtype=torch.float64, device="cuda")
    df = torch.tensor([r[1] for r in rows], dtype=torch.int64, device="cuda")
    out = torch.empty_like(x)
    lib.check(lib.lib().gcsl_pchisq(x.data_ptr(), df.data_ptr(), len(rows), out.data_ptr(), lib.stream_ptr()), "pchisq")
    got = out.cpu().numpy()
    for g, r in zip(got, rows):
        ref = gd.h2f(r[2])
        assert abs(g - ref) <= 1e-12 * abs(ref) + 1e-300, (r, g, ref)
    for (xx, d, expect) in gd.PCHISQ_GOLDEN:
        xt = torch.tensor([float(xx)], dtype=torch.float64, device="cuda")
        dt = torch.tensor([d], dtype=torch.int64, device="cuda")
        o = torch.empty_like(xt)
        lib.lib().gcsl_pchisq(xt.data_ptr(), dt.data_ptr(), 1, o.data_ptr(), lib.stream_ptr())
        assert gd.float_eq(float(o.item()), expect)


def test_pchisq_random_vs_oracle(cuda):
    torch = cuda
    lib = _L()
    rng = np.random.default_rng(11)
    n = 4000
    xs = np.concatenate([rng.uniform(0, 50, n // 2), rng.uniform(0, 5000, n // 2)])
    dfs = rng.integers(0, 3000, n)
    x = torch.from_numpy(xs).cuda()
    df = torch.from_numpy(dfs.astype(np.int64)).cuda()
    out = torch.empty_like(x)
    lib.check(lib.lib().gcsl_pchisq(x.data_ptr(), df.data_ptr(), n, out.data_ptr(), lib.stream_ptr()), "pchisq")
    got = out.cpu().numpy()
    ref = np.array([cbind.pchisq(a, b) for a, b in zip(xs, dfs)])
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    assert np.all((rel <= 1e-9) | (np.abs(got - ref) <= 1e-300)), float(rel.max())


def _disc_table(torch, data_cols, n, dims, vi, vj, S):
    lib = _L()
    p = data_cols.shape[0]
    ld = (n + 15) // 16 * 16
    buf = np.zeros((p, ld), np.uint8)
    buf[:, :n] = data_cols
    d = torch.from_numpy(buf).cuda()
    dm = torch.from_numpy(np.asarray(dims, np.uint8)).cuda()
    dims_i = [int(d) for d in dims]  # Python ints: uint8 products would wrap
    dim_s = 1
    for s in S:
        dim_s *= dims_i[s]
    T = dim_s * dims_i[vi] * dims_i[vj]
    counts = torch.zeros(T, dtype=torch.int32, device="cuda")
    out2 = torch.zeros(2, dtype=torch.float64, device="cuda")
    Sarr = (ct.c_int32 * max(1, len(S)))(*[int(s) for s in S])
    lib.check(lib.lib().gcsl_disc_table(d.data_ptr(), ld, n, dm.data_ptr(), vi, vj, Sarr, len(S), counts.data_ptr(),
                                        T, out2.data_ptr(), lib.stream_ptr()), "disc_table")
    return counts.cpu().numpy().view(np.uint32), out2.cpu().numpy()


def test_contingency_level0_crosstab(cuda):
    a = np.array([0, 1, 2, 3, 4, 5, 1, 2, 3, 4, 5, 6], np.uint8)
    b = np.array([0, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0], np.uint8)
    counts, _ = _disc_table(cuda, np.stack([a, b]), 12, [7, 2], 0, 1, [])
    expect = np.zeros((7, 2), np.uint32)
    for x, y in zip(a, b):
        expect[x, y] += 1
    assert (counts.reshape(7, 2) == expect).all()


def test_contingency_level_n_layout(cuda):
    data, expected = gd.level_n_contingency_case()
    counts, _ = _disc_table(cuda, data.T.astype(np.uint8), 100, [5, 5, 5, 5], 2, 3, [0, 1])
    assert (counts == expected.ravel()).all()


@pytest.mark.parametrize("n", [1, 15, 16, 17, 1000, 50001])
@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_contingency_and_chi2_vs_oracle(cuda, n, level):
    rng = np.random.default_rng(100 + n + level)
    p = 6
    dims = rng.integers(2, 7, p).astype(np.uint8)
    cols = np.stack([rng.integers(0, dims[v], n) for v in range(p)]).astype(np.uint8)
    S = sorted(rng.choice(np.arange(2, p), size=level, replace=False).tolist())
    counts, out2 = _disc_table(cuda, cols, n, dims, 0, 1, S)
    ref_counts = np.zeros(counts.size, np.uint32)
    Sa = np.array(S if S else [0], np.int32)
    colc = np.ascontiguousarray(cols)
    dimc = np.ascontiguousarray(dims, dtype=np.uint8)
    cbind.lib().orc_contingency(cbind.ptr(colc), n, n, cbind.ptr(dimc), 0, 1,
                                cbind.ptr(Sa) if S else None, level, cbind.ptr(ref_counts))
    assert (counts == ref_counts).all()
    chi = ct.c_double()
    work = np.zeros(counts.size + 4, np.uint32)
    pv = cbind.lib().orc_discrete_test(cbind.ptr(colc), n, n, cbind.ptr(dimc), 0, 1,
                                       cbind.ptr(Sa) if S else None, level, cbind.ptr(work), ct.byref(chi))
    assert out2[0] == chi.value  # same operations in the same order
    assert abs(out2[1] - pv) <= 1e-12 * max(abs(pv), 1e-300)
