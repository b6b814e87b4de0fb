"""Gaussian skeleton parity: GPU (C ABI) vs the FP64 oracle on seeded workloads.

Bar: skeleton bit-exact, sepsets identical (canonical enumeration order), pmax within
1e-9 relative of the oracle's FP64 evaluation, canonical test counts identical.  The
oracle's smallest decision margin |Z - tau| / tau is asserted to be far above FP64
rounding, so the bit-exact comparison is meaningful."""
import numpy as np
import pytest

from gpucsl_gb300.synthetic import gaussian_dag_data
from oracle import gaussian as og

pytestmark = pytest.mark.gpu

PMAX_RTOL = 1e-9


def run_gpu(torch, C, n, alpha, max_level, dense=False):
    from gpucsl_gb300 import engine

    thr = og.thresholds(n, alpha)
    s = engine.GaussianSolver(C.shape[0], max_level, dense_sepsets=dense)
    st = s.run(torch.from_numpy(np.ascontiguousarray(C)).cuda(), n, thr)
    G, sep, pmax = s.to_host()
    dense_sep = s.sep_dense.cpu().numpy() if dense and s.sep_dense is not None else None
    return G, sep, pmax, st, dense_sep


def assert_parity(G, sep, pmax, st, ref, margin_floor=1e-9):
    for lv in ref.levels:
        assert lv.min_margin > margin_floor, f"decision within FP64 noise at level {lv.level}"
    assert (G == ref.skeleton).all(), int((G != ref.skeleton).sum())
    assert sep.shape == ref.sepsets.shape
    assert (sep == ref.sepsets).all()
    iu = np.triu_indices(G.shape[0], 1)
    a, b = pmax[iu], ref.pmax[iu]
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    ok = (rel <= PMAX_RTOL) | (np.abs(a - b) <= 1e-300)
    assert ok.all(), float(rel.max())
    assert (pmax[np.tril_indices(G.shape[0])] == -1).all()
    # canonical executed tests and removals per level
    assert st.raw["levels_run"] == len(ref.levels)
    for lv in ref.levels:
        assert st.raw["tests"][lv.level] == lv.tests_canonical, lv
        assert st.raw["removed"][lv.level] == lv.removed, lv
        if lv.level > 0:
            assert st.raw["tests_full"][lv.level] == lv.tests_full, lv
            assert st.raw["edges"][lv.level] == lv.edges, lv


@pytest.mark.parametrize("seed,p,n,deg,alpha,L", [
    (1, 20, 1000, 2, 0.05, 3),      # the 20-variable, 1000-sample workload
    (3, 40, 500, 3, 0.05, 6),
    (4, 60, 2000, 4, 0.01, 10),
    (5, 12, 300, 5, 0.2, 10),       # dense: deep levels, the shared-memory kernel (l > 8)
])
def test_gaussian_parity(cuda, seed, p, n, deg, alpha, L):
    w = gaussian_dag_data(p, n, deg, seed)
    C = og.corrcoef(w.data)
    ref = og.skeleton(C, n, alpha, L)
    G, sep, pmax, st, _ = run_gpu(cuda, C, n, alpha, L)
    assert_parity(G, sep, pmax, st, ref)


def test_dense_sepsets_match_records(cuda):
    w = gaussian_dag_data(30, 800, 3, 9)
    C = og.corrcoef(w.data)
    G, sep, pmax, st, dense = run_gpu(cuda, C, 800, 0.05, 4, dense=True)
    assert (dense == sep).all()


def test_gaussian_parity_large(cuda):
    """p = 1000, n = 10000, alpha = 0.01, run to termination (the at-scale workload)."""
    w = gaussian_dag_data(1000, 10000, 3, 2)
    C = og.corrcoef(w.data)
    ref = og.skeleton(C, 10000, 0.01, 998)
    G, sep, pmax, st, _ = run_gpu(cuda, C, 10000, 0.01, 998)
    assert_parity(G, sep, pmax, st, ref)


def test_correlation_kernel_matches_numpy(cuda):
    torch = cuda
    from gpucsl_gb300 import engine

    for (p, n, dt) in [(20, 1000, np.float64), (257, 3001, np.float64), (130, 777, np.float32), (1, 5, np.float64)]:
        w = gaussian_dag_data(p, n, 2, p + n)
        X = w.data.astype(dt)
        C = engine.correlation(torch.from_numpy(X).cuda(), method="dfma").cpu().numpy()
        ref = np.corrcoef(X, rowvar=False) if p > 1 else np.array([[1.0]])
        assert np.allclose(C, np.atleast_2d(ref), rtol=0, atol=5e-14), float(np.abs(C - ref).max())
        assert (C <= 1).all() and (C >= -1).all()


def test_skeleton_from_gpu_correlation_matches_oracle(cuda):
    torch = cuda
    from gpucsl_gb300 import engine

    w = gaussian_dag_data(200, 5000, 3, 21)
    Cg = engine.correlation(torch.from_numpy(w.data).cuda())
    ref = og.skeleton(og.corrcoef(w.data), 5000, 0.01, 198)
    thr = og.thresholds(5000, 0.01)
    s = engine.GaussianSolver(200, 198)
    st = s.run(Cg, 5000, thr)
    G, sep, pmax = s.to_host()
    assert_parity(G, sep, pmax, st, ref, margin_floor=1e-8)


def test_determinism_repeat(cuda):
    w = gaussian_dag_data(150, 3000, 4, 31)
    C = og.corrcoef(w.data)
    outs = [run_gpu(cuda, C, 3000, 0.05, 148)[:3] for _ in range(3)]
    for o in outs[1:]:
        assert (o[0] == outs[0][0]).all() and (o[1] == outs[0][1]).all()
        assert np.array_equal(o[2], outs[0][2])


def test_repeated_solves_replay_level_graphs(cuda):
    """Repeated solves of one solver.  With GCSL_LEVEL_GRAPHS=1 the first launches its
    level batches directly, the second captures them into CUDA graphs and later ones
    replay the graphs (run by test_level_graphs_in_a_subprocess); without it every solve
    launches directly.  Every solve gives the oracle's skeleton, sepsets, test counts and
    pmax, and launches the same number of kernels (graph replays counted per kernel)."""
    from gpucsl_gb300 import _lib, engine

    torch = cuda
    w = gaussian_dag_data(400, 5000, 4, 37)
    C = og.corrcoef(w.data)
    ref = og.skeleton(C, 5000, 0.01, 398)
    Cg = torch.from_numpy(C).cuda()
    thr = og.thresholds(5000, 0.01)
    s = engine.GaussianSolver(400, 398, record_cap=400 * 400 * 4)  # no pool growth between solves
    L = _lib.lib()
    counts = []
    for _ in range(4):
        k0 = int(L.gcsl_kernel_launches())
        st = s.run(Cg, 5000, thr)
        counts.append(int(L.gcsl_kernel_launches()) - k0)
        G, sep, pmax = s.to_host()
        assert_parity(G, sep, pmax, st, ref)
    assert counts[2] == counts[0] and counts[3] == counts[0], counts


def test_level_graphs_in_a_subprocess(cuda):
    """The repeated-solve test above with level-batch graphs switched on (the switch is
    read once per process)."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    here = Path(__file__).resolve()
    env = dict(os.environ, GCSL_LEVEL_GRAPHS="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "gpu",
                        f"{here}::test_repeated_solves_replay_level_graphs"], capture_output=True, text=True,
                       env=env, cwd=here.parents[1], timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


def test_edge_cases(cuda):
    # two variables, max_level 0 (sepsets of shape (p, p, 0))
    w = gaussian_dag_data(2, 100, 1, 3)
    C = og.corrcoef(w.data)
    ref = og.skeleton(C, 100, 0.05, 0)
    G, sep, pmax, st, _ = run_gpu(cuda, C, 100, 0.05, 0)
    assert sep.shape == (2, 2, 0)
    assert (G == ref.skeleton).all() and np.allclose(pmax, ref.pmax, rtol=1e-12)
    # duplicate columns: r = 1 gives Z = inf at level 0 (edge kept) and singular blocks later
    rng = np.random.default_rng(0)
    X = rng.standard_normal((400, 6))
    X[:, 5] = X[:, 0]
    C = og.corrcoef(X)
    ref = og.skeleton(C, 400, 0.05, 4)
    G, sep, pmax, st, _ = run_gpu(cuda, C, 400, 0.05, 4)
    assert (G == ref.skeleton).all()
    # fully independent data: everything removed at level 0, loop stops
    X = rng.standard_normal((5000, 30))
    C = og.corrcoef(X)
    ref = og.skeleton(C, 5000, 0.001, 28)
    G, sep, pmax, st, _ = run_gpu(cuda, C, 5000, 0.001, 28)
    assert_parity(G, sep, pmax, st, ref)
