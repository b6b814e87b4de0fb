"""GPU edge orientation against the reference's own results (golden cases made by
tests/golden/make_orient_golden.py) and the sequential oracle on skeletons the GPU
skeleton solver produced, including PC.execute end to end."""
from pathlib import Path

import numpy as np
import pytest

from oracle import gaussian as og
from oracle import orient as oo

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "orient_cases.npz"


def test_gpu_orientation_matches_reference_cases(cuda):
    from gpucsl_gb300.orient import orient_matrix

    z = np.load(GOLD)
    for c in range(int(z["n"])):
        D, passes = orient_matrix(z[f"S{c}"], z[f"sep{c}"])
        assert np.array_equal(D, z[f"D{c}"]), c
        assert passes == oo.orient(z[f"S{c}"], z[f"sep{c}"])[1], c


@pytest.mark.parametrize("p,n,deg,seed,alpha,L", [(60, 2000, 3, 31, 0.05, 4), (200, 3000, 4, 32, 0.05, 6),
                                                   (400, 5000, 3, 33, 0.01, 8)])
def test_gpu_orientation_on_solver_output(cuda, p, n, deg, seed, alpha, L):
    from gpucsl_gb300 import engine
    from gpucsl_gb300.orient import orient_matrix
    from gpucsl_gb300.synthetic import gaussian_dag_data

    torch = cuda
    w = gaussian_dag_data(p, n, deg, seed)
    s = engine.GaussianSolver(p, L)
    C = engine.correlation(torch.from_numpy(w.data).cuda())
    s.run(C, n, engine.gaussian_thresholds(n, alpha))
    G, sep, _ = s.to_host()
    D, passes = orient_matrix(G, sep)
    ref, ref_passes = oo.orient(G, sep)
    assert np.array_equal(D, ref)
    assert passes == ref_passes


def test_pc_execute_orients_on_gpu(cuda):
    nx = pytest.importorskip("networkx")
    from gpucsl_gb300.pc.pc import GaussianPC
    from gpucsl_gb300.synthetic import gaussian_dag_data

    w = gaussian_dag_data(30, 1500, 2, 41)
    res, _ = GaussianPC(w.data, 3, 0.05).set_distribution_specific_options().execute()
    dag = res.directed_graph
    p = 30
    D = np.zeros((p, p), np.uint8)
    for a, b in dag.edges:
        D[a, b] = 1
    S = ((D + D.T) > 0).astype(np.uint8)
    ref, _ = oo.orient(S, res.separation_sets)
    assert np.array_equal(D, ref)
