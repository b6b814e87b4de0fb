"""Loader of the committed golden fixtures (reference outputs and the reference's own
test vectors, tests/test_cuda_*.py and tests/cuda/helper_test.cc of hpi-epic/gpucsl)."""
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=1)
def reference_helpers() -> dict:
    return json.loads((HERE / "reference_helpers.json").read_text())


def h2f(s: str) -> float:
    return float.fromhex(s)


# tests/cuda/helper_test.cc:10-17
BINOMIAL_GOLDEN = [(2, 3, 0), (3, 2, 3), (5, 2, 10), (20, 10, 184756), (30, 20, 30045015), (30, 30, 1)]
# tests/cuda/helper_test.cc:25-31 (EXPECT_FLOAT_EQ: within 4 float ulps)
PCHISQ_GOLDEN = [(3, 2, 0.22313016014842982), (20, 10, 0.02925268807696113), (0, 1, 1.0),
                 (10, 10, 0.4404932850652121), (0.2, 3, 0.9775892977616494)]
# tests/test_cuda_set_helpers.py:21-34: all 3-subsets of 5 positions, lexicographic
UNRANK_3_OF_5 = [[1, 2, 3], [1, 2, 4], [1, 2, 5], [1, 3, 4], [1, 3, 5], [1, 4, 5], [2, 3, 4], [2, 3, 5],
                 [2, 4, 5], [3, 4, 5]]
# tests/test_cuda_graph_helpers.py:18-46
COMPACT_IN = np.array([[0, 1, 1, 0, 0, 1], [1, 0, 1, 0, 1, 0], [0, 0, 0, 0, 0, 0], [1, 1, 1, 0, 1, 1],
                       [1, 0, 1, 0, 0, 1], [0, 1, 1, 1, 0, 0]], np.uint16)
COMPACT_OUT = np.array([[3, 1, 2, 5, 0, 0], [3, 0, 2, 4, 0, 0], [0, 0, 0, 0, 0, 0], [5, 0, 1, 2, 4, 5],
                        [3, 0, 2, 5, 0, 0], [3, 1, 2, 3, 0, 0]], np.int32)
# tests/test_cuda_graph_helpers.py:49-70
COMPACT_FULL_OUT = np.array([[5, 1, 2, 3, 4, 5], [5, 0, 2, 3, 4, 5], [5, 0, 1, 3, 4, 5], [5, 0, 1, 2, 4, 5],
                             [5, 0, 1, 2, 3, 5], [5, 0, 1, 2, 3, 4]], np.int32)


def float_eq(a: float, b: float, ulps: int = 4) -> bool:
    """googletest EXPECT_FLOAT_EQ: both values as float32, within 4 ulps."""
    fa, fb = np.float32(a), np.float32(b)
    if fa == fb:
        return True
    ia = np.array([fa]).view(np.int32)[0]
    ib = np.array([fb]).view(np.int32)[0]
    return abs(int(ia) - int(ib)) <= ulps


def level_n_contingency_case():
    """tests/test_cuda_discrete_helpers.py:44-83: seed 1, 100 rows of 4 variables in 0..4;
    S = [0, 1], v_i = 2, v_j = 3; expected layout counts[x1][x0][x2][x3]."""
    np.random.seed(1)
    data = np.random.randint(0, 5, size=(100, 4))
    expected = np.zeros((5, 5, 5, 5))
    for row in data:
        expected[row[1], row[0], row[2], row[3]] += 1
    return data, expected


def chi2_formula_case():
    """tests/test_cuda_discrete_helpers.py:128-172: seed 1 table, reference triple loop."""
    import itertools

    np.random.seed(1)
    N = np.random.randint(1, 100, size=(5, 5, 5))
    npp = np.zeros(5)
    nip = np.zeros((5, 5))
    npj = np.zeros((5, 5))
    for s, vi, vj in itertools.product(range(5), repeat=3):
        v = N[s, vi, vj]
        npp[s] += v
        nip[s, vi] += v
        npj[s, vj] += v
    chi = 0.0
    for s, vi, vj in itertools.product(range(5), repeat=3):
        o = N[s, vi, vj]
        e = nip[s, vi] * npj[s, vj] / npp[s]
        chi += (o - e) * (o - e) / e
    return N, chi
