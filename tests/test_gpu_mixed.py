"""The FP32-first level tests (default) against FP64 tests throughout
(GCSL_F64_TESTS=1), and the chunked walk of long edges (default) against walking every
edge whole in one warp (GCSL_CHUNKED=0); both switches are read once per process, so
each run is a subprocess.  Skeleton, sepsets, pmax and per-level test counts must be
bit-identical: every decision taken in FP32 has a bound that clears the FP64 knife edge,
every test whose bound can hold the z* minimum is re-evaluated in FP64, and the chunk
combine picks the smallest removing key and folds exactly the keys before it."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

CASES = [(1000, 10000, 3, 2, 0.01, 998), (300, 2000, 4, 8, 0.05, 12), (120, 500, 3, 9, 0.2, 12),
         (200, 3000, 8, 5, 0.05, 12)]
MODES = {"mixed": {}, "f64": {"GCSL_F64_TESTS": "1"}, "whole": {"GCSL_CHUNKED": "0"},
         "whole_f64": {"GCSL_CHUNKED": "0", "GCSL_F64_TESTS": "1"}}

SOLVE = r"""
import json, sys, numpy as np, torch
sys.path.insert(0, {root!r})
from gpucsl_gb300 import engine
from gpucsl_gb300.synthetic import gaussian_dag_data
p, n, deg, seed, alpha, L = {case}
X = torch.from_numpy(gaussian_dag_data(p, n, deg, seed).data).cuda()
C = engine.correlation(X)
s = engine.GaussianSolver(p, min(L, p - 2))
st = s.run(C, n, engine.gaussian_thresholds(n, alpha))
G, sep, pm = s.to_host()
np.savez({out!r}, G=G, sep=sep, pm=pm, tests=np.array(st.raw["tests"]), C=C.cpu().numpy())
"""


@pytest.mark.parametrize("case", CASES)
def test_mixed_and_chunked_equal_fp64_whole(cuda, tmp_path, case):
    outs = {}
    for mode, extra in MODES.items():
        out = str(tmp_path / f"{mode}.npz")
        env = dict(os.environ)
        env.pop("GCSL_F64_TESTS", None)
        env.pop("GCSL_CHUNKED", None)
        env.update(extra)
        r = subprocess.run([sys.executable, "-c", SOLVE.format(root=str(ROOT), case=case, out=out)], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs[mode] = np.load(out)
    a = outs["mixed"]
    for mode in ("f64", "whole", "whole_f64"):
        b = outs[mode]
        assert np.array_equal(a["C"], b["C"]), mode
        assert np.array_equal(a["G"], b["G"]), mode
        assert np.array_equal(a["sep"], b["sep"]), mode
        assert np.array_equal(a["tests"], b["tests"]), mode
        assert np.array_equal(a["pm"], b["pm"]), (mode, float(np.abs(a["pm"] - b["pm"]).max()))


def test_precision_switch_in_process(cuda):
    """gcsl_set_test_precision: FP64 tests throughout on this thread give the FP32-first
    results bit for bit (same skeleton, sepsets, test counts, pmax)."""
    import torch

    from gpucsl_gb300 import engine
    from gpucsl_gb300.synthetic import gaussian_dag_data

    p, n = 300, 2000
    X = torch.from_numpy(gaussian_dag_data(p, n, 4, 8).data).cuda()
    C = engine.correlation(X)
    thr = engine.gaussian_thresholds(n, 0.05)
    s = engine.GaussianSolver(p, 12)
    with engine.test_precision("fp32_first"):
        a = s.run(C, n, thr)
        ra = s.to_host()
    with engine.test_precision("fp64"):
        b = s.run(C, n, thr)
        rb = s.to_host()
    assert a.raw["tests"] == b.raw["tests"]
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)
