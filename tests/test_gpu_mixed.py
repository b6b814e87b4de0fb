"""The FP32-first level tests (default) against FP64 tests throughout
(GCSL_F64_TESTS=1, read once per process, so that run is a subprocess): skeleton,
sepsets, pmax and per-level test counts must be bit-identical, because every decision
taken in FP32 has a bound that clears the FP64 knife edge and every test whose bound can
hold the z* minimum is re-evaluated in FP64."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

CASES = [(1000, 10000, 3, 2, 0.01, 998), (300, 2000, 4, 8, 0.05, 12), (120, 500, 3, 9, 0.2, 12)]

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
def test_mixed_equals_fp64(cuda, tmp_path, case):
    outs = {}
    for mode in ("mixed", "f64"):
        out = str(tmp_path / f"{mode}.npz")
        env = dict(os.environ)
        env.pop("GCSL_F64_TESTS", None)
        if mode == "f64":
            env["GCSL_F64_TESTS"] = "1"
        r = subprocess.run([sys.executable, "-c", SOLVE.format(root=str(ROOT), case=case, out=out)], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs[mode] = np.load(out)
    a, b = outs["mixed"], outs["f64"]
    assert np.array_equal(a["C"], b["C"])
    assert np.array_equal(a["G"], b["G"])
    assert np.array_equal(a["sep"], b["sep"])
    assert np.array_equal(a["tests"], b["tests"])
    assert np.array_equal(a["pm"], b["pm"]), float(np.abs(a["pm"] - b["pm"]).max())
