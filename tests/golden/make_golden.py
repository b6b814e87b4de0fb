"""Generate tests/golden/reference_helpers.json from the reference's own code.

The reference's host-compilable helpers (math_helpers.cu, set_helpers.cu,
gaussian_helpers.cu of hpi-epic/gpucsl) are compiled in place by oracle/build.py into
oracle/_ref/libref_helpers.so; this script calls them on fixed inputs and stores the
outputs (doubles as float.hex strings, exact).  Run it where the reference checkout is
present:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as ct
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import cbind  # noqa: E402


def main() -> None:
    R = cbind.ref_lib()
    if R is None:
        raise SystemExit("reference helpers not buildable here (reference sources absent)")
    out: dict = {"source": "hpi-epic/gpucsl gpucsl/pc/cuda/helpers/{math,set,gaussian}_helpers.cu via oracle/ref_shim.cc"}

    out["binomial"] = [[n, k, int(R.ref_binomial(n, k))] for n in range(0, 26) for k in range(0, 9)]

    xs = [0.0, 1e-3, 0.1, 0.2, 0.5, 1.0, 2.0, 3.0, 5.0, 10.0, 20.0, 39.0, 40.5, 41.0, 50.0, 77.7, 100.0,
          250.0, 1000.0, 2500.0]
    dfs = [0, 1, 2, 3, 4, 5, 7, 10, 16, 25, 50, 99, 100, 255, 500, 2000]
    out["pchisq"] = [[x.hex(), d, float(R.ref_pchisq(x, d)).hex()] for x in xs for d in dfs]
    zs = [-7.0, -6.0, -5.99, -3.0, -2.5, -2.0, -1.5, -1.0, -0.999, -0.5, -1e-3, 0.0, 1e-3, 0.5, 1.0, 1.7, 2.0,
          4.2, 5.99, 6.0, 9.0]
    out["poz"] = [[z.hex(), float(R.ref_poz(z)).hex()] for z in zs]

    unr = []
    buf = (ct.c_int * 8)()
    for K in (5, 8, 12):
        for L in (1, 2, 3, 4):
            if K < L:
                continue
            from math import comb

            for r in range(comb(K, L)):
                R.ref_sepset_indices(L, K, r, ct.addressof(buf))
                unr.append([K, L, r, [int(buf[i]) for i in range(L)]])
    out["unrank"] = unr

    rng = np.random.default_rng(20240611)
    p = int(R.ref_pin_p())
    cases = []
    for c in range(24):
        A = rng.standard_normal((4 * p, p)) @ np.diag(rng.uniform(0.5, 2.0, p))
        A[:, 1:] += 0.6 * A[:, :-1]
        C = np.corrcoef(A, rowvar=False)
        Cc = np.ascontiguousarray(C, dtype=np.float64)
        for level in range(1, 7):
            for _ in range(3):
                vs = rng.choice(p, size=level + 2, replace=False)
                vi, vj = int(vs[0]), int(vs[1])
                S = np.sort(vs[2:]).astype(np.int32)
                Sbuf = (ct.c_int * level)(*[int(s) for s in S])
                z = R.ref_gaussian_ci_test(level, vi, vj, Cc.ctypes.data, ct.addressof(Sbuf))
                cases.append({"case": c, "level": level, "vi": vi, "vj": vj, "S": [int(s) for s in S],
                              "z": float(z).hex()})
        out.setdefault("corr_matrices", []).append([float(x).hex() for x in Cc.ravel()])
    out["gaussian_ci_test"] = {"p": p, "tests": cases}

    m2 = []
    for level in range(1, 7):
        for _ in range(4):
            B = rng.standard_normal((level + 3, level))
            M = np.corrcoef(B, rowvar=False) if level > 1 else np.array([[1.0]])
            M = np.ascontiguousarray(np.atleast_2d(M), dtype=np.float64)
            res = np.zeros(level * level)
            R.ref_m2_inv(level, M.ctypes.data, res.ctypes.data)
            m2.append({"level": level, "M": [float(x).hex() for x in M.ravel()],
                       "inv": [float(x).hex() for x in res]})
    out["m2_inv"] = m2

    path = Path(__file__).with_name("reference_helpers.json")
    path.write_text(json.dumps(out, indent=0))
    print(f"wrote {path} ({path.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
