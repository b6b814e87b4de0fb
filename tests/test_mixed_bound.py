"""CPU mirror of the FP32-first CI test with its running error bound
(gpucsl_gb300/csrc/gauss_dev.cuh: gauss_test_f32b, f32_rho2_bound): on random
correlation submatrices (well and badly conditioned), whenever the bound is usable
the FP64 partial correlation rho^2 lies inside r +- e.  FP32 rounding is emulated per
operation with numpy float32; a fused multiply-add is the exact float64 product-sum
rounded once to float32."""
import numpy as np

U = np.float32(5.9604645e-08)
f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def rho2_bound(h00, e00, h01, e01, h11, e11):
    lo00, lo11 = f32(h00 - e00), f32(h11 - e11)
    rho2 = f32(f32(h01 * h01) / f32(h00 * h11))
    ah = abs(h01)
    err = f32(2) * (f32(f32(2) * ah * e01 + e01 * e01) / f32(lo00 * lo11) + rho2 * (e00 / lo00 + e11 / lo11)
                    + f32(4) * U * rho2)
    ok = bool(e00 < f32(0.25) * h00 and e11 < f32(0.25) * h11 and rho2 + err < f32(0.98))
    return rho2, f32(err), ok


def f32b_mirror(C, vi, vj, S):
    L = len(S)
    c = C.astype(np.float32)
    if L == 1:
        s = S[0]
        m, a, b, r = c[s, s], c[vi, s], c[vj, s], c[vi, vj]
        em, ea, eb, er = U * abs(m), U * abs(a), U * abs(b), U * abs(r)
        d00, d11 = fma(-a, a, m), fma(-b, b, m)
        e00 = em + f32(2) * abs(a) * ea + U * abs(d00)
        e11 = em + f32(2) * abs(b) * eb + U * abs(d11)
        ab = f32(a * b)
        eab = abs(a) * eb + abs(b) * ea + U * abs(ab)
        n01 = fma(r, m, -ab)
        e01 = abs(m) * er + abs(r) * em + eab + U * abs(n01)
        return rho2_bound(d00, e00, n01, e01, d11, e11)
    idx = list(S) + [vi, vj]
    D = L + 2
    A = np.array([[c[idx[i], idx[k]] for k in range(D)] for i in range(D)], dtype=np.float32)
    A[L, L] = 1.0
    A[L + 1, L + 1] = 1.0
    E = (U * np.abs(A)).astype(np.float32)
    ok = True
    for j in range(L):
        piv, ep = A[j, j], E[j, j]
        ok = ok and ep < f32(0.25) * piv
        inv = f32(f32(1) / piv)
        einv = f32(ep * inv * inv * f32(1.5) + U * abs(inv))
        for i in range(j + 1, D):
            aij = A[i, j]
            t = f32(aij * inv)
            et = f32(abs(aij) * einv + abs(inv) * E[i, j] + U * abs(t))
            for k in range(j + 1, i + 1):
                akj = A[k, j]
                v = fma(-t, akj, A[i, k])
                E[i, k] = f32(E[i, k] + abs(t) * E[k, j] + abs(akj) * et + U * abs(v))
                A[i, k] = v
    r, e, ok2 = rho2_bound(A[L, L], E[L, L], A[L + 1, L], E[L + 1, L], A[L + 1, L + 1], E[L + 1, L + 1])
    return r, e, ok and ok2


def rho2_f64(C, vi, vj, S):
    idx = list(S)
    M = C[np.ix_(idx, idx)]
    B = C[np.ix_([vi, vj], idx)]
    H = C[np.ix_([vi, vj], [vi, vj])] - B @ np.linalg.solve(M, B.T)
    return H[0, 1] ** 2 / (abs(H[0, 0]) * abs(H[1, 1]))


def corr_from(X):
    C = np.corrcoef(X, rowvar=False)
    np.fill_diagonal(C, 1.0)
    return C


@np.errstate(all="ignore")  # degenerate draws give NaN bounds, which are rejected
def test_bound_encloses_fp64_rho2():
    rng = np.random.default_rng(5)
    checked = 0
    for trial in range(60):
        p = int(rng.integers(6, 16))
        n = int(rng.integers(20, 400))
        X = rng.standard_normal((n, p))
        if trial % 3 == 1:  # near-collinear columns: large conditioning
            X[:, 1] = X[:, 0] + 10 ** rng.uniform(-4, -1) * rng.standard_normal(n)
        if trial % 3 == 2:  # strongly dependent chain
            for k in range(1, p):
                X[:, k] += 0.9 * X[:, k - 1]
        C = corr_from(X)
        for _ in range(40):
            L = int(rng.integers(1, min(7, p - 1)))
            vs = rng.choice(p, size=L + 2, replace=False)
            vi, vj, S = int(vs[0]), int(vs[1]), [int(x) for x in sorted(vs[2:])]
            r, e, ok = f32b_mirror(C, vi, vj, S)
            if not ok:
                continue
            exact = rho2_f64(C, vi, vj, S)
            assert abs(float(r) - exact) <= float(e), (trial, L, float(r), exact, float(e))
            checked += 1
    assert checked > 1000
