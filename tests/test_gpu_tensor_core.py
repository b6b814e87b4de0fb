"""tcgen05 building blocks on the GPU: the BF16 tensor-core GEMM against exact
integer products (small integers are exact in BF16 and their sums exact in FP32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(torch, A, B):
    from gpucsl_gb300 import _lib

    M, K = A.shape
    N = B.shape[0]
    Ad = torch.from_numpy(A.astype(np.float32)).to(torch.bfloat16).cuda().contiguous()
    Bd = torch.from_numpy(B.astype(np.float32)).to(torch.bfloat16).cuda().contiguous()
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(_lib.lib().gcsl_tc_gemm_bf16(Ad.data_ptr(), Bd.data_ptr(), D.data_ptr(), M, N, K, err.data_ptr(),
                                            _lib.stream_ptr()), "tc_gemm")
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "tensor-core completion wait timed out"
    return D.cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (128, 256, 4096)])
def test_tc_gemm_exact_integers(cuda, M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-3, 4, size=(M, K))
    B = rng.integers(-3, 4, size=(N, K))
    D = _gemm(cuda, A, B)
    ref = A.astype(np.int64) @ B.astype(np.int64).T
    assert np.array_equal(D.astype(np.int64), ref), float(np.abs(D - ref).max())


def test_tc_gemm_random_values(cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    A = rng.standard_normal((256, 1024)).astype(np.float32)
    B = rng.standard_normal((128, 1024)).astype(np.float32)
    Ab = torch.from_numpy(A).to(torch.bfloat16).float().numpy().astype(np.float64)
    Bb = torch.from_numpy(B).to(torch.bfloat16).float().numpy().astype(np.float64)
    D = _gemm(torch, Ab, Bb)
    ref = Ab @ Bb.T
    assert np.allclose(D, ref, rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("p,n,dt", [(20, 1000, np.float64), (257, 3001, np.float64), (1000, 10000, np.float64),
                                    (130, 777, np.float32), (64, 100000, np.float64)])
def test_tc_correlation_matches_numpy(cuda, p, n, dt):
    torch = cuda
    from gpucsl_gb300 import engine
    from gpucsl_gb300.synthetic import gaussian_dag_data

    w = gaussian_dag_data(p, n, 3, p * 7 + n)
    X = w.data.astype(dt)
    X[:, 0] += 1000.0  # a large mean: centring happens in FP64 before the split
    C = engine.correlation(torch.from_numpy(X).cuda(), method="tc").cpu().numpy()
    ref = np.corrcoef(X, rowvar=False)
    err = float(np.abs(C - ref).max())
    assert np.isfinite(C).all()
    assert err <= 1e-12, err


def test_tc_correlation_skeleton_parity(cuda):
    """p = 1000, n = 10000 skeleton from the tensor-core correlation matches the oracle."""
    torch = cuda
    from gpucsl_gb300 import engine
    from gpucsl_gb300.synthetic import gaussian_dag_data
    from oracle import gaussian as og

    w = gaussian_dag_data(1000, 10000, 3, 2)
    Cg = engine.correlation(torch.from_numpy(w.data).cuda(), method="tc")
    ref = og.skeleton(og.corrcoef(w.data), 10000, 0.01, 998)
    s = engine.GaussianSolver(1000, 998)
    st = s.run(Cg, 10000, og.thresholds(10000, 0.01))
    G, sep, pmax = s.to_host()
    assert (G == ref.skeleton).all()
    assert (sep == ref.sepsets).all()
    iu = np.triu_indices(1000, 1)
    rel = np.abs(pmax[iu] - ref.pmax[iu]) / np.maximum(np.abs(ref.pmax[iu]), 1e-300)
    assert ((rel <= 1e-9) | (np.abs(pmax[iu] - ref.pmax[iu]) <= 1e-300)).all(), float(rel.max())
    assert st.tests == ref.tests_canonical
