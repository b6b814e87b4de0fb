"""The reference's own Gaussian kernels (gaussian_ci.cu, compiled unchanged for sm_103a
into oracle/_ref/ by oracle/build.py) run on the GPU with the reference's launch
geometry and level loop: their skeleton equals the oracle's, and every separation set
they record removes its edge under the oracle's CI test.  This pins the baseline that
bench.py's reference arm times beside the CPU port."""
import numpy as np
import pytest

from oracle import gaussian as og

pytestmark = pytest.mark.gpu

CASES = [(20, 1000, 2.0, 1, 0.05, 3), (1000, 10000, 3.0, 2, 0.01, 10)]


@pytest.mark.parametrize("p,n,deg,seed,alpha,L", CASES)
def test_reference_kernels_skeleton_equals_oracle(p, n, deg, seed, alpha, L):
    import torch

    from gpucsl_gb300.synthetic import gaussian_dag_data
    from oracle import ref_gpu

    try:
        K = ref_gpu.RefGaussianKernels(p, L)
    except ref_gpu.RefGpuUnavailable as e:
        pytest.skip(str(e))
    C = og.corrcoef(gaussian_dag_data(p, n, deg, seed).data)
    want = og.skeleton(C, n, alpha, L)
    thr = og.thresholds(n, alpha)
    bufs = K.alloc()
    levels = K.run(torch.from_numpy(np.ascontiguousarray(C)).cuda(), thr, bufs)
    torch.cuda.synchronize()
    G = bufs["G"].cpu().numpy() != 0
    assert levels == len(want.levels)
    assert np.array_equal(G, want.skeleton != 0)

    # each separation set the reference recorded for a removed edge separates it under
    # the oracle's test at that set's level
    sep = bufs["sep"].cpu().numpy().reshape(p, p, L)
    iu, ju = np.nonzero(np.triu(~G & (sep[:, :, 0] >= 0), 1))
    for a, b in list(zip(iu, ju))[:200]:
        S = sep[a, b][sep[a, b] >= 0]
        assert list(sep[b, a][sep[b, a] >= 0]) == list(S)
        z = og.gaussian_ci_z(C, np.array([a]), np.array([b]), S[None, :].astype(np.int64))[0]
        assert z < thr[len(S)], (a, b, S, z)


DCASES = [(24, 4000, 2.0, 5, 0.05, 3), (200, 50000, 2.0, 3, 0.05, 3)]


@pytest.mark.parametrize("p,n,deg,seed,alpha,L", DCASES)
def test_reference_discrete_kernels_skeleton_equals_oracle(p, n, deg, seed, alpha, L):
    """discrete_ci.cu on the GPU: skeleton equal to the C oracle's, and each separation
    set it records gives p >= alpha under the oracle's test."""
    import ctypes as ct

    import torch

    from gpucsl_gb300.synthetic import discrete_bn_data
    from oracle import cbind, ref_gpu

    codes, dims = ref_gpu.ordinal_encode(discrete_bn_data(p, n, deg, seed).data)
    try:
        K = ref_gpu.RefDiscreteKernels(p, n, int(dims.max()), L)
    except ref_gpu.RefGpuUnavailable as e:
        pytest.skip(str(e))
    Go = np.zeros((p, p), np.uint16)
    sepo = np.full((p, p, L), -1, np.int32)
    pmo = np.zeros((p, p))
    st = cbind.OrcStats()
    cbind.lib().orc_discrete_skeleton(cbind.ptr(codes), n, n, p, cbind.ptr(dims), alpha, L, cbind.ptr(Go),
                                      cbind.ptr(sepo), cbind.ptr(pmo), 0, ct.byref(st))
    bufs = K.alloc(codes, dims)
    K.run(alpha, bufs)
    torch.cuda.synchronize()
    G = bufs["G"].cpu().numpy() != 0
    assert np.array_equal(G, Go != 0), int((G != (Go != 0)).sum())

    sep = bufs["sep"].cpu().numpy().reshape(p, p, L)
    work = np.zeros(int(dims.max()) ** (L + 2) + 4, np.uint32)
    iu, ju = np.nonzero(np.triu(~G & (sep[:, :, 0] >= 0), 1))
    for a, b in list(zip(iu, ju))[:200]:
        S = np.ascontiguousarray(sep[a, b][sep[a, b] >= 0]).astype(np.int32)
        assert list(sep[b, a][sep[b, a] >= 0]) == list(S)
        pv = cbind.lib().orc_discrete_test(cbind.ptr(codes), n, n, cbind.ptr(dims), int(a), int(b), cbind.ptr(S),
                                           len(S), cbind.ptr(work), None)
        assert pv >= alpha, (a, b, S, pv)
