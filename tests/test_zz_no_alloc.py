"""gcsl_gauss_skeleton_noalloc: the allocation-free Gaussian skeleton entry point.

It exists for callers that cannot call cudaMalloc (for example a host runtime whose
allocator owns all device memory after start-up); its scratch space is a static device
array inside the library.  This test calls it through the C ABI twice in a row (so the
second call runs on the scratch contents the first one left) on two different problems,
and compares every output with the workspace entry point gcsl_gauss_skeleton: skeleton
and sepset records bit-exact, pmax within the 1e-9 relative tolerance of the parity
tests.  The file is named to be collected last."""
import ctypes as ct

import numpy as np
import pytest

from gpucsl_gb300.synthetic import gaussian_dag_data
from oracle import gaussian as og

pytestmark = pytest.mark.gpu


def _solve(torch, C_np, n, alpha, max_level, noalloc: bool):
    from gpucsl_gb300 import _lib, engine

    L = _lib.lib()
    p = C_np.shape[0]
    C = torch.from_numpy(np.ascontiguousarray(C_np)).cuda()
    G = torch.empty((p, p), dtype=torch.int16, device="cuda")
    pmax = torch.empty((p, p), dtype=torch.float64, device="cuda")
    rec = torch.empty(p * 64, dtype=torch.int32, device="cuda")
    thr_list = og.thresholds(n, alpha)
    thr = (ct.c_double * len(thr_list))(*thr_list)
    st = _lib.GcslStats()
    if noalloc:
        rc = L.gcsl_gauss_skeleton_noalloc(C.data_ptr(), p, n, thr, len(thr_list), max_level, G.data_ptr(), None,
                                           rec.data_ptr(), rec.numel(), pmax.data_ptr(), ct.byref(st),
                                           _lib.stream_ptr())
    else:
        ws = torch.empty(int(L.gcsl_gauss_workspace_bytes(p, max_level)), dtype=torch.uint8, device="cuda")
        rc = L.gcsl_gauss_skeleton(C.data_ptr(), p, n, thr, len(thr_list), max_level, G.data_ptr(), None,
                                   rec.data_ptr(), rec.numel(), pmax.data_ptr(), ct.byref(st), ws.data_ptr(),
                                   ws.numel(), _lib.stream_ptr())
    _lib.check(rc, "noalloc" if noalloc else "workspace")
    torch.cuda.synchronize()
    nrec = int(st.n_records)
    sep = engine.records_to_dense(rec[:nrec].cpu().numpy(), nrec, p, max_level)
    return G.cpu().numpy().view(np.uint16), sep, pmax.cpu().numpy(), st.as_dict()


def _compare(a, b):
    Ga, sa, pa, sta = a
    Gb, sb, pb, stb = b
    assert (Ga == Gb).all()
    assert (sa == sb).all()
    iu = np.triu_indices(Ga.shape[0], 1)
    rel = np.abs(pa[iu] - pb[iu]) / np.maximum(np.abs(pb[iu]), 1e-300)
    assert ((rel <= 1e-9) | (np.abs(pa[iu] - pb[iu]) <= 1e-300)).all()
    assert sta["tests"] == stb["tests"] and sta["levels_run"] == stb["levels_run"]


def test_noalloc_matches_workspace_entry_point_twice(cuda):
    torch = cuda
    cases = [gaussian_dag_data(300, 4000, 3, 41), gaussian_dag_data(120, 2500, 4, 42)]
    for w in cases:  # two calls in a row, different sizes: the second reuses the scratch
        C = og.corrcoef(w.data)
        n = w.data.shape[0]
        ref = _solve(torch, C, n, 0.01, 8, noalloc=False)
        got = _solve(torch, C, n, 0.01, 8, noalloc=True)
        _compare(got, ref)
    # and once more on the first problem after the smaller one left its contents behind
    C = og.corrcoef(cases[0].data)
    _compare(_solve(torch, C, 4000, 0.01, 8, noalloc=True), _solve(torch, C, 4000, 0.01, 8, noalloc=False))


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    torch = cuda
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    p = 513  # GCSL_NOALLOC_MAX_P + 1
    C = torch.eye(p, dtype=torch.float64, device="cuda")
    G = torch.empty((p, p), dtype=torch.int16, device="cuda")
    pmax = torch.empty((p, p), dtype=torch.float64, device="cuda")
    thr = (ct.c_double * 50)(*og.thresholds(1000, 0.05))
    rc = L.gcsl_gauss_skeleton_noalloc(C.data_ptr(), p, 1000, thr, 50, 2, G.data_ptr(), None, None, 0,
                                       pmax.data_ptr(), None, _lib.stream_ptr())
    assert rc == _lib.GCSL_ERR_UNSUPPORTED
