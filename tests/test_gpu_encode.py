"""Device ordinal encoding (gcsl_ordinal_encode) against the host encoder
(engine.ordinal_encode, the OrdinalEncoder semantics of discover_skeleton_discrete.py:38-49)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint8, np.float64])
def test_device_encoding_matches_host(cuda, dtype):
    from gpucsl_gb300 import engine

    torch = cuda
    rng = np.random.default_rng(7)
    n, p = 3001, 45
    cols = []
    for j in range(p):
        k = int(rng.integers(1, 9))
        vals = np.sort(rng.choice(200, size=k, replace=False)) - (40 if dtype != np.uint8 and j % 3 == 0 else 0)
        vals = vals if dtype != np.uint8 else np.abs(vals)
        cols.append(rng.choice(vals, size=n))
    data = np.stack(cols, axis=1).astype(dtype)
    codes, dims = engine.ordinal_encode(data)
    cdev, ddev = engine.ordinal_encode_device(torch.from_numpy(data).cuda())
    assert np.array_equal(ddev.cpu().numpy(), dims)
    assert np.array_equal(cdev.cpu().numpy()[:, :n], codes)


def test_device_encoding_rejects_unsupported(cuda):
    from gpucsl_gb300 import _lib, engine

    torch = cuda
    wide = np.arange(600, dtype=np.int64).reshape(300, 2)  # 300 distinct values per column
    with pytest.raises(_lib.GcslError):
        engine.ordinal_encode_device(torch.from_numpy(wide).cuda())
    spread = np.array([[0, 1], [5000, 2]], dtype=np.int64)  # range above 4096
    with pytest.raises(_lib.GcslError):
        engine.ordinal_encode_device(torch.from_numpy(spread).cuda())
    frac = np.array([[0.5, 1.0], [1.0, 2.0]])
    with pytest.raises(_lib.GcslError):
        engine.ordinal_encode_device(torch.from_numpy(frac).cuda())


def test_discrete_driver_uses_device_encoding(cuda):
    from gpucsl_gb300.pc.discover_skeleton_discrete import discover_skeleton_gpu_discrete
    from gpucsl_gb300.synthetic import discrete_bn_data
    from gpucsl_gb300 import engine

    d = discrete_bn_data(25, 4000, 2, 9)
    data = d.data.astype(np.int64) * 3 - 7  # gaps and negative values: same codes
    (res, _) = discover_skeleton_gpu_discrete(np.ones((25, 25), np.uint16), data, 0.05, 2, 25, 4000)
    codes, dims = engine.ordinal_encode(d.data)
    ds = engine.DiscreteSolver(25, 4000, 2, int(dims.max()))
    ds.load(codes, dims)
    ds.run(0.05)
    G, sep, pm = ds.to_host()
    assert np.array_equal(res.skeleton, G) and np.array_equal(res.seperation_sets, sep)  # reference spelling
    assert np.array_equal(res.pmax, pm)


def test_device_encoding_boundaries(cuda):
    """255 distinct values pass and 256 do not; a constant column has dims 1; values far
    from zero (a small range around 10^15) and a single sample encode like the host."""
    from gpucsl_gb300 import _lib, engine

    torch = cuda
    rng = np.random.default_rng(3)
    n = 700
    c255 = rng.permutation(np.arange(n) % 255)
    const = np.full(n, 42)
    far = 10**15 + rng.integers(0, 7, n)
    data = np.stack([c255, const, far], axis=1).astype(np.int64)
    codes, dims = engine.ordinal_encode(data)
    cdev, ddev = engine.ordinal_encode_device(torch.from_numpy(data).cuda())
    assert list(ddev.cpu().numpy()) == [255, 1, int(dims[2])]
    assert np.array_equal(cdev.cpu().numpy()[:, :n], codes)
    c256 = (np.arange(n) % 256).astype(np.int64).reshape(-1, 1)
    with pytest.raises(_lib.GcslError):
        engine.ordinal_encode_device(torch.from_numpy(c256).cuda())
    one = np.array([[3, 9, 0]], dtype=np.int64)
    cdev, ddev = engine.ordinal_encode_device(torch.from_numpy(one).cuda())
    assert list(ddev.cpu().numpy()) == [1, 1, 1] and cdev.cpu().numpy()[:, 0].tolist() == [0, 0, 0]
