"""The lane arithmetic the discrete kernels rely on, emulated in NumPy on the CPU.

* disc_test_kernel's packed path: with every code below its cardinality and a table of
  at most 256 cells, 32-bit multiply-adds on four samples' bytes give, lane by lane, the
  cell index ((sum_k s_k m_k) * di + a) * dj + b of the scalar formula (no carry between
  byte lanes).
* disc_validate_kernel's word test: for 1 <= d <= 128, ((x + (128 - d) * 0x01010101) | x)
  & 0x80808080 is non-zero exactly when some byte of x is >= d.

The GPU parity tests check the kernels themselves; this pins the reasoning behind them."""
import numpy as np

M32 = 0xFFFFFFFF


def _words(b: np.ndarray) -> np.ndarray:
    return b.view("<u4").astype(np.uint64)


def test_packed_cell_index_equals_scalar_formula():
    rng = np.random.default_rng(0)
    checked = 0
    while checked < 3000:
        L = int(rng.integers(0, 4))
        ds = [int(rng.integers(1, 9)) for _ in range(L)]
        di, dj = int(rng.integers(1, 17)), int(rng.integers(1, 17))
        T = int(np.prod(ds, dtype=np.int64)) * di * dj
        if T > 256:
            continue
        mult, m = [], 1
        for d in ds:
            mult.append(m)
            m *= d
        S = [rng.integers(0, d, 16).astype(np.uint8) for d in ds]
        a = rng.integers(0, di, 16).astype(np.uint8)
        b = rng.integers(0, dj, 16).astype(np.uint8)
        s4 = np.zeros(4, np.uint64)
        for k in range(L):
            s4 = (s4 + _words(S[k]) * mult[k]) & M32
        idx4 = (((s4 * di + _words(a)) & M32) * dj + _words(b)) & M32
        got = [(int(idx4[q >> 2]) >> (8 * (q & 3))) & 0xFF for q in range(16)]
        want = [(sum(int(S[k][q]) * mult[k] for k in range(L)) * di + int(a[q])) * dj + int(b[q]) for q in range(16)]
        assert got == want, (L, ds, di, dj)
        assert max(want) < T
        checked += 1


def test_word_range_check_is_exact():
    rng = np.random.default_rng(1)
    for _ in range(50000):
        d = int(rng.integers(1, 129))
        x = rng.integers(0, 256, 4).astype(np.uint8)
        w = int(x.view("<u4")[0])
        hit = (((w + (0x80 - d) * 0x01010101) & M32) | w) & 0x80808080
        assert (hit != 0) == bool((x >= d).any()), (d, x.tolist())
    # the edges: all bytes d - 1 pass, one byte d fails, bytes >= 128 fail
    for d in (1, 2, 5, 127, 128):
        ok = np.full(4, d - 1, np.uint8)
        w = int(ok.view("<u4")[0])
        assert ((((w + (0x80 - d) * 0x01010101) & M32) | w) & 0x80808080) == 0
        for pos in range(4):
            for bad_byte in (d, 255):
                x = ok.copy()
                x[pos] = bad_byte
                w = int(x.view("<u4")[0])
                assert ((((w + (0x80 - d) * 0x01010101) & M32) | w) & 0x80808080) != 0
