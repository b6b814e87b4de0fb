"""ORACLE — test infrastructure only. ctypes bindings of oracle/liboracle.so and of the
reference-helper shim oracle/_ref/libref_helpers.so (when built)."""
from __future__ import annotations

import ctypes as ct
from functools import lru_cache

import numpy as np

from . import build as _build

_i64 = ct.c_int64
_i32 = ct.c_int32
_dbl = ct.c_double
_vp = ct.c_void_p


class OrcStats(ct.Structure):
    _fields_ = [("levels_run", _i32), ("status", _i32),
                ("tests", _i64 * 64), ("removed", _i64 * 64)]


@lru_cache(maxsize=1)
def lib() -> ct.CDLL:
    path = _build.build_oracle()
    L = ct.CDLL(str(path))
    L.orc_binomial.restype = _i64
    L.orc_binomial.argtypes = [_i64, _i64]
    L.orc_unrank.restype = None
    L.orc_unrank.argtypes = [_i64, ct.c_int, _i64, _vp]
    L.orc_poz.restype = _dbl
    L.orc_poz.argtypes = [_dbl]
    L.orc_pchisq.restype = _dbl
    L.orc_pchisq.argtypes = [_dbl, _i64]
    L.orc_contingency.restype = None
    L.orc_contingency.argtypes = [_vp, _i64, _i64, _vp, _i32, _i32, _vp, ct.c_int, _vp]
    L.orc_chi2_level0.restype = _dbl
    L.orc_chi2_level0.argtypes = [_vp, ct.c_int, ct.c_int, _i64]
    L.orc_chi2_level_n.restype = _dbl
    L.orc_chi2_level_n.argtypes = [_vp, _i64, ct.c_int, ct.c_int]
    L.orc_discrete_test.restype = _dbl
    L.orc_discrete_test.argtypes = [_vp, _i64, _i64, _vp, _i32, _i32, _vp, ct.c_int, _vp, _vp]
    L.orc_compact.restype = None
    L.orc_compact.argtypes = [_vp, _i32, _vp]
    L.orc_discrete_skeleton.restype = ct.c_int
    L.orc_discrete_skeleton.argtypes = [_vp, _i64, _i64, _i32, _vp, _dbl, ct.c_int, _vp, _vp, _vp,
                                        ct.c_int, ct.POINTER(OrcStats)]
    return L


@lru_cache(maxsize=1)
def ref_lib():
    """The reference's own helpers compiled in place; None when not buildable here."""
    try:
        path = _build.build_ref()
    except Exception:
        path = None
    if path is None or not path.exists():
        return None
    L = ct.CDLL(str(path))
    L.ref_binomial.restype = ct.c_int
    L.ref_binomial.argtypes = [ct.c_int, ct.c_int]
    L.ref_poz.restype = _dbl
    L.ref_poz.argtypes = [_dbl]
    L.ref_pchisq.restype = _dbl
    L.ref_pchisq.argtypes = [_dbl, ct.c_int]
    L.ref_sepset_indices.restype = ct.c_int
    L.ref_sepset_indices.argtypes = [ct.c_int, ct.c_int, ct.c_int, _vp]
    L.ref_m2_inv.restype = ct.c_int
    L.ref_m2_inv.argtypes = [ct.c_int, _vp, _vp]
    L.ref_cholesky3.restype = ct.c_int
    L.ref_cholesky3.argtypes = [_vp, _vp]
    L.ref_inverse3.restype = ct.c_int
    L.ref_inverse3.argtypes = [_vp, _vp]
    L.ref_pin_p.restype = ct.c_int
    L.ref_pin_p.argtypes = []
    L.ref_gaussian_ci_test.restype = _dbl
    L.ref_gaussian_ci_test.argtypes = [ct.c_int, ct.c_uint, ct.c_uint, _vp, _vp]
    return L


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def binomial(n: int, k: int) -> int:
    return int(lib().orc_binomial(n, k))


def pchisq(x: float, df: int) -> float:
    return float(lib().orc_pchisq(float(x), int(df)))


def poz(z: float) -> float:
    return float(lib().orc_poz(float(z)))


def unrank(K: int, level: int, rank: int) -> np.ndarray:
    out = np.zeros(max(level, 1), np.int32)
    lib().orc_unrank(K, level, rank, ptr(out))
    return out[:level]


def compact(G: np.ndarray) -> np.ndarray:
    G = np.ascontiguousarray(G, dtype=np.uint16)
    p = G.shape[0]
    adj = np.zeros((p, p), np.int32)
    lib().orc_compact(ptr(G), p, ptr(adj))
    return adj
