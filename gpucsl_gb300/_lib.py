"""ctypes binding of libgpucsl_gb300.so (the C ABI declared in include/gpucsl_gb300.h).

There is no fallback: if the shared library is missing or no CUDA device is present,
every call raises.  Device buffers are torch tensors; their data pointers and the
current torch stream are handed to the C ABI.
"""
from __future__ import annotations

import ctypes as ct
from functools import lru_cache
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libgpucsl_gb300.so"

GCSL_OK = 0
GCSL_ERR_INVALID_ARG = 1
GCSL_ERR_WORKSPACE = 2
GCSL_ERR_UNSUPPORTED_LEVEL = 3
GCSL_ERR_TIMEOUT = 4
GCSL_ERR_DEVICE = 5
GCSL_ERR_CAPACITY = 6
GCSL_ERR_UNSUPPORTED = 7
GCSL_ERR_DEBUG_CHECK = 8
GCSL_MAX_LEVELS = 64
GCSL_DTYPE_F64 = 0
GCSL_DTYPE_F32 = 1
GCSL_DTYPE_I32 = 2
GCSL_DTYPE_I64 = 3
GCSL_DTYPE_U8 = 4

# every symbol the header declares (checked by the CPU test-suite)
EXPORTED = [
    "gcsl_version", "gcsl_last_error", "gcsl_status_string", "gcsl_kernel_launches",
    "gcsl_corr_workspace_bytes", "gcsl_corr_f64", "gcsl_corr_tc_workspace_bytes", "gcsl_corr_f64_tc",
    "gcsl_corr_tc_digits", "gcsl_corr_tc_product",
    "gcsl_gauss_workspace_bytes", "gcsl_gauss_skeleton", "gcsl_gauss_skeleton_noalloc",
    "gcsl_disc_workspace_bytes", "gcsl_disc_skeleton",
    "gcsl_compact", "gcsl_unrank", "gcsl_pchisq", "gcsl_disc_table", "gcsl_tc_gemm_bf16",
    "gcsl_gauss_batch_workspace_bytes", "gcsl_gauss_batch_prepare", "gcsl_gauss_batch_run",
    "gcsl_gauss_batch_collect", "gcsl_gauss_batch_set_lanes",
    "gcsl_corr_tc_batch_workspace_bytes", "gcsl_corr_tc_batch_prepare", "gcsl_corr_tc_batch_run",
    "gcsl_corr_tc_batch_run_split", "gcsl_corr_tc_batch_run_flagged", "gcsl_gauss_batch_rerun",
    "gcsl_gauss_batch_flags", "gcsl_gauss_state_bytes", "gcsl_gauss_batch_table_bytes",
    "gcsl_gauss_batch_prepare_staged", "gcsl_gauss_batch_step", "gcsl_records_to_dense",
    "gcsl_orient_workspace_bytes", "gcsl_orient_edges", "gcsl_encode_workspace_bytes", "gcsl_ordinal_encode",
    "gcsl_set_test_precision", "gcsl_debug_set_work_order", "gcsl_set_blocks_per_sm_cap",
]

GCSL_PREC_F64 = 0
GCSL_PREC_SPLIT = 1
GCSL_BATCH_MAX_LEVEL = 12


class GcslStats(ct.Structure):
    _fields_ = [
        ("levels_run", ct.c_int32),
        ("status", ct.c_int32),
        ("n_records", ct.c_int64),
        ("edges", ct.c_int64 * GCSL_MAX_LEVELS),
        ("tests", ct.c_int64 * GCSL_MAX_LEVELS),
        ("tests_full", ct.c_int64 * GCSL_MAX_LEVELS),
        ("removed", ct.c_int64 * GCSL_MAX_LEVELS),
        ("max_degree", ct.c_int32 * GCSL_MAX_LEVELS),
        ("level_ms", ct.c_float * GCSL_MAX_LEVELS),
        ("debug_site", ct.c_int32),
    ]

    def as_dict(self) -> dict:
        n = max(int(self.levels_run), 0)
        return {
            "levels_run": n,
            "status": int(self.status),
            "n_records": int(self.n_records),
            "edges": [int(x) for x in self.edges[:n]],
            "tests": [int(x) for x in self.tests[:n]],
            "tests_full": [int(x) for x in self.tests_full[:n]],
            "removed": [int(x) for x in self.removed[:n]],
            "max_degree": [int(x) for x in self.max_degree[:n]],
            "level_ms": [float(x) for x in self.level_ms[:GCSL_MAX_LEVELS] if x > 0],
            "debug_site": int(self.debug_site),
        }


class GaussInstance(ct.Structure):
    """gcsl_gauss_instance: one problem of a batch (device pointers, host thresholds)."""
    _fields_ = [
        ("C", ct.c_void_p),
        ("C32", ct.c_void_p),
        ("p", ct.c_int32),
        ("n_obs", ct.c_int64),
        ("thresholds", ct.POINTER(ct.c_double)),
        ("n_thresholds", ct.c_int32),
        ("band_lo", ct.POINTER(ct.c_double)),
        ("band_hi", ct.POINTER(ct.c_double)),
        ("G", ct.c_void_p),
        ("pmax", ct.c_void_p),
        ("rec_pool", ct.c_void_p),
        ("rec_cap", ct.c_int64),
        ("c_err", ct.c_void_p),
        ("state", ct.c_void_p),
        ("status", ct.c_int32),
        ("levels_run", ct.c_int32),
        ("n_records", ct.c_int64),
        ("tests", ct.c_int64),
        ("retests", ct.c_int64),
        ("exact_rerun", ct.c_int32),
    ]


class BatchPlan(ct.Structure):
    _fields_ = [("w", ct.c_int64 * 48)]


class GcslError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        detail = ""
        if code == GCSL_ERR_DEVICE:
            try:
                detail = lib().gcsl_last_error().decode()
            except Exception:
                detail = ""
        super().__init__(f"{what}: {status_string(code)} (status {code})" + (f" [{detail}]" if detail else ""))


_vp = ct.c_void_p
_i32 = ct.c_int32
_i64 = ct.c_int64
_sz = ct.c_size_t
_dbl = ct.c_double


@lru_cache(maxsize=2)
def lib(debug: bool = False) -> ct.CDLL:
    """The release library, or with debug the bounds-checked build (compiled on first
    use, as the reference compiles its kernels with -G when is_debug is set)."""
    if debug:
        from . import build as _build

        path = _build.build(debug=True)
    else:
        path = LIB_PATH
        if not path.exists():
            raise RuntimeError(
                f"{path.name} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(requires nvcc) before using gpucsl_gb300")
    L = ct.CDLL(str(path))
    L.gcsl_version.restype = ct.c_int
    L.gcsl_version.argtypes = []
    L.gcsl_kernel_launches.restype = ct.c_int64
    L.gcsl_kernel_launches.argtypes = []
    L.gcsl_last_error.restype = ct.c_char_p
    L.gcsl_last_error.argtypes = []
    L.gcsl_status_string.restype = ct.c_char_p
    L.gcsl_status_string.argtypes = [ct.c_int]
    L.gcsl_corr_workspace_bytes.restype = _sz
    L.gcsl_corr_workspace_bytes.argtypes = [_i64, _i32]
    L.gcsl_corr_f64.restype = ct.c_int
    L.gcsl_corr_f64.argtypes = [_vp, _i32, _i64, _i32, _i64, _vp, _vp, _sz, _vp]
    L.gcsl_corr_tc_workspace_bytes.restype = _sz
    L.gcsl_corr_tc_workspace_bytes.argtypes = [_i64, _i32]
    L.gcsl_corr_f64_tc.restype = ct.c_int
    L.gcsl_corr_f64_tc.argtypes = [_vp, _i32, _i64, _i32, _i64, _vp, _vp, _sz, _vp]
    L.gcsl_corr_tc_digits.restype = ct.c_int
    L.gcsl_corr_tc_digits.argtypes = [_vp, _i32, _i64, _i32, _i64, _vp, _sz, _vp]
    L.gcsl_corr_tc_product.restype = ct.c_int
    L.gcsl_corr_tc_product.argtypes = [_i64, _i32, _vp, _vp, _sz, _vp]
    L.gcsl_gauss_workspace_bytes.restype = _sz
    L.gcsl_gauss_workspace_bytes.argtypes = [_i32, _i32]
    L.gcsl_gauss_skeleton.restype = ct.c_int
    L.gcsl_gauss_skeleton.argtypes = [_vp, _i32, _i64, ct.POINTER(_dbl), _i32, _i32, _vp, _vp, _vp, _i64, _vp,
                                      ct.POINTER(GcslStats), _vp, _sz, _vp]
    L.gcsl_gauss_skeleton_noalloc.restype = ct.c_int
    L.gcsl_gauss_skeleton_noalloc.argtypes = [_vp, _i32, _i64, ct.POINTER(_dbl), _i32, _i32, _vp, _vp, _vp, _i64,
                                              _vp, ct.POINTER(GcslStats), _vp]
    L.gcsl_disc_workspace_bytes.restype = _sz
    L.gcsl_disc_workspace_bytes.argtypes = [_i32, _i64, _i32, _i32]
    L.gcsl_disc_skeleton.restype = ct.c_int
    L.gcsl_disc_skeleton.argtypes = [_vp, _i64, _i64, _i32, _vp, _i32, _dbl, _i32, _vp, _vp, _vp, _i64, _vp,
                                     ct.POINTER(GcslStats), _vp, _sz, _vp]
    L.gcsl_compact.restype = ct.c_int
    L.gcsl_compact.argtypes = [_vp, _i32, _vp, _vp]
    L.gcsl_unrank.restype = ct.c_int
    L.gcsl_unrank.argtypes = [_i32, _i32, _i64, _vp, _vp]
    L.gcsl_pchisq.restype = ct.c_int
    L.gcsl_pchisq.argtypes = [_vp, _vp, _i64, _vp, _vp]
    L.gcsl_disc_table.restype = ct.c_int
    L.gcsl_disc_table.argtypes = [_vp, _i64, _i64, _vp, _i32, _i32, ct.POINTER(_i32), _i32, _vp, _i64, _vp, _vp]
    L.gcsl_tc_gemm_bf16.restype = ct.c_int
    L.gcsl_tc_gemm_bf16.argtypes = [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp]
    L.gcsl_gauss_batch_workspace_bytes.restype = _sz
    L.gcsl_gauss_batch_workspace_bytes.argtypes = [ct.POINTER(_i32), _i32]
    L.gcsl_gauss_batch_prepare.restype = ct.c_int
    L.gcsl_gauss_batch_prepare.argtypes = [ct.POINTER(GaussInstance), _i32, _i32, _i32, _vp, _sz,
                                           ct.POINTER(BatchPlan), _vp]
    L.gcsl_gauss_batch_run.restype = ct.c_int
    L.gcsl_gauss_batch_run.argtypes = [ct.POINTER(BatchPlan), _vp]
    L.gcsl_gauss_batch_collect.restype = ct.c_int
    L.gcsl_gauss_batch_collect.argtypes = [ct.POINTER(BatchPlan), ct.POINTER(GaussInstance), _i32, _vp]
    L.gcsl_gauss_batch_set_lanes.restype = ct.c_int
    L.gcsl_gauss_batch_set_lanes.argtypes = [ct.POINTER(BatchPlan), _i32, _i32]
    L.gcsl_corr_tc_batch_workspace_bytes.restype = _sz
    L.gcsl_corr_tc_batch_workspace_bytes.argtypes = [ct.POINTER(_i64), ct.POINTER(_i32), _i32]
    L.gcsl_corr_tc_batch_prepare.restype = ct.c_int
    L.gcsl_corr_tc_batch_prepare.argtypes = [ct.POINTER(_vp), _i32, ct.POINTER(_i64), ct.POINTER(_i32),
                                             ct.POINTER(_i64), ct.POINTER(_vp), ct.POINTER(_vp), _i32, _vp, _sz,
                                             ct.POINTER(BatchPlan), _vp]
    L.gcsl_corr_tc_batch_run.restype = ct.c_int
    L.gcsl_corr_tc_batch_run.argtypes = [ct.POINTER(BatchPlan), _vp]
    L.gcsl_corr_tc_batch_run_split.restype = ct.c_int
    L.gcsl_corr_tc_batch_run_split.argtypes = [ct.POINTER(BatchPlan), _vp, _vp]
    L.gcsl_corr_tc_batch_run_flagged.restype = ct.c_int
    L.gcsl_corr_tc_batch_run_flagged.argtypes = [ct.POINTER(BatchPlan), _vp, _vp]
    L.gcsl_gauss_batch_rerun.restype = ct.c_int
    L.gcsl_gauss_batch_rerun.argtypes = [ct.POINTER(BatchPlan), _vp]
    L.gcsl_gauss_batch_flags.restype = _vp
    L.gcsl_gauss_batch_flags.argtypes = [ct.POINTER(BatchPlan)]
    L.gcsl_gauss_state_bytes.restype = _sz
    L.gcsl_gauss_state_bytes.argtypes = [_i32]
    L.gcsl_gauss_batch_table_bytes.restype = _sz
    L.gcsl_gauss_batch_table_bytes.argtypes = [_i32]
    L.gcsl_gauss_batch_prepare_staged.restype = ct.c_int
    L.gcsl_gauss_batch_prepare_staged.argtypes = [ct.POINTER(GaussInstance), _i32, _i32, _i32, _vp, _sz, _vp, _sz,
                                                  ct.POINTER(BatchPlan), _vp]
    L.gcsl_gauss_batch_step.restype = ct.c_int
    L.gcsl_gauss_batch_step.argtypes = [ct.POINTER(BatchPlan), _i32, _i32, _i32, _vp, _vp]
    L.gcsl_records_to_dense.restype = ct.c_int
    L.gcsl_records_to_dense.argtypes = [_vp, _i64, _i32, _i32, _vp]
    L.gcsl_set_test_precision.restype = ct.c_int
    L.gcsl_set_test_precision.argtypes = [_i32]
    L.gcsl_debug_set_work_order.restype = ct.c_int
    L.gcsl_debug_set_work_order.argtypes = [ct.c_uint64]
    L.gcsl_set_blocks_per_sm_cap.restype = ct.c_int
    L.gcsl_set_blocks_per_sm_cap.argtypes = [_i32]
    L.gcsl_encode_workspace_bytes.restype = _sz
    L.gcsl_encode_workspace_bytes.argtypes = [_i32]
    L.gcsl_ordinal_encode.restype = ct.c_int
    L.gcsl_ordinal_encode.argtypes = [_vp, _i32, _i64, _i32, _i64, _vp, _i64, _vp, _vp, _sz, _vp]
    L.gcsl_orient_workspace_bytes.restype = _sz
    L.gcsl_orient_workspace_bytes.argtypes = [_i32]
    L.gcsl_orient_edges.restype = ct.c_int
    L.gcsl_orient_edges.argtypes = [_vp, _i32, _vp, _i32, _vp, ct.POINTER(_i32), _vp, _sz, _vp]
    if L.gcsl_version() != 2:
        raise RuntimeError("libgpucsl_gb300.so ABI version mismatch")
    return L


def status_string(code: int) -> str:
    try:
        return lib().gcsl_status_string(int(code)).decode()
    except Exception:  # library not loadable: plain code
        return f"status {code}"


def check(code: int, what: str) -> None:
    if code != GCSL_OK:
        raise GcslError(code, what)


def require_cuda():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("gpucsl_gb300 needs a CUDA device (sm_103a); none is available")
    return torch


def stream_ptr(stream=None) -> int:
    torch = require_cuda()
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t) -> int | None:
    return None if t is None else int(t.data_ptr())
