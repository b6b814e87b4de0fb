"""The C-ABI library builds, loads and exports every symbol include/gpucsl_gb300.h declares.
CPU only: nothing here launches device work."""
import ctypes as ct
import re
import shutil
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "gpucsl_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gcsl_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
        pytest.skip("nvcc not available")
    from gpucsl_gb300 import build

    return build.build()


def test_header_declares_expected_entry_points():
    from gpucsl_gb300 import _lib

    assert declared_functions() == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(built_lib):
    lib = ct.CDLL(str(built_lib))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version_and_status_strings(built_lib):
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    assert L.gcsl_version() == 2
    assert L.gcsl_status_string(0) == b"ok"
    assert b"record pool" in L.gcsl_status_string(_lib.GCSL_ERR_CAPACITY)
    # argument validation happens on the host, before any device call
    assert L.gcsl_gauss_skeleton(None, 0, 0, None, 0, 0, None, None, None, 0, None, None, None, 0, None) == 1
    assert L.gcsl_disc_skeleton(None, 0, 0, 0, None, 0, 0.05, 0, None, None, None, 0, None, None, None, 0, None) == 1


def test_workspace_queries(built_lib):
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    a = L.gcsl_gauss_workspace_bytes(100, 3)
    b = L.gcsl_gauss_workspace_bytes(1000, 3)
    assert 0 < a < b
    assert b >= 1000 * 1000 * (4 + 8)
    assert L.gcsl_corr_workspace_bytes(10000, 1000) >= 1000 * 8
    assert L.gcsl_disc_workspace_bytes(200, 50000, 3, 5) >= 200 * 200 * (4 + 8)


def header_define(name: str) -> int:
    m = re.search(rf"#define\s+{name}\s+(\d+)", HEADER.read_text())
    assert m, name
    return int(m.group(1))


def test_noalloc_scratch_holds_the_largest_problem(built_lib):
    """The static scratch of gcsl_gauss_skeleton_noalloc must hold the workspace of
    p = GCSL_NOALLOC_MAX_P (the query is host arithmetic only)."""
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    pmax = header_define("GCSL_NOALLOC_MAX_P")
    need = L.gcsl_gauss_workspace_bytes(pmax, 64)
    assert need <= header_define("GCSL_NOALLOC_SCRATCH_BYTES"), need


def test_gauss_rejects_pair_index_overflow(built_lib):
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    p = header_define("GCSL_GAUSS_MAX_P") + 1
    thr = (ct.c_double * 1)(0.1)
    dummy = ct.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.gcsl_gauss_skeleton(dummy, p, 100, thr, 1, 0, dummy, None, None, 0, dummy, None, dummy, 1 << 40, None)
    assert rc == _lib.GCSL_ERR_UNSUPPORTED


@pytest.mark.parametrize("case", ["ld_not_16", "ld_below_n", "misaligned", "max_dim_0", "max_dim_256", "p_0",
                                  "no_workspace"])
def test_disc_argument_checks(built_lib, case):
    """gcsl_disc_skeleton's argument checks run on the host before any device call and
    before any pointer is dereferenced (the addresses below are never read)."""
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    a = dict(data=16, ld=64, n=50, p=4, dims=16, max_dim=5, G=16, pmax=16, ws=16, ws_bytes=1 << 40)
    expect = _lib.GCSL_ERR_INVALID_ARG
    if case == "ld_not_16":
        a["ld"] = 60
    elif case == "ld_below_n":
        a["ld"], a["n"] = 48, 50
    elif case == "misaligned":
        a["data"] = 24
    elif case == "max_dim_0":
        a["max_dim"] = 0
    elif case == "max_dim_256":
        a["max_dim"] = 256
    elif case == "p_0":
        a["p"] = 0
    elif case == "no_workspace":
        a["ws"], expect = None, _lib.GCSL_ERR_WORKSPACE
    vp = lambda x: None if x is None else ct.c_void_p(x)  # noqa: E731
    rc = L.gcsl_disc_skeleton(vp(a["data"]), a["ld"], a["n"], a["p"], vp(a["dims"]), a["max_dim"], 0.05, 3,
                              vp(a["G"]), None, None, 0, vp(a["pmax"]), None, vp(a["ws"]), a["ws_bytes"], None)
    assert rc == expect, (case, rc)


NULL_CALLS = {
    # entry point: arguments with a null required pointer (or a size out of range)
    "gcsl_corr_f64": (None, 0, 100, 4, 4, None, None, 0, None),
    "gcsl_corr_f64_tc": (None, 0, 100, 4, 4, None, None, 0, None),
    "gcsl_corr_tc_digits": (None, 0, 100, 4, 4, None, 0, None),
    "gcsl_corr_tc_product": (100, 4, None, None, 0, None),
    "gcsl_orient_edges": (None, 4, None, 0, None, None, None, 0, None),
    "gcsl_gauss_batch_run": (None, None),
    "gcsl_corr_tc_batch_run": (None, None),
    "gcsl_gauss_batch_set_lanes": (None, 1, 32),
    "gcsl_compact": (None, 4, None, None),
    "gcsl_unrank": (5, 0, 1, None, None),
    "gcsl_pchisq": (None, None, 1, None, None),
    "gcsl_tc_gemm_bf16": (None, None, None, 128, 128, 64, None, None),
}


@pytest.mark.parametrize("name", sorted(NULL_CALLS))
def test_null_or_out_of_range_arguments_are_rejected_on_the_host(built_lib, name):
    """Each compute entry point rejects a null required pointer (or a size out of range)
    with GCSL_ERR_INVALID_ARG before any device call."""
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    fn = getattr(L, name)
    if fn.argtypes is None or len(fn.argtypes) != len(NULL_CALLS[name]):
        pytest.skip(f"{name}: argtypes not declared with this arity")
    assert fn(*NULL_CALLS[name]) == _lib.GCSL_ERR_INVALID_ARG


def test_precision_switch_range(built_lib):
    from gpucsl_gb300 import _lib

    L = _lib.lib()
    assert L.gcsl_set_test_precision(3) == _lib.GCSL_ERR_INVALID_ARG
    assert L.gcsl_set_test_precision(-1) == _lib.GCSL_ERR_INVALID_ARG
    assert L.gcsl_set_test_precision(0) == _lib.GCSL_OK


def test_release_library_has_no_debug_work_order(built_lib):
    """The work-order switch belongs to the bounds-checked build; the release library
    refuses it on the host (no device work)."""
    from gpucsl_gb300 import _lib

    assert _lib.lib().gcsl_debug_set_work_order(1) == _lib.GCSL_ERR_UNSUPPORTED
