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
    assert L.gcsl_version() == 1
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
