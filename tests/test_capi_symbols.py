"""The C-ABI library loads and exports every function the header declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "smolyax_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:int64_t|int|void|size_t|char\s*\*|const char\s*\*)\s*\**\s*(smx_\w+)\s*\(", src, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from smolyax_gb300 import _capi, build

    if not os.path.exists(_capi.LIB_PATH):
        build.build()
    return ctypes.CDLL(_capi.LIB_PATH)


def test_header_lists_entry_points():
    names = _declared()
    assert "smx_eval" in names and "smx_lambda_count" in names and len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_binding_table_matches_header():
    from smolyax_gb300 import _capi

    assert sorted(_capi.SIGNATURES) == _declared()


def test_version_and_error_string(lib):
    from smolyax_gb300 import _capi

    l = _capi.load()
    assert l.smx_version().startswith(b"smolyax_gb300")
    assert isinstance(l.smx_last_error_string(), bytes)
