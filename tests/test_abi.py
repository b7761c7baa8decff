"""The C ABI library loads and exports every entry point include/tmc_gb300.h declares (no GPU
needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from tmc_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def declared():
    hdr = open(os.path.join(ROOT, "include", "tmc_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:tmc_status|const char\*|void\*|int64_t|int32_t)\s+(tmc_\w+)\(", hdr, re.M)))


def test_header_declares_entry_points():
    names = declared()
    assert "tmc_dmc_extract" in names and "tmc_tmc_sharedvertex" in names


def test_library_exports_every_declared_symbol(lib):
    from tmc_gb300 import native
    for name in declared():
        assert hasattr(lib, name), name
    assert sorted(native.EXPORTS) == declared()
