"""The C-ABI library loads and exports every symbol include/*.h declares (CPU only:
no compute calls)."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(mgr_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from magritte_gb300 import _abi, build
    build.build_gpu()
    return _abi.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("mgr_model_create", "mgr_formal_solve_fo2", "mgr_last_error", "mgr_model_free"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(lib):
    from magritte_gb300 import _abi
    assert set(declared_symbols()) == set(_abi.SIGNATURES)
