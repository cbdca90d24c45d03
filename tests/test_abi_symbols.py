"""The C-ABI library loads and exports every entry point include/oofem_gb300.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "oofem_gb300.h")) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ogb_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_all_declared_symbols(native_lib):
    lib = ctypes.CDLL(native_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(native_lib):
    assert set(declared_symbols()) == set(native_lib.SIGNATURES)


def test_error_string_without_gpu(native_lib):
    lib = native_lib.load()
    assert lib.ogb_version() == 1
    assert lib.ogb_last_error() is not None
