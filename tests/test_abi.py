"""The C-ABI library builds, loads and exports every entry point include/sph_gb300.h declares
(no compute calls: this runs without a GPU)."""
import os
import re

from conftest import ROOT


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sph_nl_count" in names and "sph_radix_sort_pairs" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_table_matches_header():
    from pytorchsph_gb300 import _native
    assert sorted(_native.SIGNATURES) == declared_functions()


def test_abi_version_and_status_strings(native_lib):
    import ctypes
    native_lib.sph_abi_version.restype = ctypes.c_int32
    assert native_lib.sph_abi_version() >= 1
    native_lib.sph_status_string.restype = ctypes.c_char_p
    native_lib.sph_status_string.argtypes = [ctypes.c_int32]
    assert native_lib.sph_status_string(0) == b"ok"


def test_product_path_refuses_cpu():
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    from pytorchsph_gb300 import _native
    with pytest.raises(RuntimeError):
        _native.load()
