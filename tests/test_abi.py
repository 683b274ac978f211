"""The C-ABI library builds, loads and exports every entry point include/sph_gb300.h declares
(no compute calls: this runs without a GPU)."""
import os
import re

import pytest

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


def _compile_c_host(native_path, out):
    """Compile tests/c_abi/search_host.c, a plain C program that drives the search through
    the C ABI alone, against the built library and the CUDA runtime."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    libdir = os.path.join(cuda, "lib64")
    if not os.path.exists(os.path.join(libdir, "libcudart.so")):
        import glob
        libdir = os.path.dirname(sorted(glob.glob(os.path.join(cuda, "targets", "*", "lib", "libcudart.so")))[0])
    lib = os.path.dirname(native_path)
    cmd = ["gcc", "-O2", "-Wall", "-Werror", "-o", out, os.path.join(ROOT, "tests", "c_abi", "search_host.c"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           "-L", lib, "-lsph_gb300", "-L", libdir, "-lcudart", "-lm", f"-Wl,-rpath,{lib}:{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_c_host_program_compiles_against_the_header(native_lib, tmp_path):
    _compile_c_host(native_lib._name, str(tmp_path / "search_host"))


@pytest.mark.gpu
def test_c_host_program_runs_the_search(native_lib, cuda, tmp_path):
    """The search pipeline called from C with cudaMalloc buffers (no torch anywhere on the
    path): the pair set equals a brute-force evaluation of the reference's predicate and the
    fused densities match a float64 Wendland sum."""
    import subprocess
    exe = _compile_c_host(native_lib._name, str(tmp_path / "search_host"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ") and int(r.stdout.split()[1]) > 4096 * 20
