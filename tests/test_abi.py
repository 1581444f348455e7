"""CPU tests of the C-ABI boundary: the library builds, loads without a GPU and exports
every entry point declared in include/mpsgb.h; the Python binding covers them all."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mpsgb.h")
LIB = os.path.join(ROOT, "mpskit.jl_gb300", "mpsgb", "libmpsgb.so")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", txt)))


def _stale():
    if not os.path.exists(LIB):
        return True
    csrc = os.path.join(ROOT, "mpskit.jl_gb300", "csrc")
    newest = max(os.path.getmtime(os.path.join(csrc, f)) for f in os.listdir(csrc))
    return max(newest, os.path.getmtime(HEADER)) > os.path.getmtime(LIB)


@pytest.fixture(scope="module")
def lib():
    if _stale():
        from mpsgb.build import build
        build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared()
    assert "gb_heff_apply" in names and "gb_env_transfer_left" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    from mpsgb import _lib
    assert sorted(_lib.exported_names()) == declared()


def test_version_without_gpu(lib):
    lib.gb_version.restype = ctypes.c_int
    assert lib.gb_version() >= 10000


def test_null_arguments_are_rejected_without_gpu(lib):
    lib.gb_tensor_norm.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    lib.gb_tensor_norm.restype = ctypes.c_int
    lib.gb_last_error.restype = ctypes.c_char_p
    assert lib.gb_tensor_norm(None, None) == 1  # GB_ERR_ARG
    assert b"null" in lib.gb_last_error()
