"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, and
exports every function declared in include/casars_cuda.h (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "casars_cuda.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(cr_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("cr_build", os.path.join(ROOT, "casa-rs_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    return ctypes.CDLL(path)


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("cr_ctx_create", "cr_grid_dirty", "cr_degrid", "cr_dirty_image", "cr_hogbom",
                 "cr_wproj_create", "cr_apply_weighting", "cr_adjoint", "cr_predict"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from casars_cuda import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_string(lib):
    lib.cr_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.cr_version()
