"""The C-ABI library on a host without a GPU: it builds for sm_103a, loads,
exports every function include/shape_atrophy_gb300.h declares, and refuses
to create a context when no device exists (an error code, not a crash).
No compute call runs here."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "shape_atrophy_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(sa_[A-Za-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from shape_atrophy_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("sa_create", "sa_destroy", "sa_error_message", "sa_forward", "sa_varifold",
                 "sa_deformation_frame", "sa_computeObjfcn_frame", "sa_session_create", "sa_session_step",
                 "sa_server_create", "sa_server_submit", "sa_server_result", "sa_varifold_noalloc"):
        assert must in names


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_context_creation_fails_cleanly_without_a_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.sa_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    h = C.c_void_p()
    rc = lib.sa_create(C.byref(h), 0)
    assert rc != 0 and not h.value
