"""CPU tests of the C-ABI library: it builds, loads, exports every symbol include/gkrgpu.h
declares, and its host-only entry points behave (no device compute here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gkrgpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gkrgpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from gkr_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["gkrgpu_create", "gkrgpu_circuit_load", "gkrgpu_evaluate", "gkrgpu_prove", "gkrgpu_prove_device",
              "gkrgpu_proof_size", "gkrgpu_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from gkr_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert bound == set(declared_symbols())


def test_host_only_entry_points(lib):
    assert lib.gkrgpu_num_repetitions(10) == 3
    assert lib.gkrgpu_num_repetitions(8) == 3
    assert lib.gkrgpu_num_repetitions(7) == 3
    assert lib.gkrgpu_num_repetitions(6) == 4
    assert b"sm_103a" in lib.gkrgpu_version()
    assert lib.gkrgpu_proof_size(None, 16, 10) == 0


def test_create_reports_errors_instead_of_crashing(lib):
    h = ctypes.c_void_p()
    assert lib.gkrgpu_create(-1, ctypes.byref(h)) != 0
    assert lib.gkrgpu_last_error()
    rc = lib.gkrgpu_create(0, ctypes.byref(h))
    if rc == 0:  # a GPU is present
        lib.gkrgpu_destroy(h)
    else:
        assert lib.gkrgpu_last_error()
