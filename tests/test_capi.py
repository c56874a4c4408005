"""The C ABI library builds, loads and exports every function include/bsg.h
declares (no compute: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(REPO, "include", "bsg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(bsg_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_api():
    names = declared_functions()
    for need in ["bsg_create", "bsg_hafnian_batched", "bsg_build_site", "bsg_site_sigma", "bsg_cut_spectra",
                 "bsg_build_mps", "bsg_pattern_amplitudes"]:
        assert need in names


def test_library_exports_every_declared_symbol():
    from bosonsupremacy_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libbsg.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    loaded = _lib.load()  # every binding in SIGNATURES resolves
    assert loaded.bsg_version() >= 10000
    for name in _lib.SIGNATURES:
        assert name in declared_functions(), name


def test_errors_are_reported_not_raised_in_c():
    from bosonsupremacy_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libbsg.so not built")
    lib = _lib.load()
    assert lib.bsg_hafnian_batched(None, None, 0, None, 0, 0, None, 0, None, None) == -1
    assert b"null handle" in lib.bsg_last_error()
