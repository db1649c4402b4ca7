"""The C-ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "flag4j_cuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(f4j_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for must in ("f4j_create", "f4j_dgemm", "f4j_zgemm", "f4j_spmv", "f4j_spmm", "f4j_spmm_t", "f4j_sddmm",
                 "f4j_csr_from_coo", "f4j_dgemm_adjoint", "f4j_last_error"):
        assert must in syms


def test_library_exports_every_symbol(lib):
    from flag4j_gb300 import _lib
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, "no ctypes signature for %s" % s


def test_errors_without_device(lib):
    # Null arguments are rejected before any device work.
    from flag4j_gb300 import _lib
    assert lib.f4j_dgemm(None, 1, 1, 1, None, 0, None, 0, None, 0, None) == _lib.F4J_ERR_ARG
    assert "null context" in _lib.last_error()
    assert lib.f4j_create(0, None) == _lib.F4J_ERR_ARG
    assert lib.f4j_buf_size(None) == 0
    assert lib.f4j_version() == 100


def test_report_struct_layout():
    from flag4j_gb300 import _lib
    assert ctypes.sizeof(_lib.f4j_report) == 96
    assert ctypes.sizeof(_lib.f4j_dispatch_config) == 48
