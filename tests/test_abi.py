"""The C ABI: the library loads without a GPU and exports every symbol include/symeig.h
declares; host-side argument checks return error codes without touching the device."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "symeig.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(symeig_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for want in ("symeig_qr_f64", "symeig_qr_f64_dev", "symeig_qr_f64_q32", "symeig_qr_f64_q32_dev",
                 "symeig_apply_givens_f64", "symeig_apply_givens_f32",
                 "symeig_apply_givens_f64_dev", "symeig_apply_givens_f32_dev",
                 "symeig_eigen_decomp_f64", "symeig_create", "symeig_destroy"):
        assert want in syms


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert name in pkg._lib.SIGNATURES, f"{name} has no ctypes signature"


def test_checked_library_has_the_same_abi(pkg):
    """The checked build (device index checks in the wave tile) links the same entry points and
    loads without a GPU; host-side argument checks behave the same."""
    L = pkg.load_checked()
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert L.symeig_status_string(0) == b"ok"
    assert L.symeig_apply_givens_f64(None, None, 1, 0, 0, None, 0) == 5


def test_status_strings(pkg):
    lib = pkg.load_library()
    assert lib.symeig_status_string(0) == b"ok"
    assert b"NULL" in lib.symeig_status_string(1)
    assert lib.symeig_status_string(12345) == b"unknown status"


def test_null_handle_is_rejected_on_the_host(pkg):
    lib = pkg.load_library()
    conv, it = ctypes.c_int32(), ctypes.c_int64()
    assert lib.symeig_qr_f64(None, None, None, 4, None, 1, 0, 128, 1e-16, 100,
                             ctypes.byref(conv), ctypes.byref(it)) == 5
    assert lib.symeig_apply_givens_f64(None, None, 1, 0, 0, None, 0) == 5
    assert lib.symeig_destroy(None) == 5
    assert lib.symeig_get_stats(None, None) == 5
    assert lib.symeig_create(None, 0) == 1
