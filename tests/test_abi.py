"""The C-ABI library (no GPU needed): it loads, exports every symbol that
include/fpg.h declares, and validates arguments before touching the device."""

from __future__ import annotations

import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "fpg.h")).read()
    return sorted(set(re.findall(r"\b(fpg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = _declared_symbols()
    for s in ["fpg_operator_create", "fpg_apply", "fpg_summed_expect", "fpg_summed_apply_weighted",
              "fpg_expect_strings", "fpg_sparse_repr", "fpg_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    from fast_pauli import _abi

    lib = _abi.lib()
    missing = [s for s in _declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers the header too
    assert set(_declared_symbols()) <= set(_abi.SIGNATURES)


def test_version_and_device_count():
    from fast_pauli import _abi

    assert _abi.lib().fpg_abi_version() == 1
    c = ctypes.c_int(-1)
    assert _abi.lib().fpg_device_count(ctypes.byref(c)) == 0
    assert c.value >= 0


def test_invalid_character_is_rejected_before_device_work():
    from fast_pauli import _abi

    h = ctypes.c_void_p()
    rc = _abi.lib().fpg_operator_create(b"XAZ", 1, 3, ctypes.byref(h))
    assert rc == _abi.FPG_ERR_INVALID
    assert b"Invalid Pauli character A" in _abi.lib().fpg_last_error()
    assert not h


def test_argument_checks():
    from fast_pauli import _abi

    L = _abi.lib()
    h = ctypes.c_void_p()
    assert L.fpg_operator_create(b"X", 1, 0, ctypes.byref(h)) == _abi.FPG_ERR_UNSUPPORTED
    assert L.fpg_operator_create(b"X", 1, 41, ctypes.byref(h)) == _abi.FPG_ERR_UNSUPPORTED
    assert L.fpg_operator_create(b"X", -1, 1, ctypes.byref(h)) == _abi.FPG_ERR_INVALID
    assert L.fpg_operator_create(b"X", 1, 1, None) == _abi.FPG_ERR_INVALID
    assert L.fpg_apply(None, None, None, None, 1, 0, None) == _abi.FPG_ERR_INVALID
    assert L.fpg_summed_expect(None, None, 1, None, None, 1, 0, None) == _abi.FPG_ERR_INVALID
    assert L.fpg_operator_destroy(None) == _abi.FPG_OK


def test_pointer_classification_of_host_memory():
    from fast_pauli import _abi

    buf = ctypes.create_string_buffer(64)
    d = ctypes.c_int(7)
    assert _abi.lib().fpg_pointer_is_device(ctypes.cast(buf, ctypes.c_void_p), ctypes.byref(d)) == 0
    assert d.value == 0


def test_memory_pool_entry_points_without_device():
    from fast_pauli import _abi

    import fast_pauli as fp

    L = _abi.lib()
    assert L.fpg_device_alloc(None, 16, None) == _abi.FPG_ERR_INVALID
    assert L.fpg_device_free(None, None) == _abi.FPG_OK
    # nothing allocated yet in this process: releasing is a no-op
    assert L.fpg_release_cached_memory() == _abi.FPG_OK
    assert fp.release_cached_memory() is None
