"""ctypes wrapper over oracle/_ref/libfpref.so: the reference's own C++
implementation (qognitive/fast-pauli headers compiled unmodified by
oracle/build_ref.sh), driven through oracle/ref_driver.cpp.

TEST INFRASTRUCTURE ONLY.  Available only where the reference sources were
present at build time; callers check :func:`available` first.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libfpref.so")
_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        lib()
    except OSError:
        return False
    return True


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        ci = ctypes.c_int
        d = ctypes.c_double
        L.fpref_sparse_repr.argtypes = [ctypes.c_char_p, ci, P, P]
        L.fpref_string_apply_batch.argtypes = [ctypes.c_char_p, ci, i64, P, P, d, d]
        L.fpref_string_apply_1d.argtypes = [ctypes.c_char_p, ci, P, P]
        L.fpref_string_expectation.argtypes = [ctypes.c_char_p, ci, i64, P, P, d, d]
        L.fpref_op_apply.argtypes = [ctypes.c_char_p, i64, ci, P, i64, P, P]
        L.fpref_op_expectation.argtypes = [ctypes.c_char_p, i64, ci, P, i64, P, P]
        L.fpref_summed_expectation.argtypes = [ctypes.c_char_p, i64, ci, P, i64, i64, P, P]
        L.fpref_summed_apply.argtypes = [ctypes.c_char_p, i64, ci, P, i64, i64, P, P]
        L.fpref_summed_apply_weighted.argtypes = [ctypes.c_char_p, i64, ci, P, i64, i64, P, P, P]
        L.fpref_pauli_strings_max_weight.argtypes = [ci, ci, ctypes.c_char_p]
        L.fpref_pauli_strings_max_weight.restype = i64
        L.fpref_summed_square.argtypes = [ctypes.c_char_p, i64, ci, P, i64, ctypes.c_char_p, P]
        L.fpref_summed_square.restype = i64
        L.fpref_op_product.argtypes = [ctypes.c_char_p, P, i64, ctypes.c_char_p, P, i64, ci, ctypes.c_char_p, P]
        L.fpref_op_product.restype = i64
        _lib = L
    return _lib


def _c(a, dtype=np.complex128):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data


def _join(strings):
    strings = [str(s) for s in strings]
    return "".join(strings).encode(), len(strings[0])


def _as2d(psi):
    return psi.reshape(psi.shape[0], 1) if psi.ndim == 1 else psi


def sparse_repr(string: str):
    n = len(string)
    k = np.zeros(1 << n, dtype=np.uint64)
    m = np.zeros(1 << n, dtype=np.complex128)
    lib().fpref_sparse_repr(string.encode(), n, _p(k), _p(m))
    return k, m


def string_apply(string: str, psi, coeff=1.0):
    psi = _c(psi)
    out = np.zeros_like(psi)
    if psi.ndim == 1:
        lib().fpref_string_apply_1d(string.encode(), len(string), _p(psi), _p(out))
        return out
    c = complex(coeff)
    lib().fpref_string_apply_batch(string.encode(), len(string), psi.shape[1], _p(psi), _p(out), c.real, c.imag)
    return out


def string_expectation(string: str, psi, coeff=1.0):
    p2 = _as2d(_c(psi))
    ev = np.zeros(p2.shape[1], dtype=np.complex128)
    c = complex(coeff)
    lib().fpref_string_expectation(string.encode(), len(string), p2.shape[1], _p(p2), _p(ev), c.real, c.imag)
    return ev


def op_apply(strings, coeffs, psi):
    psi = _c(psi)
    p2 = _as2d(psi)
    b, n = _join(strings)
    c = _c(coeffs)
    out = np.zeros_like(p2)
    lib().fpref_op_apply(b, len(strings), n, _p(c), p2.shape[1], _p(p2), _p(out))
    return out.reshape(psi.shape)


def op_expectation(strings, coeffs, psi):
    p2 = _as2d(_c(psi))
    b, n = _join(strings)
    c = _c(coeffs)
    ev = np.zeros(p2.shape[1], dtype=np.complex128)
    lib().fpref_op_expectation(b, len(strings), n, _p(c), p2.shape[1], _p(p2), _p(ev))
    return ev


def summed_expectation(strings, h, psi):
    psi = _c(psi)
    p2 = _as2d(psi)
    b, n = _join(strings)
    h = _c(h)
    out = np.zeros((h.shape[1], p2.shape[1]), dtype=np.complex128)
    lib().fpref_summed_expectation(b, len(strings), n, _p(h), h.shape[1], p2.shape[1], _p(p2), _p(out))
    return out[:, 0] if psi.ndim == 1 else out


def summed_apply(strings, h, psi):
    psi = _c(psi)
    p2 = _as2d(psi)
    b, n = _join(strings)
    h = _c(h)
    out = np.zeros_like(p2)
    lib().fpref_summed_apply(b, len(strings), n, _p(h), h.shape[1], p2.shape[1], _p(p2), _p(out))
    return out.reshape(psi.shape)


def summed_apply_weighted(strings, h, psi, data):
    psi = _c(psi)
    p2 = _as2d(psi)
    b, n = _join(strings)
    h = _c(h)
    data = _c(data, np.float64)
    d2 = data.reshape(data.shape[0], 1) if data.ndim == 1 else data
    out = np.zeros_like(p2)
    lib().fpref_summed_apply_weighted(b, len(strings), n, _p(h), h.shape[1], p2.shape[1], _p(p2), _p(d2), _p(out))
    return out.reshape(psi.shape)


def pauli_strings_max_weight(n: int, w: int) -> list[str]:
    cnt = lib().fpref_pauli_strings_max_weight(n, w, None)
    buf = ctypes.create_string_buffer(int(cnt) * n + 1)
    lib().fpref_pauli_strings_max_weight(n, w, buf)
    raw = buf.raw[: cnt * n].decode()
    return [raw[j * n : (j + 1) * n] for j in range(cnt)]


def summed_square(strings, h):
    b, n = _join(strings)
    h = _c(h)
    P, K = h.shape
    cnt = lib().fpref_summed_square(b, P, n, _p(h), K, None, None)
    sbuf = ctypes.create_string_buffer(int(cnt) * n + 1)
    out_h = np.zeros((cnt, K), dtype=np.complex128)
    lib().fpref_summed_square(b, P, n, _p(h), K, sbuf, _p(out_h))
    raw = sbuf.raw[: cnt * n].decode()
    return [raw[j * n : (j + 1) * n] for j in range(cnt)], out_h


def op_product(a_coeffs, a_strings, b_coeffs, b_strings):
    """The reference's PauliOp operator*: (strings, coefficients) as it
    returns them (one entry per string per OpenMP thread map)."""
    ab, n = _join(a_strings)
    bb, _ = _join(b_strings)
    a = _c(a_coeffs)
    b = _c(b_coeffs)
    cnt = lib().fpref_op_product(ab, _p(a), len(a_strings), bb, _p(b), len(b_strings), n, None, None)
    sbuf = ctypes.create_string_buffer(int(cnt) * n + 1)
    out = np.zeros(cnt, dtype=np.complex128)
    lib().fpref_op_product(ab, _p(a), len(a_strings), bb, _p(b), len(b_strings), n, sbuf, _p(out))
    raw = sbuf.raw[: cnt * n].decode()
    return [raw[j * n : (j + 1) * n] for j in range(cnt)], out
