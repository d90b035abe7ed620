"""CPU oracle for the Pauli apply / expectation path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, and there only as the checker.  No
product code imports it.

Two layers:

* ``fp_oracle.c`` -- a plain-C/OpenMP restatement of the reference's
  algorithms (each function cites the reference header it follows), built by
  :func:`build` into ``oracle/_build/libfporacle.so``.
* ``_ref/libfpref.so`` -- when ``oracle/build_ref.sh`` could compile the
  reference's own headers (only where the reference sources are present), a
  C-ABI over the reference itself.  :mod:`oracle.ref` wraps it; it pins the
  restatement and generates the golden fixtures in ``tests/golden``.

Complex arrays are complex128, row-major, states laid out (2**n, n_states).
All ``*_into`` style C functions accumulate; the wrappers here start from zero.
"""

from __future__ import annotations

import ctypes
import itertools
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libfporacle.so")
_lib = None

_CODE = {"I": 0, "X": 1, "Y": 2, "Z": 3}


def build(force: bool = False) -> str:
    """Compile fp_oracle.c (gcc, -O3, OpenMP) into oracle/_build/."""
    src = os.path.join(HERE, "fp_oracle.c")
    if (
        not force
        and os.path.exists(_LIB_PATH)
        and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)
    ):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(
        ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp]
    )
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        ci = ctypes.c_int
        d = ctypes.c_double
        L.fpo_sparse_repr.argtypes = [P, ci, P, P]
        L.fpo_string_apply_batch.argtypes = [P, ci, i64, P, P, d, d]
        L.fpo_string_expectation.argtypes = [P, ci, i64, P, P, d, d]
        L.fpo_op_apply.argtypes = [P, i64, ci, P, i64, P, P]
        L.fpo_op_expectation.argtypes = [P, i64, ci, P, i64, P, P]
        L.fpo_summed_expectation.argtypes = [P, i64, ci, P, i64, i64, P, P]
        L.fpo_summed_apply.argtypes = [P, i64, ci, P, i64, i64, P, P]
        L.fpo_summed_apply_weighted.argtypes = [P, i64, ci, P, i64, i64, P, P, P]
        L.fpo_summed_square.argtypes = [P, i64, ci, P, i64, P, i64, P]
        L.fpo_summed_square.restype = ci
        L.fpo_summed_to_tensor.argtypes = [P, i64, ci, P, i64, P]
        L.fpo_op_product.argtypes = [P, P, i64, P, P, i64, ci, P, P]
        L.fpo_op_product.restype = i64
        L.fpo_max_threads.restype = ci
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().fpo_max_threads())


# --------------------------------------------------------------------------
# helpers: restatement of fast_pauli/cpp/include/__pauli_helpers.hpp
# --------------------------------------------------------------------------


def get_nontrivial_paulis(weight: int) -> list[str]:
    """__pauli_helpers.hpp:36-60: all words over {X,Y,Z} of length `weight`,
    built by appending X, Y, Z to each shorter word (first letter slowest)."""
    if weight == 0:
        return []
    return ["".join(p) for p in itertools.product("XYZ", repeat=weight)]


def idx_combinations(n: int, k: int) -> list[list[int]]:
    """__pauli_helpers.hpp:69-89: index sets of size k from a bitmask of k
    leading ones walked by prev_permutation, i.e. combinations in
    lexicographic order."""
    return [list(c) for c in itertools.combinations(range(n), k)]


def calculate_pauli_strings(n: int, weight: int) -> list[str]:
    """__pauli_helpers.hpp:99-134: nontrivial letter words outer, index
    combinations inner."""
    if weight == 0:
        return ["I" * n]
    out = []
    for word in get_nontrivial_paulis(weight):
        for combo in idx_combinations(n, weight):
            s = ["I"] * n
            for q, idx in enumerate(combo):
                s[idx] = word[q]
            out.append("".join(s))
    return out


def calculate_pauli_strings_max_weight(n: int, weight: int) -> list[str]:
    """__pauli_helpers.hpp:144-153 (weights 0..weight; includes the identity)."""
    out: list[str] = []
    for w in range(weight + 1):
        out.extend(calculate_pauli_strings(n, w))
    return out


# --------------------------------------------------------------------------
# numpy wrappers around fp_oracle.c
# --------------------------------------------------------------------------


def codes_of(strings) -> tuple[np.ndarray, int]:
    strings = [str(s) for s in strings]
    n = len(strings[0]) if strings else 0
    arr = np.zeros((len(strings), max(n, 1)), dtype=np.uint8)
    for j, s in enumerate(strings):
        if len(s) != n:
            raise ValueError("All PauliStrings must have the same size")
        arr[j, :n] = [_CODE[c] for c in s]
    return np.ascontiguousarray(arr[:, :n]), n


def _c(a, dtype=np.complex128) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def sparse_repr(string: str) -> tuple[np.ndarray, np.ndarray]:
    codes, n = codes_of([string])
    D = 1 << n
    k = np.zeros(D, dtype=np.uint64)
    m = np.zeros(D, dtype=np.complex128)
    lib().fpo_sparse_repr(_p(codes), n, _p(k), _p(m))
    return k, m


def _as2d(psi: np.ndarray) -> np.ndarray:
    return psi.reshape(psi.shape[0], 1) if psi.ndim == 1 else psi


def string_apply(string: str, psi, coeff: complex = 1.0) -> np.ndarray:
    psi = _c(psi)
    p2 = _as2d(psi)
    codes, n = codes_of([string])
    out = np.zeros_like(p2)
    c = complex(coeff)
    lib().fpo_string_apply_batch(_p(codes), n, p2.shape[1], _p(p2), _p(out), c.real, c.imag)
    return out.reshape(psi.shape)


def string_expectation(string: str, psi, coeff: complex = 1.0) -> np.ndarray:
    p2 = _as2d(_c(psi))
    codes, n = codes_of([string])
    ev = np.zeros(p2.shape[1], dtype=np.complex128)
    c = complex(coeff)
    lib().fpo_string_expectation(_p(codes), n, p2.shape[1], _p(p2), _p(ev), c.real, c.imag)
    return ev


def op_apply(strings, coeffs, psi) -> np.ndarray:
    psi = _c(psi)
    p2 = _as2d(psi)
    codes, n = codes_of(strings)
    c = _c(coeffs)
    out = np.zeros_like(p2)
    lib().fpo_op_apply(_p(codes), len(strings), n, _p(c), p2.shape[1], _p(p2), _p(out))
    return out.reshape(psi.shape)


def op_expectation(strings, coeffs, psi) -> np.ndarray:
    p2 = _as2d(_c(psi))
    codes, n = codes_of(strings)
    c = _c(coeffs)
    ev = np.zeros(p2.shape[1], dtype=np.complex128)
    lib().fpo_op_expectation(_p(codes), len(strings), n, _p(c), p2.shape[1], _p(p2), _p(ev))
    return ev


def summed_expectation(strings, h, psi) -> np.ndarray:
    """h: (P, K) complex; returns (K, S), or (K,) for 1-D psi."""
    psi = _c(psi)
    p2 = _as2d(psi)
    codes, n = codes_of(strings)
    h = _c(h)
    K = h.shape[1]
    out = np.zeros((K, p2.shape[1]), dtype=np.complex128)
    lib().fpo_summed_expectation(_p(codes), len(strings), n, _p(h), K, p2.shape[1], _p(p2), _p(out))
    return out[:, 0] if psi.ndim == 1 else out


def summed_apply(strings, h, psi) -> np.ndarray:
    psi = _c(psi)
    p2 = _as2d(psi)
    codes, n = codes_of(strings)
    h = _c(h)
    out = np.zeros_like(p2)
    lib().fpo_summed_apply(_p(codes), len(strings), n, _p(h), h.shape[1], p2.shape[1], _p(p2), _p(out))
    return out.reshape(psi.shape)


def summed_apply_weighted(strings, h, psi, data) -> np.ndarray:
    psi = _c(psi)
    p2 = _as2d(psi)
    codes, n = codes_of(strings)
    h = _c(h)
    data = _c(data, np.float64)
    d2 = data.reshape(data.shape[0], 1) if data.ndim == 1 else data
    out = np.zeros_like(p2)
    lib().fpo_summed_apply_weighted(
        _p(codes), len(strings), n, _p(h), h.shape[1], p2.shape[1], _p(p2), _p(d2), _p(out)
    )
    return out.reshape(psi.shape)


def summed_to_tensor(strings, h) -> np.ndarray:
    """Dense matrices (K, 2^n, 2^n) of the operators sum_j h(j,k) P_j."""
    codes, n = codes_of(strings)
    h = _c(h)
    K = h.shape[1]
    out = np.zeros((K, 1 << n, 1 << n), dtype=np.complex128)
    lib().fpo_summed_to_tensor(_p(codes), len(strings), n, _p(h), K, _p(out))
    return out


def summed_square(strings, h, sq_strings) -> np.ndarray:
    """Coefficients (A, K) of the squared operators over the strings
    sq_strings (SummedPauliOp::square); raises if a product is missing."""
    codes, n = codes_of(strings)
    sq_codes, n2 = codes_of(sq_strings)
    h = _c(h)
    K = h.shape[1]
    out = np.zeros((len(sq_strings), K), dtype=np.complex128)
    rc = lib().fpo_summed_square(_p(codes), len(strings), n, _p(h), K, _p(sq_codes), len(sq_strings), _p(out))
    if rc != 0:
        raise ValueError("a product of two strings is not among the squared strings")
    return out


def op_product(a_coeffs, a_strings, b_coeffs, b_strings) -> dict:
    """PauliOp product with equal strings merged (PauliOp operator*):
    {string: coefficient}, strings in order of first appearance."""
    ac, n = codes_of(a_strings)
    bc, n2 = codes_of(b_strings)
    if n != n2:
        raise ValueError("Mismatched dimensions for provided PauliOp")
    a = _c(a_coeffs)
    b = _c(b_coeffs)
    N = len(a_strings) * len(b_strings)
    codes = np.zeros((max(N, 1), max(n, 1)), dtype=np.uint8)
    coeffs = np.zeros(max(N, 1), dtype=np.complex128)
    cnt = lib().fpo_op_product(_p(ac), _p(a), len(a_strings), _p(bc), _p(b), len(b_strings), n, _p(codes), _p(coeffs))
    letters = "IXYZ"
    return {"".join(letters[c] for c in codes[k, :n]): coeffs[k] for k in range(cnt)}


# --------------------------------------------------------------------------
# dense construction (the reference tests' own oracle: kron of 2x2 matrices,
# tests/fast_pauli/... naive_pauli_converter; small n only)
# --------------------------------------------------------------------------

_PAULI = {
    "I": np.array([[1, 0], [0, 1]], dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def dense(string: str) -> np.ndarray:
    m = np.array([[1.0 + 0j]])
    for ch in string:
        m = np.kron(m, _PAULI[ch])
    return m


# --------------------------------------------------------------------------
# seeded synthetic inputs (configs of the headline workloads)
# --------------------------------------------------------------------------


def unit_norm_states(rng: np.random.Generator, D: int, S: int) -> np.ndarray:
    """re/im ~ N(0,1), each column normalised to unit 2-norm in float64."""
    psi = rng.standard_normal((D, S)) + 1j * rng.standard_normal((D, S))
    psi /= np.linalg.norm(psi, axis=0, keepdims=True)
    return np.ascontiguousarray(psi)


def uniform_strings(rng: np.random.Generator, n: int, P: int) -> list[str]:
    letters = np.array(list("IXYZ"))
    idx = rng.integers(0, 4, size=(P, n))
    return ["".join(letters[row]) for row in idx]
