"""The reference's own Python parity grids, run through this library on the GPU.

* SummedPauliOp apply / apply_weighted / expectation_value over
  n_states in {1, 10, 1000} x n_operators in {1, 10, 100} x n_qubits in
  {1, 2, 6}, all strings of weight <= 2, coefficients and states drawn
  uniformly from [0, 1) as complex128 with zero imaginary part and states not
  normalised (tests/fast_pauli/test_summed_pauli_op.py:46-180); one state is
  passed as a 1-D array.
* PauliOp apply (1-D and batched) and expectation_value on the ordered string
  sets of tests/fast_pauli/test_pauli_op.py:172-320 (pauli_strings_with_size
  with its limits), random complex coefficients and states with uniform
  [0, 1) parts, and the integer / float input cases of those tests.

Each result is checked with the reference tests' own tolerance
(numpy.testing.assert_allclose, atol as in the reference, default rtol) and,
in addition, against the oracle within this repository's normwise bound."""

from __future__ import annotations

import itertools

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, normwise

pytestmark = pytest.mark.gpu

fp = pytest.importorskip("fast_pauli")

GRID = [(s, o, q) for s in (1, 10, 1000) for o in (1, 10, 100) for q in (1, 2, 6)]


def _grid_inputs(n_states, n_operators, n_qubits, seed):
    rng = np.random.default_rng(seed)
    strings = [str(s) for s in fp.helpers.calculate_pauli_strings_max_weight(n_qubits, 2)]
    coeffs = rng.random((len(strings), n_operators)).astype(np.complex128)
    psi = rng.random((1 << n_qubits, n_states)).astype(np.complex128)
    return rng, strings, coeffs, psi


def _dense_ops(strings, coeffs):
    mats = np.stack([oracle.dense(s) for s in strings])  # (P, D, D)
    return np.einsum("pk,pij->kij", coeffs, mats)  # (K, D, D)


@pytest.mark.parametrize("n_states,n_operators,n_qubits", GRID)
def test_summed_apply_grid(n_states, n_operators, n_qubits):
    _, strings, coeffs, psi = _grid_inputs(n_states, n_operators, n_qubits, 11 * n_states + n_operators + n_qubits)
    op = fp.SummedPauliOp(strings, coeffs)
    A = _dense_ops(strings, coeffs).sum(0)
    if n_states == 1:
        got = op.apply(psi[:, 0].copy())
        assert got.shape == (1 << n_qubits,)
        want = A @ psi[:, 0]
    else:
        got = op.apply(psi)
        want = A @ psi
    np.testing.assert_allclose(got, want, atol=1e-13)
    assert normwise(got, oracle.summed_apply(strings, coeffs, psi).reshape(got.shape)) < TOL_C128


@pytest.mark.parametrize("n_states,n_operators,n_qubits", GRID)
def test_summed_apply_weighted_grid(n_states, n_operators, n_qubits):
    rng, strings, coeffs, psi = _grid_inputs(n_states, n_operators, n_qubits, 13 * n_states + n_operators + n_qubits)
    data = rng.random((n_operators, n_states))
    op = fp.SummedPauliOp(strings, coeffs)
    mats = _dense_ops(strings, coeffs)
    want = np.einsum("kij,jt,kt->it", mats, psi, data)
    if n_states == 1:
        got = op.apply_weighted(psi[:, 0].copy(), data[:, 0].copy())
        assert got.shape == (1 << n_qubits,)
        want = want[:, 0]
    else:
        got = op.apply_weighted(psi, data)
    np.testing.assert_allclose(got, want, atol=1e-13)
    assert normwise(got, oracle.summed_apply_weighted(strings, coeffs, psi, data).reshape(got.shape)) < TOL_C128


@pytest.mark.parametrize("n_states,n_operators,n_qubits", GRID)
def test_summed_expectation_grid(n_states, n_operators, n_qubits):
    _, strings, coeffs, psi = _grid_inputs(n_states, n_operators, n_qubits, 17 * n_states + n_operators + n_qubits)
    op = fp.SummedPauliOp(strings, coeffs)
    mats = _dense_ops(strings, coeffs)
    want = np.einsum("it,kij,jt->kt", psi.conj(), mats, psi)
    if n_states == 1:
        got = op.expectation_value(psi[:, 0].copy())
        assert got.shape == (n_operators,)
        want = want[:, 0]
    else:
        got = op.expectation_value(psi)
        assert got.shape == (n_operators, n_states)
    np.testing.assert_allclose(got, want, atol=1e-13)
    assert normwise(got, oracle.summed_expectation(strings, coeffs, psi).reshape(got.shape)) < TOL_C128


# ----------------------------------------------------------------- PauliOp


def _ordered_strings(size, limit=1000):
    out = []
    for s in itertools.product("IXYZ", repeat=size):
        if limit and len(out) >= limit:
            break
        out.append("".join(s))
    return out


STRING_SETS = {
    "n2": lambda: _ordered_strings(2),
    "n3": lambda: _ordered_strings(3),
    "n4": lambda: _ordered_strings(4),
    "n7_128": lambda: _ordered_strings(7, 128),
    "n8_first100": lambda: _ordered_strings(8, 200)[:100],
    "n8_next100": lambda: _ordered_strings(8, 200)[100:],
    "n10_64": lambda: _ordered_strings(10, 64),
}


def _rand_complex(rng, *shape):
    return rng.random(shape) + 1j * rng.random(shape)


def _dense_op(coeffs, strings):
    return np.einsum("p,pij->ij", coeffs, np.stack([oracle.dense(s) for s in strings]))


@pytest.mark.parametrize("name", list(STRING_SETS))
def test_pauli_op_apply_expectation_string_sets(name):
    rng = np.random.default_rng(321)
    strings = STRING_SETS[name]()
    coeffs = _rand_complex(rng, len(strings))
    po = fp.PauliOp(coeffs, strings)
    A = _dense_op(coeffs, strings)
    # 1-D state
    psi = _rand_complex(rng, po.dim)
    np.testing.assert_allclose(po.apply(psi), A @ psi, atol=1e-15)
    np.testing.assert_allclose(po.expectation_value(psi), (A @ psi) @ psi.conj(), atol=1e-15)
    # a batch of states with a state count drawn like the reference's (0..99)
    n_states = int(100 * rng.random())
    psis = _rand_complex(rng, po.dim, n_states)
    np.testing.assert_allclose(po.apply(psis), A @ psis, atol=1e-15)
    np.testing.assert_allclose(po.expectation_value(psis), np.einsum("it,ij,jt->t", psis.conj(), A, psis), atol=1e-15)
    if n_states:
        assert normwise(po.apply(psis), oracle.op_apply(strings, coeffs, psis)) < TOL_C128
        assert normwise(po.expectation_value(psis), oracle.op_expectation(strings, coeffs, psis)) < TOL_C128


def test_pauli_op_integer_and_float_inputs():
    """The fixed cases of the reference's PauliOp tests: integer and float
    arrays and lists are converted to complex128 like its bindings do."""
    np.testing.assert_allclose(fp.PauliOp([1, 2], ["IXYZ", "ZYXI"]).apply(np.zeros(16)), np.zeros(16), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([0.5, 0.5], ["III", "III"]).apply(np.arange(8)), np.arange(8), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1j], ["XYZ"]).apply(np.ones(8)), oracle.dense("XYZ").sum(1) * 1j,
                               atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1, 2], ["IXYZ", "ZYXI"]).apply(np.zeros((16, 16))), np.zeros((16, 16)),
                               atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([0.5, 0.5], ["III", "III"]).apply(np.arange(64).reshape(8, 8)),
                               np.arange(64).reshape(8, 8), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1j], ["XYZ"]).apply(np.eye(8)), 1j * oracle.dense("XYZ"), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1, 2], ["IXYZ", "ZYXI"]).expectation_value(np.zeros(16)), 0, atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1, 2], ["IXYZ", "ZYXI"]).expectation_value(np.zeros((16, 16))),
                               np.zeros(16), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1, 1], ["III", "III"]).expectation_value(np.arange(8)),
                               2 * np.square(np.arange(8)).sum(), atol=1e-15)
    np.testing.assert_allclose(fp.PauliOp([1, 1], ["III", "III"]).expectation_value(np.arange(64).reshape(8, 8)),
                               2 * np.square(np.arange(64)).reshape(8, 8).sum(0), atol=1e-15)
