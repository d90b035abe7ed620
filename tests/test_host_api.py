"""Host-side behaviour of the Python surface (no GPU needed): construction,
properties, string algebra, helpers, pickling and the ValueError contract,
mirroring the reference's tests (tests/fast_pauli/test_pauli.py,
test_pauli_string.py, test_pauli_op.py, test_summed_pauli_op.py)."""

from __future__ import annotations

import itertools
import pickle

import numpy as np
import pytest

import oracle
from conftest import golden

fp = pytest.importorskip("fast_pauli")


def test_pauli_cayley_table():
    # reference test_pauli.cpp:60-100: sigma_a sigma_b against dense products
    for a, b in itertools.product("IXYZ", repeat=2):
        phase, p = fp.Pauli(a) @ fp.Pauli(b)
        np.testing.assert_allclose(phase * oracle.dense(str(p)), oracle.dense(a) @ oracle.dense(b), atol=1e-15)


def test_pauli_ctor_errors_and_pickle():
    with pytest.raises(ValueError):
        fp.Pauli(4)
    with pytest.raises(ValueError):
        fp.Pauli("A")
    for c in "IXYZ":
        p = fp.Pauli(c)
        assert str(pickle.loads(pickle.dumps(p))) == c
        assert str(fp.Pauli("IXYZ".index(c))) == c


def test_pauli_string_basics():
    s = fp.PauliString("XYZI")
    assert s.n_qubits == 4 and s.dim == 16 and s.weight == 3 and str(s) == "XYZI"
    assert fp.PauliString().dim == 0
    assert str(fp.PauliString([fp.Pauli("X"), fp.Pauli(3)])) == "XZ"
    assert str(pickle.loads(pickle.dumps(s))) == "XYZI"
    with pytest.raises(ValueError):
        fp.PauliString("XQ")
    with pytest.raises(ValueError):
        fp.PauliString("XY") @ fp.PauliString("XYZ")


def test_pauli_string_products_match_dense():
    rng = np.random.default_rng(5)
    for _ in range(30):
        a, b = oracle.uniform_strings(rng, 4, 2)
        phase, p = fp.PauliString(a) @ fp.PauliString(b)
        np.testing.assert_allclose(phase * oracle.dense(str(p)), oracle.dense(a) @ oracle.dense(b), atol=1e-14)


def test_pauli_string_sum_and_difference():
    a, b = fp.PauliString("XY"), fp.PauliString("ZZ")
    s = a + b
    d = a - b
    assert s.pauli_strings_as_str == ["XY", "ZZ"] and s.coeffs == [1, 1]
    assert d.coeffs == [1, -1]


def test_pauli_op_construction_and_properties():
    po = fp.PauliOp([4j, 4j], ["III", "III"])
    assert po.dim == 8 and po.n_qubits == 3 and po.n_pauli_strings == 2
    assert po.pauli_strings_as_str == ["III", "III"]
    np.testing.assert_equal(po.coeffs, [4j, 4j])
    for empty in (fp.PauliOp(), fp.PauliOp([]), fp.PauliOp([], [])):
        assert empty.dim == 0 and empty.n_qubits == 0 and empty.n_pauli_strings == 0
    po = fp.PauliOp(np.array([1.0, 2.0j]), [fp.PauliString("XY"), fp.PauliString("ZI")])
    assert po.coeffs == [1, 2j]
    po = fp.PauliOp(["XX", "YY"])
    assert po.coeffs == [1, 1]


def test_pauli_op_exceptions():
    # reference test_pauli_op.py:886-946 (host-side checks)
    with pytest.raises(ValueError):
        fp.PauliOp(["ABC"])
    with pytest.raises(ValueError):
        fp.PauliOp(["XI", "XY", "XZ", "III"])
    with pytest.raises(ValueError):
        fp.PauliOp([1, 1], ["X", "YZ"])
    with pytest.raises(ValueError):
        fp.PauliOp([1, 2, 3], ["I", "X", "Y", "Z"])
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]) @ fp.PauliOp([1], ["III"])
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]) @ fp.PauliString("X")
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]) + fp.PauliOp([1], ["X"])
    with pytest.raises(ValueError):
        p = fp.PauliOp([-1, 1], ["IX", "YZ"])
        p += fp.PauliOp([1], ["Z"])
    with pytest.raises(ValueError):
        p = fp.PauliOp([-1, 1], ["IX", "YZ"])
        p -= fp.PauliOp([1], ["ZZZ"])
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]) + fp.PauliString("XXXX")
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]) - fp.PauliString("XXXX")
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]).extend(fp.PauliString("X"), 1j, dedupe=True)
    with pytest.raises(ValueError):
        fp.PauliOp([-1, 1], ["IX", "YZ"]).extend(fp.PauliOp([1j], ["XXX"]))


def _as_dict(op):
    d = {}
    for c, s in zip(op.coeffs, op.pauli_strings_as_str):
        d[s] = d.get(s, 0) + c
    return d


def _dense_op(op):
    n = op.n_qubits
    m = np.zeros((1 << n, 1 << n), dtype=complex)
    for c, s in zip(op.coeffs, op.pauli_strings_as_str):
        m += c * oracle.dense(s)
    return m


def test_pauli_op_algebra_matches_dense():
    rng = np.random.default_rng(9)
    a_s = oracle.uniform_strings(rng, 3, 6)
    b_s = oracle.uniform_strings(rng, 3, 5)
    a = fp.PauliOp(list(rng.standard_normal(6) + 1j * rng.standard_normal(6)), a_s)
    b = fp.PauliOp(list(rng.standard_normal(5) + 1j * rng.standard_normal(5)), b_s)
    # PauliOp @ PauliOp runs on the GPU: tests/test_gpu_product.py
    ps = fp.PauliString("XYZ")
    np.testing.assert_allclose(_dense_op(a @ ps), _dense_op(a) @ oracle.dense("XYZ"), atol=1e-12)
    np.testing.assert_allclose(_dense_op(ps @ a), oracle.dense("XYZ") @ _dense_op(a), atol=1e-12)
    np.testing.assert_allclose(_dense_op(a + b), _dense_op(a) + _dense_op(b), atol=1e-12)
    np.testing.assert_allclose(_dense_op(a - b), _dense_op(a) - _dense_op(b), atol=1e-12)
    np.testing.assert_allclose(_dense_op(a * 2j), 2j * _dense_op(a), atol=1e-12)
    np.testing.assert_allclose(_dense_op(3 * a), 3 * _dense_op(a), atol=1e-12)
    c = a.clone()
    c *= -1
    np.testing.assert_allclose(_dense_op(c), -_dense_op(a), atol=1e-12)
    c = a.clone()
    c.extend(fp.PauliString("III"), 2.0)
    np.testing.assert_allclose(_dense_op(c), _dense_op(a) + 2 * np.eye(8), atol=1e-12)
    f = rng.standard_normal(6) + 0j
    c = a.clone()
    c.scale(f)
    np.testing.assert_allclose(c.coeffs, np.array(a.coeffs) * f)
    with pytest.raises(ValueError):
        c.scale(np.ones(3, dtype=complex))


def test_pauli_op_pickle():
    op = fp.PauliOp([1, 1j, 2], ["I", "X", "Y"])
    u = pickle.loads(pickle.dumps(op))
    assert u.coeffs == op.coeffs and u.pauli_strings_as_str == op.pauli_strings_as_str


def test_summed_pauli_op_host_side():
    strings = fp.helpers.calculate_pauli_strings_max_weight(3, 2)
    P = len(strings)
    rng = np.random.default_rng(1)
    h = rng.standard_normal((P, 4)) + 1j * rng.standard_normal((P, 4))
    op = fp.SummedPauliOp(strings, h)
    assert op.dim == 8 and op.n_operators == 4 and op.n_pauli_strings == P
    np.testing.assert_array_equal(op.coeffs, h.T)  # getter returns (K, P)
    op2 = fp.SummedPauliOp([str(s) for s in strings], h)
    np.testing.assert_array_equal(op2.coeffs, h.T)
    new = rng.standard_normal((4, P)) + 0j
    op.coeffs = new
    np.testing.assert_array_equal(op.coeffs, new)
    with pytest.raises(ValueError):
        op.coeffs = np.ones((P, 4), dtype=complex)
    parts = op.split()
    assert len(parts) == 4
    for k, part in enumerate(parts):
        np.testing.assert_array_equal(part.coeffs, new[k])
    u = pickle.loads(pickle.dumps(op))
    np.testing.assert_array_equal(u.coeffs, op.coeffs)
    with pytest.raises(ValueError):
        fp.SummedPauliOp(["XX", "Y"], np.ones((2, 1)))
    with pytest.raises(ValueError):
        fp.SummedPauliOp(["XX", "YY"], np.ones((3, 1)))


def test_helpers_match_oracle_and_golden():
    g = golden("helpers.npz")
    for key in g.files:
        if key.startswith("max_weight_"):
            _, _, n, w = key.split("_")
            got = [str(s) for s in fp.helpers.calculate_pauli_strings_max_weight(int(n), int(w))]
            assert got == [str(x) for x in g[key]]
    assert fp.helpers.get_nontrivial_paulis(2) == oracle.get_nontrivial_paulis(2)
    assert [str(s) for s in fp.helpers.calculate_pauli_strings(5, 2)] == oracle.calculate_pauli_strings(5, 2)
    assert len(fp.helpers.calculate_pauli_strings_max_weight(14, 2)) == 862
