"""The CPU oracle pinned against the reference: golden vectors produced by the
reference's own C++ implementation (tests/golden/make_golden.py) and the
known-answer tests of the reference's unit tests."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import golden, normwise


def test_sparse_repr_golden_bit_exact():
    g = golden("sparse_repr.npz")
    for s in g["strings"]:
        s = str(s)
        k, m = oracle.sparse_repr(s)
        np.testing.assert_array_equal(k, g[f"cols_{s}"])
        np.testing.assert_array_equal(m, g[f"vals_{s}"])


def test_sparse_repr_matches_dense_kron():
    # reference test_pauli_string.cpp:194-215 / test_pauli_string.py:430
    for s in ["X", "Y", "Z", "XY", "YZX", "IYZI", "ZXYIY"]:
        k, m = oracle.sparse_repr(s)
        d = oracle.dense(s)
        D = len(k)
        np.testing.assert_array_equal(np.count_nonzero(d, axis=1), np.ones(D))
        np.testing.assert_allclose(d[np.arange(D), k.astype(np.int64)], m, atol=0)


def test_helper_ordering_known_answers():
    # reference test_pauli_helpers.cpp:120-166
    r = oracle.calculate_pauli_strings(4, 2)
    assert len(r) == 54 and r[0] == "XXII" and r[1] == "XIXI" and r[53] == "IIZZ"
    assert oracle.calculate_pauli_strings_max_weight(2, 1) == ["II", "XI", "IX", "YI", "IY", "ZI", "IZ"]
    assert len(oracle.calculate_pauli_strings_max_weight(4, 2)) == 67
    assert len(oracle.calculate_pauli_strings_max_weight(12, 2)) == 631
    g = golden("helpers.npz")
    for key in g.files:
        if key.startswith("max_weight_"):
            _, _, n, w = key.split("_")
            assert oracle.calculate_pauli_strings_max_weight(int(n), int(w)) == [str(x) for x in g[key]]
        else:
            _, n, w = key.split("_")
            assert len(oracle.calculate_pauli_strings_max_weight(int(n), int(w))) == int(g[key])


def test_pauli_op_apply_n10_golden():
    g = golden("pauli_op_apply_n10.npz")
    got = oracle.op_apply([str(s) for s in g["strings"]], g["coeffs"], g["states"])
    assert normwise(got, g["out"]) < 1e-14


def test_small_methods_golden():
    g = golden("small_methods.npz")
    s = [str(x) for x in g["strings"]]
    c = complex(g["c"])
    psi, psi1 = g["states"], g["state1"]
    checks = {
        "string_apply_2d": oracle.string_apply(s[0], psi, c),
        # the reference's 1-D PauliString.apply ignores the coefficient
        "string_apply_1d": oracle.string_apply(s[0], psi1),
        "string_expectation": oracle.string_expectation(s[1], psi, c),
        "op_apply": oracle.op_apply(s, g["coeffs"], psi),
        "op_expectation": oracle.op_expectation(s, g["coeffs"], psi),
        "summed_expectation": oracle.summed_expectation(s, g["h"], psi),
        "summed_apply": oracle.summed_apply(s, g["h"], psi),
        "summed_apply_weighted": oracle.summed_apply_weighted(s, g["h"], psi, g["data"]),
    }
    for k, v in checks.items():
        assert normwise(v, g[k]) < 1e-14, k


@pytest.mark.parametrize("name", ["summed_square.npz", "summed_square_n6.npz"])
def test_summed_square_golden(name):
    g = golden(name)
    got = oracle.summed_square([str(x) for x in g["strings"]], g["h"], [str(x) for x in g["sq_strings"]])
    assert normwise(got, g["sq_h"]) < 1e-14
    # the squared set is the helper's max-weight set
    n = len(str(g["strings"][0]))
    w = max(sum(c != "I" for c in str(x)) for x in g["strings"])
    assert [str(x) for x in g["sq_strings"]] == oracle.calculate_pauli_strings_max_weight(n, min(n, 2 * w))


def test_summed_to_tensor_matches_dense_kron():
    rng = np.random.default_rng(12)
    strings = oracle.uniform_strings(rng, 4, 9) + ["IIII"]
    h = rng.standard_normal((10, 3)) + 1j * rng.standard_normal((10, 3))
    want = np.stack([sum(h[j, k] * oracle.dense(s) for j, s in enumerate(strings)) for k in range(3)])
    assert normwise(oracle.summed_to_tensor(strings, h), want) < 1e-15


def test_summed_square_missing_product_is_reported():
    with pytest.raises(ValueError):
        oracle.summed_square(["XI", "IZ"], np.ones((2, 1)), ["II", "XI", "IZ"])  # XZ missing


def test_summed_expectation_weight2_n8_golden():
    g = golden("summed_expectation_weight2_n8.npz")
    got = oracle.summed_expectation([str(x) for x in g["strings"]], g["h"], g["states"])
    assert normwise(got, g["out"]) < 1e-14


def test_expectation_against_dense_small():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3):
        psi = oracle.unit_norm_states(rng, 1 << n, 4)
        for s in oracle.calculate_pauli_strings_max_weight(n, n):
            want = np.einsum("it,ij,jt->t", psi.conj(), oracle.dense(s), psi)
            np.testing.assert_allclose(oracle.string_expectation(s, psi), want, atol=1e-14)


@pytest.mark.parametrize("ref_available", [True])
def test_restatement_matches_reference_when_present(ref_available):
    from oracle import ref

    if not ref.available():
        pytest.skip("reference oracle not built on this machine")
    rng = np.random.default_rng(11)
    strings = oracle.uniform_strings(rng, 7, 30)
    h = rng.standard_normal((30, 4)) + 1j * rng.standard_normal((30, 4))
    psi = oracle.unit_norm_states(rng, 128, 9)
    data = rng.standard_normal((4, 9))
    assert normwise(oracle.summed_expectation(strings, h, psi), ref.summed_expectation(strings, h, psi)) < 1e-14
    assert normwise(oracle.summed_apply_weighted(strings, h, psi, data),
                    ref.summed_apply_weighted(strings, h, psi, data)) < 1e-14


def _merged(strings, coeffs):
    d = {}
    for s, c in zip(strings, coeffs):
        d[str(s)] = d.get(str(s), 0) + c
    return d


@pytest.mark.parametrize("case", ["ab", "ww"])
def test_op_product_golden(case):
    # the reference's PauliOp operator* lists a string once per OpenMP thread
    # map; merged, it must equal the oracle's single map
    g = golden("op_product.npz")
    if case == "ab":
        got = oracle.op_product(g["a_coeffs"], g["a_strings"], g["b_coeffs"], g["b_strings"])
    else:
        got = oracle.op_product(g["w_coeffs"], g["w_strings"], g["w_coeffs"], g["w_strings"])
    want = _merged(g[f"{case}_strings"], g[f"{case}_coeffs"])
    assert sorted(got) == sorted(want)
    assert max(abs(got[s] - want[s]) for s in want) < 1e-12


def test_op_product_matches_dense():
    rng = np.random.default_rng(12)
    for n in (1, 2, 3):
        a_s, b_s = oracle.uniform_strings(rng, n, 5), oracle.uniform_strings(rng, n, 4)
        a_c = rng.standard_normal(5) + 1j * rng.standard_normal(5)
        b_c = rng.standard_normal(4) + 1j * rng.standard_normal(4)
        got = oracle.op_product(a_c, a_s, b_c, b_s)
        m = sum(c * oracle.dense(s) for s, c in got.items())
        want = sum(c * oracle.dense(s) for s, c in zip(a_s, a_c)) @ sum(c * oracle.dense(s) for s, c in zip(b_s, b_c))
        np.testing.assert_allclose(m, want, atol=1e-13)
