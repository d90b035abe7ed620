"""GPU PauliOp products (fpg_op_product): against dense matrices at small n
(the reference's own check, test_pauli_op.py:508-570) and, at larger sizes,
against the pairwise products of the host PauliString @ PauliString
(itself checked against dense matrices in test_host_api.py)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import golden

pytestmark = pytest.mark.gpu

fp = pytest.importorskip("fast_pauli")


def _dense_op(op):
    n = op.n_qubits
    m = np.zeros((1 << n, 1 << n), dtype=complex)
    for c, s in zip(op.coeffs, op.pauli_strings_as_str):
        m += c * oracle.dense(s)
    return m


def _strs(a):
    return [str(x) for x in a]


def _masks(s):
    n = len(s)
    x = z = 0
    for q, ch in enumerate(s):
        b = n - 1 - q
        if ch in "XY":
            x |= 1 << b
        if ch in "YZ":
            z |= 1 << b
    return x, z


def _pairwise(a_c, a_s, b_c, b_s):
    out = {}
    for ca, sa in zip(a_c, a_s):
        pa = fp.PauliString(sa)
        for cb, sb in zip(b_c, b_s):
            phase, p = pa @ fp.PauliString(sb)
            out[str(p)] = out.get(str(p), 0) + phase * ca * cb
    return out


def _rand_op(rng, n, P):
    s = oracle.uniform_strings(rng, n, P)
    c = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    return c, s


@pytest.mark.parametrize("n,Pa,Pb", [(1, 3, 4), (2, 6, 5), (3, 6, 5), (5, 12, 9)])
def test_product_matches_dense(n, Pa, Pb):
    rng = np.random.default_rng(10 * n + Pa)
    ac, as_ = _rand_op(rng, n, Pa)
    bc, bs = _rand_op(rng, n, Pb)
    a, b = fp.PauliOp(list(ac), as_), fp.PauliOp(list(bc), bs)
    got = a @ b
    np.testing.assert_allclose(_dense_op(got), _dense_op(a) @ _dense_op(b), atol=1e-12)
    # each string once
    assert len(set(got.pauli_strings_as_str)) == got.n_pauli_strings


def test_product_reference_cases():
    # reference test_pauli_op.py:508-530: identity factors
    ixyz = fp.PauliOp([1, 1j, -1, -1j], ["I", "X", "Y", "Z"])
    ident = fp.PauliOp([1], ["I"])
    np.testing.assert_allclose((ident @ ident).to_tensor(), np.eye(2), atol=1e-15)
    np.testing.assert_allclose((ixyz @ ident).to_tensor(), ixyz.to_tensor(), atol=1e-15)
    np.testing.assert_allclose((ident @ ixyz @ ident).to_tensor(), ixyz.to_tensor(), atol=1e-15)
    # chains
    rng = np.random.default_rng(5)
    lc, ls = _rand_op(rng, 3, 7)
    rc, rs = _rand_op(rng, 3, 4)
    l_op, r_op = fp.PauliOp(list(lc), ls), fp.PauliOp(list(rc), rs)
    want = _dense_op(l_op) @ _dense_op(r_op) @ _dense_op(l_op) @ _dense_op(r_op)
    np.testing.assert_allclose(_dense_op(l_op @ r_op @ l_op @ r_op), want, atol=1e-11)


@pytest.mark.parametrize("case", ["ab", "ww"])
def test_product_vs_reference_golden(case):
    # the reference's output (tests/golden/op_product.npz) lists a string once
    # per OpenMP thread map; merged it must equal ours, where each string
    # appears once
    g = golden("op_product.npz")
    a = ("a", "b") if case == "ab" else ("w", "w")
    got = fp.PauliOp(list(g[f"{a[0]}_coeffs"]), _strs(g[f"{a[0]}_strings"])) @ fp.PauliOp(
        list(g[f"{a[1]}_coeffs"]), _strs(g[f"{a[1]}_strings"])
    )
    want = {}
    for s, c in zip(_strs(g[f"{case}_strings"]), g[f"{case}_coeffs"]):
        want[s] = want.get(s, 0) + c
    strs = got.pauli_strings_as_str
    assert len(set(strs)) == len(strs) and sorted(strs) == sorted(want)
    g_c = dict(zip(strs, got.coeffs))
    assert max(abs(g_c[s] - want[s]) for s in want) < 1e-12


@pytest.mark.parametrize("n,Pa,Pb", [(10, 300, 200), (40, 50, 40), (33, 60, 70)])
def test_product_matches_pairwise_products(n, Pa, Pb):
    """Sizes past the dense check, keys wider than 64 bits (n > 32), repeated
    strings in the inputs; the result is sorted by (x, z), each string once,
    and its coefficients match the sums of the pairwise products."""
    rng = np.random.default_rng(n + Pa)
    ac, as_ = _rand_op(rng, n, Pa)
    bc, bs = _rand_op(rng, n, Pb)
    as_[3] = as_[1]  # a repeated string
    got = fp.PauliOp(list(ac), as_) @ fp.PauliOp(list(bc), bs)
    want = _pairwise(ac, as_, bc, bs)
    orc = oracle.op_product(ac, as_, bc, bs)
    assert max(abs(orc[s] - want[s]) for s in want) <= 1e-12 * max(1.0, max(abs(v) for v in want.values()))
    strs = got.pauli_strings_as_str
    assert sorted(strs) == sorted(want)
    keys = [_masks(s) for s in strs]
    assert keys == sorted(keys)
    g = np.array(got.coeffs)
    w = np.array([want[s] for s in strs])
    assert np.abs(g - w).max() <= 1e-12 * max(1.0, np.abs(w).max())


def test_product_deterministic_and_cancelling():
    # A @ A for a Hermitian A: anticommuting pairs cancel exactly (their
    # products come in pair order, so equal runs sum the same way each call)
    rng = np.random.default_rng(8)
    s = oracle.uniform_strings(rng, 6, 40)
    c = rng.standard_normal(40)
    a = fp.PauliOp(list(c.astype(complex)), s)
    r1, r2 = a @ a, a @ a
    assert r1.pauli_strings_as_str == r2.pauli_strings_as_str
    np.testing.assert_array_equal(np.array(r1.coeffs), np.array(r2.coeffs))
    np.testing.assert_allclose(_dense_op(r1), _dense_op(a) @ _dense_op(a), atol=1e-11)
