"""qiskit interop (fast_pauli.from_qiskit / to_qiskit), following the
reference's tests/fast_pauli/test_qiskit_interface.py: a PauliOp goes to a
SparsePauliOp and back unchanged, and a PauliString becomes a Pauli with
phase exponent 0, the same qubit count and the same dense matrix.

qiskit is not installed here, so ``qiskit.quantum_info`` is replaced by a
minimal stand-in with the parts of the qiskit API the conversions use
(SparsePauliOp(labels, coeffs), SparsePauliOp.to_list(array=True),
Pauli(label) with .phase, .num_qubits, .to_matrix()).  When qiskit is
installed, the same tests run against it."""

from __future__ import annotations

import itertools
import sys
import types

import numpy as np
import pytest

import oracle

fp = pytest.importorskip("fast_pauli")


def _stand_in_quantum_info():
    class Pauli:
        def __init__(self, label):
            self.label = str(label)
            self.phase = 0
            self.num_qubits = len(self.label)

        def to_matrix(self):
            return oracle.dense(self.label)

    class SparsePauliOp:
        def __init__(self, labels, coeffs):
            self.labels = [str(x) for x in labels]
            self.coeffs = np.asarray(coeffs, dtype=np.complex128).copy()

        def to_list(self, array=False):
            pairs = list(zip(self.labels, self.coeffs))
            if array:
                out = np.empty(len(pairs), dtype=object)
                out[:] = [tuple(p) for p in pairs]
                return out
            return pairs

    mod = types.ModuleType("qiskit.quantum_info")
    mod.Pauli, mod.SparsePauliOp = Pauli, SparsePauliOp
    return mod


@pytest.fixture
def quantum_info(monkeypatch):
    try:
        import qiskit.quantum_info as qi  # noqa: F401

        return qi
    except ImportError:
        qi = _stand_in_quantum_info()
        pkg = types.ModuleType("qiskit")
        pkg.quantum_info = qi
        monkeypatch.setitem(sys.modules, "qiskit", pkg)
        monkeypatch.setitem(sys.modules, "qiskit.quantum_info", qi)
        return qi


def _strings(size, limit=1000):
    return ["".join(s) for s in itertools.islice(itertools.product("IXYZ", repeat=size), limit)]


@pytest.mark.parametrize("size", [1, 2, 3, 4, 5])
def test_pauli_op_round_trip(quantum_info, size):
    rng = np.random.default_rng(321)
    paulis = _strings(size)
    coeffs = rng.random(len(paulis)) + 1j * rng.random(len(paulis))
    op = fp.PauliOp(coeffs, paulis)
    q_op = fp.to_qiskit(op)
    assert isinstance(q_op, quantum_info.SparsePauliOp)
    back = fp.from_qiskit(q_op)
    np.testing.assert_allclose(op.coeffs, back.coeffs)
    np.testing.assert_array_equal(op.pauli_strings_as_str, back.pauli_strings_as_str)


@pytest.mark.parametrize("n_qubits", [1, 2, 3, 4])
def test_pauli_string_to_qiskit(quantum_info, n_qubits):
    for ps in _strings(n_qubits):
        pauli = fp.PauliString(ps)
        q = fp.to_qiskit(pauli)
        assert isinstance(q, quantum_info.Pauli)
        assert q.phase == 0
        assert pauli.n_qubits == q.num_qubits


@pytest.mark.gpu
@pytest.mark.parametrize("n_qubits", [1, 2, 3, 4])
def test_pauli_string_to_qiskit_dense_matrix(quantum_info, n_qubits):
    # PauliString.to_tensor runs on the GPU
    for ps in _strings(n_qubits):
        pauli = fp.PauliString(ps)
        np.testing.assert_allclose(pauli.to_tensor(), fp.to_qiskit(pauli).to_matrix())


def test_unsupported_types_raise(quantum_info):
    with pytest.raises(NotImplementedError):
        fp.to_qiskit(fp.SummedPauliOp(["XY"], np.ones((1, 2), dtype=complex)))
    with pytest.raises(NotImplementedError):
        fp.from_qiskit(quantum_info.Pauli("XY"))
    with pytest.raises(NotImplementedError):
        fp.from_qiskit("XY")
