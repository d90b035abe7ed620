"""Conversions between fast_pauli and qiskit.quantum_info types.

Same behaviour as the reference's compatibility layer
(fast_pauli/qiskit_helpers.py:25-87):

* ``from_qiskit(SparsePauliOp)`` -> ``PauliOp`` with the operator's labels and
  coefficients, in the operator's order;
* ``to_qiskit(PauliOp)`` -> ``SparsePauliOp(labels, coeffs)``;
  ``to_qiskit(PauliString)`` -> ``Pauli(label)`` (phase exponent 0);
* any other type raises ``NotImplementedError``.

Labels mean the same thing on both sides: the leftmost character acts on the
most significant bit of the row index (qiskit's qubit n-1), so a label's
matrix is the Kronecker product of its letters' matrices from left to right.

qiskit is imported when a conversion is made, not when ``fast_pauli`` is
imported, so the package works without it; a conversion without qiskit
installed raises ``ImportError``.
"""

from __future__ import annotations

from typing import Any

from ._fast_pauli import PauliOp, PauliString


def _quantum_info():
    try:
        from qiskit.quantum_info import Pauli, SparsePauliOp
    except ImportError as e:  # pragma: no cover - depends on the environment
        raise ImportError("fast_pauli's qiskit conversions need qiskit (qiskit.quantum_info)") from e
    return Pauli, SparsePauliOp


def from_qiskit(qiskit_type: Any) -> Any:
    """Convert a qiskit ``SparsePauliOp`` to a ``PauliOp``."""
    _, SparsePauliOp = _quantum_info()
    if isinstance(qiskit_type, SparsePauliOp):
        pairs = qiskit_type.to_list(array=True)
        strings = [str(label) for label, _ in pairs]
        coeffs = [complex(c) for _, c in pairs]
        return PauliOp(coeffs, strings)
    raise NotImplementedError(f"Conversion from {type(qiskit_type)} to fast_pauli equivalent isn't supported.")


def to_qiskit(fast_pauli_type: Any) -> Any:
    """Convert a ``PauliOp`` to a qiskit ``SparsePauliOp``, or a
    ``PauliString`` to a qiskit ``Pauli``."""
    Pauli, SparsePauliOp = _quantum_info()
    if isinstance(fast_pauli_type, PauliOp):
        return SparsePauliOp(list(fast_pauli_type.pauli_strings_as_str), fast_pauli_type.coeffs)
    if isinstance(fast_pauli_type, PauliString):
        return Pauli(str(fast_pauli_type))
    raise NotImplementedError(f"Conversion from {type(fast_pauli_type)} to Qiskit equivalent isn't supported.")
