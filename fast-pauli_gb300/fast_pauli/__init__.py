"""fast_pauli on GB300: a drop-in for the Pauli string / operator hot path of
qognitive/fast-pauli (``fast_pauli/__init__.py`` of the reference re-exports
the same names from its nanobind module).

``Pauli``, ``PauliString``, ``PauliOp``, ``SummedPauliOp`` and ``helpers``
come from the compiled module ``_fast_pauli``; their apply / expectation
methods run on the GPU (libfpg.so) and there is no CPU fallback: importing
fails loudly if the extension has not been built.
"""

from ._fast_pauli import (  # noqa: F401
    Pauli,
    PauliOp,
    PauliString,
    SummedPauliOp,
    helpers,
    release_cached_memory,
)


def from_qiskit(*args, **kwargs):  # pragma: no cover - qiskit is not installed here
    """qiskit interop (reference: fast_pauli/qiskit_helpers.py); needs qiskit."""
    from .qiskit_helpers import from_qiskit as _f

    return _f(*args, **kwargs)


def to_qiskit(*args, **kwargs):  # pragma: no cover
    """qiskit interop (reference: fast_pauli/qiskit_helpers.py); needs qiskit."""
    from .qiskit_helpers import to_qiskit as _f

    return _f(*args, **kwargs)
