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
from .qiskit_helpers import from_qiskit, to_qiskit  # noqa: F401  (qiskit itself is imported on use)
