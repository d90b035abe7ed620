"""pytest configuration: paths, the ``gpu`` marker and shared helpers."""

from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fast-pauli_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name))


def normwise(got, want) -> float:
    """max|got - want| / max|want| over the whole array (0 if want is 0)."""
    got = np.asarray(got)
    want = np.asarray(want)
    den = np.abs(want).max() if want.size else 0.0
    num = np.abs(got - want).max() if want.size else 0.0
    return float(num / den) if den > 0 else float(num)


# float64 GPU path vs the float64 oracle (normwise relative)
TOL_C128 = 1e-12
# mixed path (complex64 storage, float32 arithmetic) vs the float64 oracle:
# expectation values of the weight <= 2 operator sets, the mixed-precision
# target (<= 1e-6 relative to float64)
TOL_MIXED_W2 = 1e-6
# mixed path elsewhere: apply / apply_weighted outputs (complex64 results),
# uniform random strings, square and the batch and serving paths
TOL_MIXED = 1e-5
