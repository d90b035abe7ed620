"""Parity at the full size of the two headline SummedPauliOp workloads.

* n = 14, the 861 weight <= 2 strings, K = 1000, 16384 x 1024 complex128
  states: exactly the inputs the benchmark times (same generator and seed),
  float64 path against the float64 oracle over the whole (1000, 1024) output.
* n = 18, the 1431 weight <= 2 strings, K = 1000, 262144 x 512 states in
  complex64 (the mixed-precision path), against the float64 oracle evaluated
  on the float64 states before their conversion to complex64, on a slice of
  the columns (every output column depends only on its own state column, so a
  slice checks the same kernels and contraction on the full-size launch).

Reference: SummedPauliOp::expectation_value,
fast_pauli/cpp/include/__summed_pauli_op.hpp:520-614."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, TOL_MIXED_W2, normwise

pytestmark = pytest.mark.gpu


def _problem(n, K, S, seed):
    import bench

    return bench.weight2_problem(n=n, K=K, S=S, seed=seed)


def test_weight2_n14_full_size_float64_vs_oracle():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    n, K, S = 14, 1000, 1024
    strings, h, psi = _problem(n, K, S, seed=1002)
    assert len(strings) == 861 and psi.shape == (1 << n, S)
    L = _abi.lib()
    op = _abi.Operator(strings)
    dh = torch.from_numpy(h).cuda()
    out = torch.zeros((K, S), dtype=torch.complex128, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, psi.data_ptr(), out.data_ptr(), S, _abi.FPG_C128, st))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    op.close()
    want = oracle.summed_expectation(strings, h, psi.cpu().numpy())
    err = normwise(got, want)
    assert err < TOL_C128, err
    # the public API on the same device tensors gives the same result
    import fast_pauli as fp

    api = fp.SummedPauliOp(strings, h).expectation_value(psi).cpu().numpy()
    assert normwise(api, want) < TOL_C128


def test_weight2_n18_full_size_mixed_vs_float64_oracle():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    n, K, S = 18, 1000, 512
    strings, h, psi = _problem(n, K, S, seed=1003)
    assert len(strings) == 1431
    L = _abi.lib()
    op = _abi.Operator(strings)
    h64 = torch.from_numpy(h).to(torch.complex64).cuda()
    psi64 = psi.to(torch.complex64)
    # float64 copy of a column slice for the oracle, taken before psi goes
    cols = np.r_[0:24, S // 2 : S // 2 + 8, S - 32 : S]
    psi_slice = psi[:, torch.from_numpy(cols).cuda()].cpu().numpy()
    del psi
    torch.cuda.empty_cache()
    out = torch.zeros((K, S), dtype=torch.complex64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(L.fpg_summed_expect(op.handle, h64.data_ptr(), K, psi64.data_ptr(), out.data_ptr(), S, _abi.FPG_C64, st))
    torch.cuda.synchronize()
    got = out.cpu().numpy()[:, cols].astype(np.complex128)
    op.close()
    want = oracle.summed_expectation(strings, h, psi_slice)
    err = normwise(got, want)
    assert err < TOL_MIXED_W2, err
