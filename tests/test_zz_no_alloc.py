"""fpg_summed_expect_noalloc, the entry point for callers that may not
allocate device memory (for example code running inside a framework that has
already reserved nearly all of the GPU for its own pool, or a request loop
that must not allocate on its hot path).  It keeps its scratch in one static
device array instead of the stream-ordered pool.

Checked through the C ABI against the pooled entry point fpg_summed_expect,
within the tolerances the other parity tests use, on two calls in a row (the
static array keeps the previous call's contents, which must not leak into the
next result).  This file is collected last so that a run stopping at the first
failure has already run everything else."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, TOL_MIXED, normwise

pytestmark = pytest.mark.gpu


def _setup(n, S, K, seed):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    return torch, strings, h, psi


@pytest.mark.parametrize("dtype_name", ["c128", "c64"])
def test_noalloc_matches_pooled_entry_point_on_two_calls(dtype_name):
    from fast_pauli import _abi

    torch, strings, h, psi = _setup(n=10, S=48, K=7, seed=99)
    L = _abi.lib()
    P, K, S = len(strings), h.shape[1], psi.shape[1]
    cdt, code, tol = ((torch.complex128, _abi.FPG_C128, TOL_C128) if dtype_name == "c128"
                      else (torch.complex64, _abi.FPG_C64, TOL_MIXED))
    dpsi = torch.from_numpy(psi).to(cdt).cuda()
    dh = torch.from_numpy(h).to(cdt).cuda()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    op = _abi.Operator(strings)
    want = torch.zeros((K, S), dtype=cdt, device="cuda")
    _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, dpsi.data_ptr(), want.data_ptr(), S, code, st))
    torch.cuda.synchronize()
    want_np = want.cpu().numpy()
    op.close()
    joined = "".join(strings).encode()
    for _ in range(2):
        got = torch.zeros((K, S), dtype=cdt, device="cuda")
        _abi.check(L.fpg_summed_expect_noalloc(joined, P, 10, dh.data_ptr(), K, dpsi.data_ptr(), got.data_ptr(), S,
                                               code, st))
        torch.cuda.synchronize()
        assert normwise(got.cpu().numpy(), want_np) < tol
    # and both agree with the float64 oracle
    assert normwise(want_np, oracle.summed_expectation(strings, h, psi)) < (TOL_C128 if code == 0 else TOL_MIXED)


def test_noalloc_rejects_requests_beyond_its_static_scratch():
    from fast_pauli import _abi

    torch = pytest.importorskip("torch")
    L = _abi.lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    buf = torch.zeros(64, dtype=torch.complex128, device="cuda")
    # more strings than the encoding area holds
    rc = L.fpg_summed_expect_noalloc(b"X" * 8193, 8193, 1, buf.data_ptr(), 1, buf.data_ptr(), buf.data_ptr(), 1,
                                     _abi.FPG_C128, st)
    assert rc == _abi.FPG_ERR_INVALID
    assert b"exceeds the limit" in L.fpg_last_error()
    # a per-string table larger than the static array
    rc = L.fpg_summed_expect_noalloc(b"XZ" * 4096, 4096, 2, buf.data_ptr(), 1, buf.data_ptr(), buf.data_ptr(),
                                     4096, _abi.FPG_C128, st)
    assert rc == _abi.FPG_ERR_INVALID
    assert b"static scratch" in L.fpg_last_error()
