"""fpg_summed_expect_noalloc, the entry point for callers that may not
allocate device memory (for example code running inside a framework that has
already reserved nearly all of the GPU for its own pool, or a request loop
that must not allocate on its hot path).  It keeps its scratch in one static
device array instead of the stream-ordered pool.

Checked through the C ABI against the pooled entry point fpg_summed_expect,
within the tolerances the other parity tests use, on two calls in a row with
different inputs (the static array keeps the previous call's contents, which
must not leak into the next result).  This file is collected last so that a run stopping at the first
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


def _pooled(L, _abi, torch, strings, dh, K, dpsi, S, code, cdt, st):
    op = _abi.Operator(strings)
    want = torch.zeros((K, S), dtype=cdt, device="cuda")
    _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, dpsi.data_ptr(), want.data_ptr(), S, code, st))
    torch.cuda.synchronize()
    op.close()
    return want.cpu().numpy()


def _noalloc(L, _abi, torch, strings, n, dh, K, dpsi, S, code, cdt, st):
    got = torch.zeros((K, S), dtype=cdt, device="cuda")
    _abi.check(L.fpg_summed_expect_noalloc("".join(strings).encode(), len(strings), n, dh.data_ptr(), K,
                                           dpsi.data_ptr(), got.data_ptr(), S, code, st))
    torch.cuda.synchronize()
    return got.cpu().numpy()


@pytest.mark.parametrize("dtype_name", ["c128", "c64"])
def test_noalloc_matches_pooled_entry_point_on_two_calls(dtype_name):
    """Two calls in a row with different inputs: the second call has fewer
    strings in another order, more states and new amplitudes, so a table
    entry or an encoding record left over from the first call would change
    its result."""
    from fast_pauli import _abi

    torch, strings, h, psi = _setup(n=10, S=48, K=7, seed=99)
    L = _abi.lib()
    P, K, S = len(strings), h.shape[1], psi.shape[1]
    cdt, code, tol = ((torch.complex128, _abi.FPG_C128, TOL_C128) if dtype_name == "c128"
                      else (torch.complex64, _abi.FPG_C64, TOL_MIXED))
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dpsi = torch.from_numpy(psi).to(cdt).cuda()
    dh = torch.from_numpy(h).to(cdt).cuda()
    want1 = _pooled(L, _abi, torch, strings, dh, K, dpsi, S, code, cdt, st)
    got1 = _noalloc(L, _abi, torch, strings, 10, dh, K, dpsi, S, code, cdt, st)
    assert normwise(got1, want1) < tol
    assert normwise(want1, oracle.summed_expectation(strings, h, psi)) < (TOL_C128 if code == 0 else TOL_MIXED)

    rng = np.random.default_rng(7)
    pick = rng.permutation(P)[: P // 3]
    strings2 = [strings[i] for i in pick]
    K2, S2 = 3, 61
    h2 = (rng.standard_normal((len(strings2), K2)) + 1j * rng.standard_normal((len(strings2), K2))) / 4
    psi2 = oracle.unit_norm_states(rng, 1 << 10, S2)
    dpsi2 = torch.from_numpy(psi2).to(cdt).cuda()
    dh2 = torch.from_numpy(h2).to(cdt).cuda()
    want2 = _pooled(L, _abi, torch, strings2, dh2, K2, dpsi2, S2, code, cdt, st)
    got2 = _noalloc(L, _abi, torch, strings2, 10, dh2, K2, dpsi2, S2, code, cdt, st)
    assert normwise(got2, want2) < tol
    assert normwise(want2, oracle.summed_expectation(strings2, h2, psi2)) < (TOL_C128 if code == 0 else TOL_MIXED)


def test_noalloc_refuses_a_capturing_stream():
    """The encoding is copied from host arrays that the next call
    overwrites, so a call made while the stream is being captured into a
    CUDA graph is refused instead of recording those copies."""
    from fast_pauli import _abi

    torch = pytest.importorskip("torch")
    L = _abi.lib()
    s = torch.cuda.Stream()
    buf = torch.zeros(64, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.graph(g, stream=s):
        rc = L.fpg_summed_expect_noalloc(b"XZ", 1, 2, buf.data_ptr(), 1, buf.data_ptr(), buf.data_ptr() + 256, 1,
                                         _abi.FPG_C128, ctypes.c_void_p(s.cuda_stream))
    assert rc == _abi.FPG_ERR_UNSUPPORTED
    assert b"captured" in L.fpg_last_error()


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
