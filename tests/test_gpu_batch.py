"""Batched persistent launch (fpg_batch_*): many expectation problems of
uneven size in one work-queue launch sequence, plain and CUDA-graph replayed,
with the autotuner; each result against the CPU oracle and independent of
the rest of the batch."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, TOL_MIXED, normwise

pytestmark = pytest.mark.gpu


def _problems(rng, count, n_range=(3, 12), p_range=(1, 120), s_range=(1, 40), k_range=(1, 3)):
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        P = int(rng.integers(p_range[0], p_range[1] + 1))
        S = int(rng.integers(s_range[0], s_range[1] + 1))
        K = int(rng.integers(k_range[0], k_range[1] + 1))
        strings = oracle.uniform_strings(rng, n, P)
        h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
        psi = oracle.unit_norm_states(rng, 1 << n, S)
        out.append((strings, h, psi))
    return out


def _build(torch, problems, dtype_code, cdt):
    from fast_pauli import _abi

    b = _abi.Batch(dtype_code)
    outs = []
    for strings, h, psi in problems:
        op = _abi.Operator(strings)
        dh = torch.from_numpy(h).to(cdt).cuda()
        dpsi = torch.from_numpy(psi).to(cdt).cuda()
        out = torch.full((h.shape[1], psi.shape[1]), 7.0 + 7j, dtype=cdt, device="cuda")  # overwritten
        b.add(op, dh.data_ptr(), h.shape[1], dpsi.data_ptr(), out.data_ptr(), psi.shape[1], keep=(dh, dpsi, out))
        outs.append(out)
    return b, outs


@pytest.mark.parametrize("dtype_name", ["c128", "c64"])
def test_batch_matches_oracle_plain_graph_and_tuned(dtype_name):
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    rng = np.random.default_rng(5 if dtype_name == "c128" else 6)
    problems = _problems(rng, 14)
    cdt, code, tol = ((torch.complex128, _abi.FPG_C128, TOL_C128) if dtype_name == "c128"
                      else (torch.complex64, _abi.FPG_C64, TOL_MIXED))
    b, outs = _build(torch, problems, code, cdt)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    wants = [oracle.summed_expectation(s, h, psi) for s, h, psi in problems]

    b.run(st)
    torch.cuda.synchronize()
    first = [o.cpu().numpy().copy() for o in outs]
    for got, want in zip(first, wants):
        assert normwise(got, want) < tol
    # outputs are overwritten, not accumulated: a second run is bitwise identical
    b.run(st)
    torch.cuda.synchronize()
    for o, f in zip(outs, first):
        np.testing.assert_array_equal(o.cpu().numpy(), f)
    # graph capture and replay
    for _ in range(2):
        b.run_graph(st)
        torch.cuda.synchronize()
        for o, f in zip(outs, first):
            np.testing.assert_array_equal(o.cpu().numpy(), f)
    # autotuner picks a tuning among its candidates; results stay correct
    best, ms = b.autotune(st)
    assert best["threads_per_cta"] in (128, 256) and ms > 0
    b.run_graph(st)
    torch.cuda.synchronize()
    for o, want in zip(outs, wants):
        assert normwise(o.cpu().numpy(), want) < tol
    n_problems, n_items, tuning = b.info()
    assert n_problems == 14 and n_items > 0 and tuning == best
    b.close()


def test_batch_result_independent_of_batch_composition():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    rng = np.random.default_rng(12)
    problems = _problems(rng, 6, n_range=(6, 11))
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    b, outs = _build(torch, problems, _abi.FPG_C64, torch.complex64)
    b.run(st)
    torch.cuda.synchronize()
    mixed = [o.cpu().numpy() for o in outs]
    b.close()
    for i, prob in enumerate(problems):
        alone, (o,) = _build(torch, [prob], _abi.FPG_C64, torch.complex64)
        alone.run(st)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(o.cpu().numpy(), mixed[i])
        alone.close()


def test_batch_argument_errors():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    b = _abi.Batch(_abi.FPG_C128)
    op = _abi.Operator(["XY"])
    buf = torch.zeros(8, dtype=torch.complex128, device="cuda")
    assert L.fpg_batch_add(b.handle, op.handle, buf.data_ptr(), 0, buf.data_ptr(), buf.data_ptr(), 1) == \
        _abi.FPG_ERR_INVALID
    assert L.fpg_batch_plan(b.handle, None) == _abi.FPG_ERR_INVALID  # empty batch
    bad = _abi.BatchTuning(96, 4, 4096, 40)
    b.add(op, buf.data_ptr(), 1, buf.data_ptr(), buf.data_ptr(), 1)
    assert L.fpg_batch_plan(b.handle, ctypes.byref(bad)) == _abi.FPG_ERR_INVALID
    assert L.fpg_batch_create(9, ctypes.byref(ctypes.c_void_p())) == _abi.FPG_ERR_INVALID
    b.close()
