"""Serving loop (fpg_server_*): requests of different sizes submitted while
others run are admitted as slots and HBM budget free up, overlap on the
device, and give the same result alone and in the mix.  Failure handling is
exercised on the host (malformed requests, over-budget requests, unknown
tickets); nothing here faults or hangs the GPU."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, TOL_MIXED, normwise

pytestmark = pytest.mark.gpu


def _make_requests(torch, rng, count, cdt, rdt):
    from fast_pauli import _abi

    reqs = []
    for i in range(count):
        n = int(rng.integers(5, 12))
        P = int(rng.integers(4, 90))
        S = int(rng.integers(1, 24))
        K = int(rng.integers(1, 5))
        kind = _abi.FPG_REQ_EXPECT if i % 2 == 0 else _abi.FPG_REQ_APPLY_WEIGHTED
        strings = oracle.uniform_strings(rng, n, P)
        h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
        psi = oracle.unit_norm_states(rng, 1 << n, S)
        data = rng.standard_normal((K, S))
        op = _abi.Operator(strings)
        dev = {
            "h": torch.from_numpy(h).to(cdt).cuda(),
            "psi": torch.from_numpy(psi).to(cdt).cuda(),
            "data": torch.from_numpy(data).to(rdt).cuda(),
        }
        out_shape = (K, S) if kind == _abi.FPG_REQ_EXPECT else (1 << n, S)
        reqs.append(dict(kind=kind, op=op, strings=strings, h=h, psi=psi, data=data, K=K, S=S, dev=dev,
                         out_shape=out_shape))
    return reqs


def _submit(server, torch, r, cdt):
    out = torch.full(r["out_shape"], 3.0 - 1j, dtype=cdt, device="cuda")  # overwritten by the server
    t = server.submit(r["kind"], r["op"], r["dev"]["h"].data_ptr(), r["K"], r["dev"]["psi"].data_ptr(),
                      out.data_ptr(), r["S"], r["dev"]["data"].data_ptr())
    return t, out


@pytest.mark.parametrize("dtype_name", ["c128", "c64"])
def test_results_same_alone_and_in_the_mix(dtype_name):
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    cdt, rdt, code, tol = ((torch.complex128, torch.float64, _abi.FPG_C128, TOL_C128) if dtype_name == "c128"
                           else (torch.complex64, torch.float32, _abi.FPG_C64, TOL_MIXED))
    rng = np.random.default_rng(41)
    reqs = _make_requests(torch, rng, 24, cdt, rdt)

    # alone: one slot, one request at a time
    alone = []
    srv = _abi.Server(code, n_slots=1)
    for r in reqs:
        t, out = _submit(srv, torch, r, cdt)
        srv.wait(t)
        alone.append(out.cpu().numpy())
    srv.close()

    # in the mix: all submitted at once to 6 slots, continuous admission
    srv = _abi.Server(code, n_slots=6, hbm_budget_bytes=1 << 30)
    pending = [_submit(srv, torch, r, cdt) for r in reqs]
    infos = [srv.wait(t, timeout_ms=60000) for t, _ in pending]
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["peak_running"] >= 2  # requests overlapped on the device
    # every expectation request here is small: all ran through merged runs
    n_expect = sum(r["kind"] == _abi.FPG_REQ_EXPECT for r in reqs)
    assert stats["merged_requests"] == n_expect and 1 <= stats["merged_runs"] <= n_expect
    for r, (t, out), a, info in zip(reqs, pending, alone, infos):
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got, a)  # identical alone and in the mix
        if r["kind"] == _abi.FPG_REQ_EXPECT:
            want = oracle.summed_expectation(r["strings"], r["h"], r["psi"])
        else:
            want = oracle.summed_apply_weighted(r["strings"], r["h"], r["psi"], r["data"])
        assert normwise(got, want) < tol
        assert info["submit_us"] <= info["start_us"] <= info["done_us"]


def test_small_requests_queued_together_share_one_merged_run():
    """Small expectation requests that queue while the only slot is busy are
    admitted together into one merged run (one launch sequence for all of
    them); each result is bit-identical to the request served alone and
    matches the oracle."""
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    rng = np.random.default_rng(17)
    cdt = torch.complex128
    small = [r for r in _make_requests(torch, rng, 24, cdt, torch.float64) if r["kind"] == _abi.FPG_REQ_EXPECT]
    # a medium request that keeps the slot busy while the small ones arrive
    n, P, S = 18, 1000, 32
    strings = oracle.uniform_strings(rng, n, P)
    big = dict(kind=_abi.FPG_REQ_EXPECT, op=_abi.Operator(strings), K=1, S=S, out_shape=(1, S),
               dev={"h": torch.ones((P, 1), dtype=cdt, device="cuda"),
                    "psi": torch.randn((1 << n, S), dtype=cdt, device="cuda"),
                    "data": torch.zeros(1, device="cuda")})
    alone = []
    srv = _abi.Server(_abi.FPG_C128, n_slots=1)
    for r in small:
        t, out = _submit(srv, torch, r, cdt)
        srv.wait(t)
        alone.append(out.cpu().numpy())
    srv.close()

    srv = _abi.Server(_abi.FPG_C128, n_slots=1)
    tb, _ = _submit(srv, torch, big, cdt)
    pending = [_submit(srv, torch, r, cdt) for r in small]
    srv.wait(tb, timeout_ms=60000)
    for t, _ in pending:
        srv.wait(t, timeout_ms=60000)
    st = srv.stats()
    srv.close()
    assert st["failed"] == 0 and st["merged_requests"] == len(small)
    assert st["merged_runs"] < len(small)  # at least two requests shared a run
    for r, (t, out), a in zip(small, pending, alone):
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got, a)
        assert normwise(got, oracle.summed_expectation(r["strings"], r["h"], r["psi"])) < TOL_C128


def test_admission_by_hbm_budget_and_refusals():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    rng = np.random.default_rng(3)
    reqs = _make_requests(torch, rng, 10, torch.complex128, torch.float64)
    need = max(r["P"] if "P" in r else 0 for r in reqs)  # noqa: F841
    # a budget that fits only a few requests at a time: the rest must queue
    srv = _abi.Server(_abi.FPG_C128, n_slots=8, hbm_budget_bytes=600_000)
    pending, refused = [], 0
    for r in reqs:
        try:
            pending.append(_submit(srv, torch, r, torch.complex128))
        except _abi.FpgError as e:
            assert e.code == _abi.FPG_ERR_BUSY
            refused += 1
    for t, _ in pending:
        info = srv.wait(t, timeout_ms=60000)
        assert info["scratch_bytes"] <= 600_000
    st = srv.stats()
    assert st["peak_reserved_bytes"] <= 600_000
    assert st["refused"] == refused and st["completed"] == len(pending)
    # malformed request: null array -> FPG_ERR_INVALID, nothing launched
    bad = _abi.Request(_abi.FPG_REQ_EXPECT, 0, reqs[0]["op"].handle, None, 1, None, None, None, 1)
    t = ctypes.c_uint64()
    assert _abi.lib().fpg_server_submit(srv.handle, ctypes.byref(bad), ctypes.byref(t)) == _abi.FPG_ERR_INVALID
    bad.kind = 9
    assert _abi.lib().fpg_server_submit(srv.handle, ctypes.byref(bad), ctypes.byref(t)) == _abi.FPG_ERR_INVALID
    # unknown ticket
    info = _abi.TicketInfo()
    assert _abi.lib().fpg_server_wait(srv.handle, 10**9, 0, ctypes.byref(info)) == _abi.FPG_ERR_INVALID
    srv.close()
