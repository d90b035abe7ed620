"""GPU parity: the CUDA path against the reference's golden outputs and the CPU
oracle on the same seeded inputs (float64 path within 1e-12 normwise relative;
index/sign/phase work bit-exact), plus size-independent properties at the
full size of the n=14 weight<=2 workload.  Everything runs through libfpg's C ABI: via the
Python module (C++ host API -> C ABI) or directly via ctypes."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_C128, TOL_MIXED, TOL_MIXED_W2, golden, normwise

pytestmark = pytest.mark.gpu

fp = pytest.importorskip("fast_pauli")


def _strs(a):
    return [str(x) for x in a]


# ---------------------------------------------------------------- goldens


def test_sparse_repr_bit_exact_vs_reference():
    g = golden("sparse_repr.npz")
    for s in _strs(g["strings"]):
        cols, vals = fp.helpers.pauli_string_sparse_repr([fp.Pauli(c) for c in s])
        np.testing.assert_array_equal(np.array(cols, dtype=np.uint64), g[f"cols_{s}"])
        np.testing.assert_array_equal(np.array(vals), g[f"vals_{s}"])


def test_pauli_op_apply_n10_vs_reference():
    g = golden("pauli_op_apply_n10.npz")
    got = fp.PauliOp(g["coeffs"], _strs(g["strings"])).apply(g["states"])
    assert got.shape == (1024, 100) and got.dtype == np.complex128
    assert normwise(got, g["out"]) < TOL_C128


def test_small_methods_vs_reference():
    g = golden("small_methods.npz")
    s = _strs(g["strings"])
    c = complex(g["c"])
    psi, psi1 = g["states"], g["state1"]
    sop = fp.SummedPauliOp(s, g["h"])
    got = {
        "string_apply_2d": fp.PauliString(s[0]).apply(psi, c),
        "string_apply_1d": fp.PauliString(s[0]).apply(psi1, c),  # 1-D ignores coeff, as the reference
        "string_expectation": fp.PauliString(s[1]).expectation_value(psi, c),
        "op_apply": fp.PauliOp(g["coeffs"], s).apply(psi),
        "op_expectation": fp.PauliOp(g["coeffs"], s).expectation_value(psi),
        "summed_expectation": sop.expectation_value(psi),
        "summed_apply": sop.apply(psi),
        "summed_apply_weighted": sop.apply_weighted(psi, g["data"]),
    }
    for k, v in got.items():
        assert v.shape == g[k].shape, k
        assert normwise(v, g[k]) < TOL_C128, (k, normwise(v, g[k]))


def test_summed_expectation_weight2_n8_vs_reference():
    g = golden("summed_expectation_weight2_n8.npz")
    got = fp.SummedPauliOp(_strs(g["strings"]), g["h"]).expectation_value(g["states"])
    assert normwise(got, g["out"]) < TOL_C128


# ------------------------------------------------------ seeded oracle sweeps


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 9])
@pytest.mark.parametrize("S", [1, 3, 32, 37])
def test_uniform_strings_all_methods(n, S):
    rng = np.random.default_rng(100 * n + S)
    P, K = 2 + 3 * n, 3
    strings = oracle.uniform_strings(rng, n, P)
    coeffs = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    data = rng.standard_normal((K, S))
    op = fp.PauliOp(coeffs, strings)
    sop = fp.SummedPauliOp(strings, h)
    assert normwise(op.apply(psi), oracle.op_apply(strings, coeffs, psi)) < TOL_C128
    assert normwise(op.expectation_value(psi), oracle.op_expectation(strings, coeffs, psi)) < TOL_C128
    assert normwise(sop.expectation_value(psi), oracle.summed_expectation(strings, h, psi)) < TOL_C128
    assert normwise(sop.apply(psi), oracle.summed_apply(strings, h, psi)) < TOL_C128
    assert normwise(sop.apply_weighted(psi, data), oracle.summed_apply_weighted(strings, h, psi, data)) < TOL_C128


@pytest.mark.parametrize("n", [5, 6, 8, 11])
@pytest.mark.parametrize("S", [1, 16, 40])
def test_weight2_strings_summed_expectation(n, S):
    # the weight <= 2 string set (all weight <= 2 strings minus the
    # identity): large x-groups, mixed #Y parities, paired and unpaired rows
    rng = np.random.default_rng(7 * n + S)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P, K = len(strings), 5
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    got = fp.SummedPauliOp(strings, h).expectation_value(psi)
    assert normwise(got, oracle.summed_expectation(strings, h, psi)) < TOL_C128


@pytest.mark.parametrize("n,S", [(22, 3), (20, 18)])
def test_large_n_weight2_subset(n, S):
    """Row indices past 2^20: a random subset of the weight <= 2 strings
    (every kernel family: pair, marginal with up to 17 high row bits,
    transform) against the oracle: expectation and apply_weighted."""
    rng = np.random.default_rng(1000 + n)
    every = oracle.calculate_pauli_strings_max_weight(n, 2)
    pick = sorted(set(rng.choice(len(every), size=70, replace=False).tolist()) | {1, 2, 3})
    strings = [every[i] for i in pick]
    # a whole one-position group and part of the diagonal group
    strings += [s for s in every if s.startswith("X") and s.count("I") >= n - 2][:30]
    strings += [s for s in every if set(s) <= {"I", "Z"}][:20]
    strings = list(dict.fromkeys(strings))
    P, K = len(strings), 2
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    sop = fp.SummedPauliOp(strings, h)
    assert normwise(sop.expectation_value(psi), oracle.summed_expectation(strings, h, psi)) < TOL_C128
    data = rng.standard_normal((K, S))
    assert normwise(sop.apply_weighted(psi, data), oracle.summed_apply_weighted(strings, h, psi, data)) < TOL_C128


def _two_position_strings(n, pairs, kinds=("XX", "XY", "YX", "YY")):
    out = []
    for a, b in pairs:  # qubit positions (string index), a < b
        for k in kinds:
            s = ["I"] * n
            s[a], s[b] = k[0], k[1]
            out.append("".join(s))
    return out


@pytest.mark.parametrize(
    "case,n,S",
    [("tiles_and_pairs", 10, 9), ("few_groups", 10, 6), ("below_min_qubits", 7, 5), ("pairs_past_l2", 20, 4)],
)
@pytest.mark.parametrize("c64", [False, True])
def test_two_position_groups_tile_and_pair_kernels(case, n, S, c64):
    """The two-position x-groups (XX, XY, YX, YY on two qubits) go to the tile
    kernel, several per pass, when at least six of them have signs only on
    their lower qubit; the rest, and every such group of an operator on
    fewer than eight qubits, stay with the pair kernel; a state whose column
    tile does not fit in L2 runs the tile groups through the pair kernel."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(hash(case) % 1000 + n)
    every_pair = [(a, b) for a in range(n) for b in range(a + 1, n)]
    if case == "tiles_and_pairs":
        strings = _two_position_strings(n, every_pair[:20])
        # X X Z on three qubits with X X: signs on a third qubit (pair kernel)
        for a, b, c in [(0, 5, 8), (2, 3, 9), (4, 7, 1)]:
            s = ["I"] * n
            s[a], s[b] = "X", "X"
            strings.append("".join(s))
            s[c] = "Z"
            strings.append("".join(s))
        strings += ["Z" + "I" * (n - 1), "X" + "I" * (n - 1)]
    elif case == "few_groups":
        strings = _two_position_strings(n, every_pair[:5])
    elif case == "below_min_qubits":
        strings = _two_position_strings(n, every_pair)
    else:
        strings = _two_position_strings(n, every_pair[::17][:10])
    P, K = len(strings), 3
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = oracle.summed_expectation(strings, h, psi)
    states = torch.from_numpy(psi).to(torch.complex64 if c64 else torch.complex128).cuda()
    got = fp.SummedPauliOp(strings, h).expectation_value(states).cpu().numpy()
    assert normwise(got, want) < (TOL_MIXED_W2 if c64 else TOL_C128)


@pytest.mark.parametrize("kind", ["weight2", "uniform", "weight2_c64", "weight2_tiny"])
def test_pinned_host_states(kind):
    """Pinned host states (as torch's pinned tensors give them): float64 and
    complex64, operators with and without direct chunks, amplitudes outside
    the double-float range."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(91)
    n, S, K = 9, 24, 3
    if kind == "uniform":
        strings = oracle.uniform_strings(rng, n, 30)
    else:
        strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    if kind == "weight2_tiny":
        psi *= 1e-30
    want = oracle.summed_expectation(strings, h, psi)
    dt = torch.complex64 if kind == "weight2_c64" else torch.complex128
    t = torch.empty(psi.shape, dtype=dt, pin_memory=True)
    t.copy_(torch.from_numpy(psi))
    got = fp.SummedPauliOp(strings, h).expectation_value(t.numpy())
    tol = TOL_MIXED_W2 if kind == "weight2_c64" else TOL_C128
    assert normwise(got, want) < tol


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("chunks,S,c64", [(2, 128, False), (3, 300, False), (4, 257, True), (9, 200, False)])
def test_pinned_host_states_in_column_chunks(monkeypatch, chunks, S, c64, pinned):
    """Host states (pinned, or ordinary pageable numpy arrays) of many
    columns are computed in column chunks, each chunk's copy overlapping the
    previous chunk's computation: the results (odd widths, more chunks asked
    for than 64-column pieces exist) match the oracle and the one-call device
    path."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(chunks * 1000 + S)
    n, K = 8, 5
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = oracle.summed_expectation(strings, h, psi)
    dt = torch.complex64 if c64 else torch.complex128
    t = torch.empty(psi.shape, dtype=dt, pin_memory=True)
    t.copy_(torch.from_numpy(psi))
    sop = fp.SummedPauliOp(strings, h)
    whole = sop.expectation_value(t.cuda()).cpu().numpy()
    monkeypatch.setenv("FPG_HOST_CHUNKS", str(chunks))
    got = sop.expectation_value(t.numpy() if pinned else np.array(t.numpy(), copy=True))
    assert got.shape == (K, S)
    tol = TOL_MIXED_W2 if c64 else TOL_C128
    assert normwise(got, want) < tol
    assert normwise(got, whole) < tol


def test_concurrent_host_calls_from_threads():
    """Calls from several host threads at once (each on its per-thread
    stream, each with its own side stream for the concurrent kernel
    families) give the results of the same calls made one at a time."""
    import threading

    rng = np.random.default_rng(78)
    n, S = 10, 40
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P, K = len(strings), 3
    ops = []
    for j in range(4):
        h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
        ops.append((fp.SummedPauliOp(strings, h), oracle.unit_norm_states(rng, 1 << n, S)))
    alone = [op.expectation_value(psi) for op, psi in ops]
    got = [None] * len(ops)

    def run(j):
        for _ in range(3):
            got[j] = ops[j][0].expectation_value(ops[j][1])

    threads = [threading.Thread(target=run, args=(j,)) for j in range(len(ops))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for j in range(len(ops)):
        np.testing.assert_array_equal(got[j], alone[j])


def test_pool_memory_reused_and_released():
    # temporaries come from the library's pool: back-to-back host-buffer
    # calls (each synchronises) reuse it; after release_cached_memory the
    # next call maps fresh memory and gives the same result
    rng = np.random.default_rng(77)
    n, S = 9, 33
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P, K = len(strings), 4
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    sop = fp.SummedPauliOp(strings, h)
    first = sop.expectation_value(psi)
    assert normwise(first, oracle.summed_expectation(strings, h, psi)) < TOL_C128
    np.testing.assert_array_equal(sop.expectation_value(psi), first)
    fp.release_cached_memory()
    np.testing.assert_array_equal(sop.expectation_value(psi), first)


def _masks_to_string(n, x, z):
    # row bit r <-> character n-1-r
    ch = {(0, 0): "I", (1, 0): "X", (1, 1): "Y", (0, 1): "Z"}
    return "".join(ch[((x >> (n - 1 - q)) & 1, (z >> (n - 1 - q)) & 1)] for q in range(n))


def _pair_group_strings(rng, n, n_groups):
    """x-groups whose signs, without the pairing bit (top bit of x), use one
    row bit at most: the shape the pair kernel takes.  Sign bits below and
    above the 32-row block, rows paired across blocks (x >= 32) and inside
    them (x < 32), the diagonal group (x = 0) and groups without any sign
    bit are all drawn."""
    out = []
    xs = {0}
    while len(xs) < n_groups:
        w = int(rng.integers(1, min(3, n) + 1))
        xs.add(int(sum(1 << int(b) for b in rng.choice(n, size=w, replace=False))))
    for x in sorted(xs):
        pbit = (1 << (x.bit_length() - 1)) if x else 0
        a = int(rng.integers(-1, n))
        if a >= 0 and (1 << a) == pbit:
            a = -1
        zs = {0, pbit}
        if a >= 0:
            zs |= {1 << a, (1 << a) | pbit}
        # every string of the group: x fixed, z' in {0, e_a}
        cands = sorted(zs)
        k = int(rng.integers(1, len(cands) + 1))
        for z in rng.choice(cands, size=k, replace=False):
            out.append(_masks_to_string(n, x, int(z)))
    return out


@pytest.mark.parametrize("n", [3, 4, 6, 9, 13])
def test_pair_kernel_groups_per_string(n):
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(500 + n)
    strings = _pair_group_strings(rng, n, min(12, (1 << n) - 1))
    P, S = len(strings), 6
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = np.stack([oracle.string_expectation(s, psi).real for s in strings])
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for dtype, tdt, tol in ((_abi.FPG_C128, torch.complex128, 1e-13), (_abi.FPG_C64, torch.complex64, 2e-6)):
        dpsi = torch.from_numpy(psi).to(tdt).cuda()
        ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
        _abi.check(L.fpg_expect_strings(op.handle, dpsi.data_ptr(), ev.data_ptr(), S, dtype, st))
        torch.cuda.synchronize()
        assert np.abs(ev.cpu().numpy() - want).max() < tol, dtype
    op.close()


def _marginal_group_strings(rng, n, n_groups):
    """x-groups of >= 4 strings whose z' (pairing bit dropped) each have at
    most one bit, over several bits: the shape the marginal kernel takes
    (e.g. X_a, Y_a, X_a Z_b, Y_a Z_b)."""
    out = []
    xs = {0}
    while len(xs) < n_groups:
        w = int(rng.integers(1, min(2, n) + 1))
        xs.add(int(sum(1 << int(b) for b in rng.choice(n, size=w, replace=False))))
    for x in sorted(xs):
        pbit = (1 << (x.bit_length() - 1)) if x else 0
        cands = [0] + [1 << b for b in range(n) if (1 << b) != pbit]
        cands = cands + [c | pbit for c in cands] if pbit else cands
        k = int(rng.integers(4, min(len(cands), 24) + 1))
        for z in rng.choice(cands, size=k, replace=False):
            out.append(_masks_to_string(n, x, int(z)))
    return out


@pytest.mark.parametrize("n,S", [(3, 5), (4, 2), (6, 7), (9, 33), (14, 3), (20, 2)])
def test_marginal_kernel_groups_per_string(n, S):
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(700 + n)
    strings = _marginal_group_strings(rng, n, min(6, (1 << n) - 1))
    P = len(strings)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = np.stack([oracle.string_expectation(s, psi).real for s in strings])
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for dtype, tdt, tol in ((_abi.FPG_C128, torch.complex128, 1e-13), (_abi.FPG_C64, torch.complex64, 2e-6)):
        dpsi = torch.from_numpy(psi).to(tdt).cuda()
        ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
        _abi.check(L.fpg_expect_strings(op.handle, dpsi.data_ptr(), ev.data_ptr(), S, dtype, st))
        torch.cuda.synchronize()
        assert np.abs(ev.cpu().numpy() - want).max() < tol, dtype
    op.close()


@pytest.mark.parametrize("scale_psi,scale_h", [(1.0, 1.0), (1e-30, 1.0), (1e-20, 1.0), (1e-12, 1.0), (1e15, 1.0),
                                               (1.0, 1e20), (1.0, 1e-35)])
def test_float64_path_far_from_unit_scale(scale_psi, scale_h):
    """The float64 path runs its kernels in double-float arithmetic on the
    float32 pipes for elements below 2^40 in states whose columns reach 2^-39,
    and recomputes in float64 otherwise: results must meet the float64
    tolerance at any scale (1e-20: every element above 2^-90, yet products
    below float's normal range), and for states
    with exact zeros (basis states)."""
    rng = np.random.default_rng(61)
    n, S, K = 9, 12, 5
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * scale_h
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    psi[:, 0] = 0
    psi[5, 0] = 1.0  # a basis state: all other amplitudes exactly zero
    psi *= scale_psi
    want = oracle.summed_expectation(strings, h, psi)
    got = fp.SummedPauliOp(strings, h).expectation_value(psi)
    assert normwise(got, want) < TOL_C128


@pytest.mark.parametrize("scale_psi,scale_h", [(1.0, 1.0), (1e-30, 1.0), (1e15, 1.0), (1.0, 1e20), (1.0, 1e-35),
                                               (1e-20, 1e-20), (1e-20, 1.0)])
def test_float64_apply_far_from_unit_scale(scale_psi, scale_h):
    """The float64 apply runs in double-float arithmetic on the float32 pipes
    when the elements of states and coefficients stay below 2^40 and their
    columns reach 2^-39, and in float64 otherwise (the double-float kernel
    then leaves the output untouched)."""
    rng = np.random.default_rng(64)
    n, S, K = 8, 40, 3
    strings = oracle.uniform_strings(rng, n, 50) + oracle.calculate_pauli_strings_max_weight(n, 1)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * scale_h
    psi = oracle.unit_norm_states(rng, 1 << n, S) * scale_psi
    data = rng.standard_normal((K, S))
    coeffs = h[:, 0]
    op = fp.PauliOp(coeffs, strings)
    sop = fp.SummedPauliOp(strings, h)
    assert normwise(op.apply(psi), oracle.op_apply(strings, coeffs, psi)) < TOL_C128
    assert normwise(sop.apply(psi), oracle.summed_apply(strings, h, psi)) < TOL_C128
    assert normwise(sop.apply_weighted(psi, data), oracle.summed_apply_weighted(strings, h, psi, data)) < TOL_C128
    # accumulating into a non-zero output (+=) through the C ABI path
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    o = _abi.Operator(strings)
    dpsi = torch.from_numpy(psi).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(coeffs)).cuda()
    base = oracle.unit_norm_states(rng, 1 << n, S) * scale_psi
    out = torch.from_numpy(base.copy()).cuda()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(L.fpg_apply(o.handle, dc.data_ptr(), dpsi.data_ptr(), out.data_ptr(), S, _abi.FPG_C128, st))
    torch.cuda.synchronize()
    assert normwise(out.cpu().numpy(), base + oracle.op_apply(strings, coeffs, psi)) < TOL_C128
    o.close()


@pytest.mark.parametrize("n,S", [(2, 3), (9, 5), (9, 40), (12, 33)])
def test_float64_apply_weighted_class_sums(n, S):
    """A float64 apply_weighted whose operator holds 3 or more strings per
    x-group on average sums each thread's four rows' diagonals by classes of
    z & 3 and a 4-point transform (weight <= 2 sets); the results match the
    oracle, also with coefficients and states far from unit scale (still
    inside the double-float range: the weights below 2^40 with column maxima
    above 2^-39, and the states likewise)."""
    rng = np.random.default_rng(300 + n + S)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P, K = len(strings), 4
    for scale_h, scale_psi in ((1.0, 1.0), (1e8, 1e-9), (1e-9, 3.0)):
        h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * scale_h
        psi = oracle.unit_norm_states(rng, 1 << n, S) * scale_psi
        data = rng.standard_normal((K, S))
        got = fp.SummedPauliOp(strings, h).apply_weighted(psi, data)
        assert normwise(got, oracle.summed_apply_weighted(strings, h, psi, data)) < TOL_C128, (scale_h, scale_psi)


@pytest.mark.parametrize("n", [2, 9])
@pytest.mark.parametrize("scale", [1.0, 1e-30])
def test_apply_group_diagonal_table_matches_register_sums(n, scale):
    """A plain apply of 4 or more columns whose x-groups hold two or more
    strings on average reads the group diagonals from a table built once per
    call (one more launch); below 4 columns every thread sums its groups'
    strings itself.  A column's arithmetic is the same either way, so the
    first 3 columns of an 8-column apply equal a 3-column apply bit for bit,
    in both precisions.  n=2: fewer rows than one thread's rows; scale 1e-30:
    the float64 range check sends both calls to the float64 kernel, which
    never reads the table."""
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(71 + n)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    coeffs = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    psi = oracle.unit_norm_states(rng, 1 << n, 8) * scale
    want = oracle.op_apply(strings, coeffs, psi)
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for dtype, tdt, tol in ((_abi.FPG_C128, torch.complex128, TOL_C128), (_abi.FPG_C64, torch.complex64, TOL_MIXED)):
        dc = torch.from_numpy(coeffs).to(tdt).cuda()
        outs, launches = [], []
        for S in (3, 8):
            dpsi = torch.from_numpy(np.ascontiguousarray(psi[:, :S])).to(tdt).cuda()
            out = torch.zeros_like(dpsi)
            before = _abi.kernel_launches()
            _abi.check(L.fpg_apply(op.handle, dc.data_ptr(), dpsi.data_ptr(), out.data_ptr(), S, dtype, st))
            torch.cuda.synchronize()
            launches.append(_abi.kernel_launches() - before)
            outs.append(out.cpu().numpy())
        assert launches[1] == launches[0] + 1, (dtype, launches)
        assert np.array_equal(outs[1][:, :3], outs[0]), dtype
        assert normwise(outs[1], want) < tol, dtype
    op.close()


def test_float64_contraction_mixed_magnitudes():
    """The float64 contraction scales every row of H^T and of the per-string
    expectation table by a power of two and multiplies digit slices on the
    tensor cores: coefficients spanning 16 decades inside one operator, an
    all-zero operator and 300 columns (a ragged 64-column tile) must still
    meet the float64 tolerance."""
    rng = np.random.default_rng(62)
    n, S, K = 8, 300, 7
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    mag = 10.0 ** rng.uniform(-8, 8, size=(P, K))
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * mag
    h[:, 3] = 0
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = oracle.summed_expectation(strings, h, psi)
    got = fp.SummedPauliOp(strings, h).expectation_value(psi)
    assert normwise(got, want) < TOL_C128
    assert np.all(got[3] == 0)
    for k in (0, 1, 2, 4, 5, 6):
        assert normwise(got[k], want[k]) < TOL_C128


def test_float64_contraction_non_finite_coefficients():
    """A non-finite coefficient routes the contraction to the float64 GEMM:
    infinities and NaNs land where plain float64 arithmetic puts them."""
    rng = np.random.default_rng(63)
    n, S, K = 6, 9, 4
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    h[2, 1] = np.inf
    h[5, 3] = complex(np.nan, 0.0)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    ev = np.stack([oracle.string_expectation(s, psi).real for s in strings])  # (P, S)
    # real and imaginary parts contract separately (E is real)
    with np.errstate(invalid="ignore"):
        want = h.real.T @ ev + 1j * (h.imag.T @ ev)
    got = fp.SummedPauliOp(strings, h).expectation_value(psi)
    np.testing.assert_array_equal(np.isnan(got.real), np.isnan(want.real))
    np.testing.assert_array_equal(np.isinf(got.real), np.isinf(want.real))
    np.testing.assert_array_equal(np.isnan(got.imag), np.isnan(want.imag))
    fin = np.isfinite(want)
    assert normwise(got[fin], want[fin]) < TOL_C128


def test_exhaustive_small_strings_vs_dense():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3):
        psi = oracle.unit_norm_states(rng, 1 << n, 5)
        for s in oracle.calculate_pauli_strings_max_weight(n, n):
            d = oracle.dense(s)
            want = np.einsum("it,ij,jt->t", psi.conj(), d, psi)
            got = fp.PauliString(s).expectation_value(psi)
            np.testing.assert_allclose(got, want, atol=1e-14)
            np.testing.assert_allclose(fp.PauliString(s).apply(psi), d @ psi, atol=1e-14)


def test_one_dimensional_and_edge_inputs():
    rng = np.random.default_rng(4)
    strings = ["XYZ", "ZZI", "IYX"]
    coeffs = np.array([1.0, -2j, 0.5])
    psi = oracle.unit_norm_states(rng, 8, 1)[:, 0].copy()
    op = fp.PauliOp(coeffs, strings)
    out = op.apply(psi)
    assert out.shape == (8,)
    assert normwise(out, oracle.op_apply(strings, coeffs, psi)) < TOL_C128
    ev = op.expectation_value(psi)
    assert ev.shape == (1,)
    sop = fp.SummedPauliOp(strings, np.ones((3, 2), dtype=complex))
    assert sop.expectation_value(psi).shape == (2,)
    w = sop.apply_weighted(psi, np.array([0.5, -1.0]))
    assert w.shape == (8,)
    # int / float inputs are converted like the reference's nanobind conversion
    np.testing.assert_allclose(fp.PauliString("III").apply(np.arange(8)), np.arange(8), atol=1e-15)
    np.testing.assert_allclose(fp.PauliString("IXYZ").apply(np.zeros((16, 16))), np.zeros((16, 16)), atol=0)
    # zero states
    assert fp.PauliOp(coeffs, strings).apply(np.zeros((8, 0), dtype=complex)).shape == (8, 0)
    # non-C-contiguous complex128 input -> ValueError (reference __nb_helpers.hpp:55-74)
    with pytest.raises(ValueError):
        op.apply(np.asfortranarray(oracle.unit_norm_states(rng, 8, 4)))
    # shape errors (reference test_pauli_op.py:936-946)
    with pytest.raises(ValueError):
        fp.PauliOp([1, 1, 1], ["X", "Y", "Z"]).apply(np.ones(3))
    with pytest.raises(ValueError):
        fp.PauliOp([1, 1, 1], ["X", "Y", "Z"]).apply(np.eye(4))
    with pytest.raises(ValueError):
        fp.PauliOp([1, 1], ["XYZ", "ZYX"]).expectation_value(np.ones(32))
    with pytest.raises(ValueError):
        fp.PauliOp([1, 1], ["XYZ", "ZYX"]).expectation_value(np.eye(16))
    with pytest.raises(ValueError):
        sop.apply_weighted(np.ones((8, 3)), np.ones((3, 3)))


def test_duplicate_strings_and_identity():
    rng = np.random.default_rng(8)
    strings = ["XX", "XX", "II", "ZY", "II"]
    coeffs = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    psi = oracle.unit_norm_states(rng, 4, 6)
    op = fp.PauliOp(coeffs, strings)
    assert normwise(op.apply(psi), oracle.op_apply(strings, coeffs, psi)) < TOL_C128
    assert normwise(op.expectation_value(psi), oracle.op_expectation(strings, coeffs, psi)) < TOL_C128


def test_to_tensor_matches_dense():
    rng = np.random.default_rng(2)
    strings = oracle.uniform_strings(rng, 3, 5)
    c = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    want = sum(ci * oracle.dense(s) for ci, s in zip(c, strings))
    np.testing.assert_allclose(fp.PauliOp(c, strings).to_tensor(), want, atol=1e-14)
    np.testing.assert_allclose(fp.PauliString("XYZ").to_tensor(), oracle.dense("XYZ"), atol=0)
    h = np.stack([c, 2 * c], axis=1)
    t = fp.SummedPauliOp(strings, h).to_tensor()
    np.testing.assert_allclose(t[1], 2 * want, atol=1e-13)


@pytest.mark.parametrize("n,P,K", [(1, 3, 1), (4, 20, 3), (7, 60, 2)])
def test_to_tensor_device_vs_dense_and_accumulates(n, P, K):
    """fpg_to_tensor against the kron-built dense matrices (duplicates and
    identity strings included), accumulating into the output like the
    reference's to_tensor."""
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(90 + n)
    strings = oracle.uniform_strings(rng, n, P)
    strings[0] = "I" * n
    strings[-1] = strings[1]
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    want = np.stack([sum(h[j, k] * oracle.dense(s) for j, s in enumerate(strings)) for k in range(K)])
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    D = 1 << n
    for dtype, tdt, tol in ((_abi.FPG_C128, torch.complex128, 1e-13), (_abi.FPG_C64, torch.complex64, 1e-5)):
        dh = torch.from_numpy(h).to(tdt).cuda()
        out = torch.ones((K, D, D), dtype=tdt, device="cuda")
        _abi.check(L.fpg_to_tensor(op.handle, dh.data_ptr(), K, out.data_ptr(), dtype, st))
        torch.cuda.synchronize()
        assert normwise(out.cpu().numpy() - 1.0, want) < tol, dtype
    op.close()


# ------------------------------------------------------------ device tensors


def test_torch_device_tensors_c128_and_mixed():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    n, S, K = 9, 48, 6
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = oracle.summed_expectation(strings, h, psi)
    sop = fp.SummedPauliOp(strings, h)
    t128 = torch.from_numpy(psi).cuda()
    got = sop.expectation_value(t128)
    assert isinstance(got, torch.Tensor) and got.is_cuda and got.dtype == torch.complex128
    assert normwise(got.cpu().numpy(), want) < TOL_C128
    t64 = t128.to(torch.complex64)
    got64 = sop.expectation_value(t64)
    assert got64.dtype == torch.complex64
    assert normwise(got64.cpu().numpy(), want) < TOL_MIXED_W2
    # apply on device, both precisions
    wa = oracle.summed_apply(strings, h, psi)
    assert normwise(sop.apply(t128).cpu().numpy(), wa) < TOL_C128
    assert normwise(sop.apply(t64).cpu().numpy(), wa) < TOL_MIXED


# ------------------------------------------------- tensor-core contraction


@pytest.mark.parametrize("K,S,n", [(1, 1, 3), (300, 200, 7), (130, 129, 6)])
def test_tensor_core_contraction_3xtf32(K, S, n):
    """Mixed path: the tcgen05 3xTF32 contraction across several 128x128
    tiles and 32-deep k chunks, isolated from the expectation stage by
    contracting the same float64 per-string table on the host."""
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(K + S + n)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d64 = torch.from_numpy(psi).to(torch.complex64).cuda()
    h64 = torch.from_numpy(h).to(torch.complex64).cuda()
    ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
    _abi.check(L.fpg_expect_strings(op.handle, d64.data_ptr(), ev.data_ptr(), S, _abi.FPG_C64, st))
    out = torch.zeros((K, S), dtype=torch.complex64, device="cuda")
    _abi.check(L.fpg_summed_expect(op.handle, h64.data_ptr(), K, d64.data_ptr(), out.data_ptr(), S, _abi.FPG_C64,
                                   st))
    code = ctypes.c_int(-1)
    _abi.check(L.fpg_device_error(ctypes.byref(code), st))
    assert code.value == 0
    want = h64.cpu().numpy().astype(np.complex128).T @ ev.cpu().numpy()
    assert normwise(out.cpu().numpy(), want) < 2e-6  # 3xTF32 with float32 accumulation
    # a single output (K = S = 1) is one cancelling sum of 36 terms: its
    # relative error is the complex64 rounding of the terms times the
    # cancellation ratio, so it is held to the looser bound
    tol = TOL_MIXED if K * S == 1 else TOL_MIXED_W2
    assert normwise(out.cpu().numpy(), oracle.summed_expectation(strings, h, psi)) < tol
    op.close()


def test_tensor_core_weighted_coefficients():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    n, S, K = 6, 150, 140
    strings = oracle.uniform_strings(rng, n, 40)
    P = len(strings)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    data = rng.standard_normal((K, S))
    sop = fp.SummedPauliOp(strings, h)
    got = sop.apply_weighted(torch.from_numpy(psi).to(torch.complex64).cuda(),
                             torch.from_numpy(data).to(torch.float32).cuda())
    want = oracle.summed_apply_weighted(strings, h, psi, data)
    assert normwise(got.cpu().numpy(), want) < TOL_MIXED


# ------------------------------------------------------------ square


@pytest.mark.parametrize("name", ["summed_square.npz", "summed_square_n6.npz"])
def test_summed_square_vs_reference(name):
    g = golden(name)
    op = fp.SummedPauliOp(_strs(g["strings"]), g["h"])
    sq = op.square()
    assert sq.pauli_strings_as_str == _strs(g["sq_strings"])
    assert normwise(sq.coeffs.T, g["sq_h"]) < TOL_C128


@pytest.mark.parametrize("n,w,K,dup", [(5, 2, 4, False), (8, 2, 9, False), (7, 1, 3, True), (4, 4, 2, False)])
def test_summed_square_vs_oracle(n, w, K, dup):
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(40 + n + w)
    strings = oracle.calculate_pauli_strings_max_weight(n, w)
    if dup:  # repeated strings: their products with each other are the identity
        strings = strings + strings[3:9]
    rng.shuffle(strings)
    P = len(strings)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    sq_strings = oracle.calculate_pauli_strings_max_weight(n, min(n, 2 * w))
    want = oracle.summed_square(strings, h, sq_strings)
    op, q = _abi.Operator(strings), _abi.Operator(sq_strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for dtype, tdt, tol in ((_abi.FPG_C128, torch.complex128, TOL_C128), (_abi.FPG_C64, torch.complex64, TOL_MIXED)):
        dh = torch.from_numpy(h).to(tdt).cuda()
        out = torch.full((len(sq_strings), K), 7.0, dtype=tdt, device="cuda")  # overwritten
        _abi.check(L.fpg_summed_square(op.handle, dh.data_ptr(), K, q.handle, out.data_ptr(), dtype, st))
        assert normwise(out.cpu().numpy(), want) < tol, dtype
    # a squared set that misses products is an argument error, reported after the run
    small = _abi.Operator(sq_strings[: len(sq_strings) // 2])
    out = torch.zeros((len(sq_strings) // 2, K), dtype=torch.complex128, device="cuda")
    dh = torch.from_numpy(h).cuda()
    rc = L.fpg_summed_square(op.handle, dh.data_ptr(), K, small.handle, out.data_ptr(), _abi.FPG_C128, st)
    assert rc == _abi.FPG_ERR_INVALID
    for o in (op, q, small):
        o.close()


# ------------------------------------------------------------ raw C ABI


def test_c_abi_direct_device_buffers():
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    L = _abi.lib()
    rng = np.random.default_rng(31)
    n, S, K = 8, 20, 4
    strings = oracle.uniform_strings(rng, n, 30)
    P = len(strings)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    op = _abi.Operator(strings)
    nq, ps, ng = op.info()
    assert (nq, ps) == (n, P) and 1 <= ng <= P
    dpsi = torch.from_numpy(psi).cuda()
    dh = torch.from_numpy(h).cuda()
    dout = torch.zeros((K, S), dtype=torch.complex128, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, dpsi.data_ptr(), dout.data_ptr(), S,
                                   _abi.FPG_C128, st))
    # outputs accumulate: a second call doubles the result
    _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, dpsi.data_ptr(), dout.data_ptr(), S,
                                   _abi.FPG_C128, st))
    torch.cuda.synchronize()
    assert normwise(dout.cpu().numpy(), 2 * oracle.summed_expectation(strings, h, psi)) < TOL_C128
    ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
    _abi.check(L.fpg_expect_strings(op.handle, dpsi.data_ptr(), ev.data_ptr(), S, _abi.FPG_C128, st))
    torch.cuda.synchronize()
    for j in (0, 7, P - 1):
        want = oracle.string_expectation(strings[j], psi)
        assert np.abs(ev[j].cpu().numpy() - want.real).max() < 1e-13
        assert np.abs(want.imag).max() < 1e-13  # Hermitian: expectations are real
    dtype_bad = L.fpg_summed_expect(op.handle, dh.data_ptr(), K, dpsi.data_ptr(), dout.data_ptr(), S, 7, st)
    assert dtype_bad == _abi.FPG_ERR_INVALID
    op.close()


# ---------------------- full-size properties (n=14, weight <= 2, 1024 states)


def test_weight2_n14_full_size_properties():
    """n=14, all 861 weight<=2 strings, S=1024 (the bench workload's shape,
    K reduced): size-independent properties instead of the oracle."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1002)
    n, S = 14, 1024
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)
    P = len(strings)  # 862 incl. the identity at index 0
    psi = torch.from_numpy(oracle.unit_norm_states(rng, 1 << n, S)).cuda()
    K = 3
    h1 = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    h2 = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    e1 = fp.SummedPauliOp(strings, h1).expectation_value(psi).cpu().numpy()
    e2 = fp.SummedPauliOp(strings, h2).expectation_value(psi).cpu().numpy()
    a = 0.3 - 1.7j
    e12 = fp.SummedPauliOp(strings, a * h1 + h2).expectation_value(psi).cpu().numpy()
    assert normwise(e12, a * e1 + e2) < 1e-12  # linearity in the coefficients
    # identity string: <psi|psi> = 1 for unit-norm columns
    eid = fp.PauliString("I" * n).expectation_value(psi).cpu().numpy()
    np.testing.assert_allclose(eid, np.ones(S), atol=1e-12)
    # consistency of two kernels: <psi| (A psi) > == expectation of A
    coeffs = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    op = fp.PauliOp(coeffs, strings)
    applied = op.apply(psi)
    via_apply = torch.einsum("it,it->t", psi.conj(), applied).cpu().numpy()
    assert normwise(op.expectation_value(psi).cpu().numpy(), via_apply) < 1e-12
    # P^2 = I for a single string (to the double-float representation of the
    # amplitudes, 48 significand bits: ~2^-48 relative)
    s = fp.PauliString("XYZI" * 3 + "YZ")
    back = s.apply(s.apply(psi))
    assert normwise(back.cpu().numpy(), psi.cpu().numpy()) < 1e-14


def _strings_on_bits(n, xbit, zpairs, xchar="X"):
    """Strings with `xchar` on row bit xbit and Z on the row bits of each pair
    (character q acts on row bit n-1-q)."""
    out = []
    for a, b in zpairs:
        s = ["I"] * n
        s[n - 1 - xbit] = xchar
        s[n - 1 - a] = "Z"
        s[n - 1 - b] = "Z"
        out.append("".join(s))
    return out


@pytest.mark.parametrize("n,xbit", [(6, 1), (6, 5), (10, 1), (10, 3), (10, 6)])
@pytest.mark.parametrize("S", [5, 12, 40])
@pytest.mark.parametrize("c64", [False, True])
def test_transform_kernel_groups_with_two_bit_signs(n, xbit, S, c64):
    """Groups of >= 10 strings sharing one x whose signs use two row bits go
    to the transform kernel.  x below the 16-row block (x = 2, 8) with 40
    states (32 column lanes, 8 row lanes) takes the second level across a
    round's 8 blocks -- at n = 6 the round holds fewer blocks than that; with
    12 states (16 column lanes, 16 row lanes) the float32 form takes a
    16-point second level and the float64 forms keep one level; x = 32, 64
    pairs blocks and keeps per-block sums; 5 states (8 column lanes, 32 row
    lanes) keep one level.  X and Y on the same bit give both parts."""
    torch = pytest.importorskip("torch")
    K = 3
    rng = np.random.default_rng(50 + 7 * n + xbit + S)
    pairs = [(a, b) for a in range(n) for b in range(a + 1, n) if xbit not in (a, b)][:20]
    strings = _strings_on_bits(n, xbit, pairs) + _strings_on_bits(n, xbit, pairs, "Y")
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    want = oracle.summed_expectation(strings, h, psi)
    states = torch.from_numpy(psi).to(torch.complex64 if c64 else torch.complex128).cuda()
    got = fp.SummedPauliOp(strings, h).expectation_value(states).cpu().numpy()
    assert normwise(got, want) < (TOL_MIXED if c64 else TOL_C128)


def test_family_stats_partition_the_operator_work():
    """fpg_operator_family_stats splits fpg_operator_stats' work by kernel
    family; for the 861 weight <= 2 strings at n = 14 the 91 two-position
    groups are the tile kernel's, the 14 one-position groups the marginal
    kernel's and the diagonal group (I, Z, ZZ) the transform kernel's."""
    from fast_pauli import _abi

    n = 14
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    op = _abi.Operator(strings)
    try:
        _, visits, adds = op.stats()
        fam = op.family_stats()
    finally:
        op.close()
    assert sum(v for v, _ in fam.values()) == visits
    assert sum(a for _, a in fam.values()) == adds
    half = 1 << (n - 1)
    assert fam["tile"] == (91 * half, 0)
    assert fam["marginal"][0] == 14 * half
    assert fam["transform"][0] == 1 << n
    assert fam["pair"] == (0, 0) and fam["direct"] == (0, 0)


@pytest.mark.parametrize("tiny", [2.0**-70, 2.0**-45, 1e-35])
def test_float64_columns_of_very_different_scale(tiny):
    """Each state column is its own state: a column scaled far below the
    others (uniform amplitudes of 2^-70 or 2^-45, whose products fall below
    float's normal range, or a Gaussian column at 1e-35) keeps float64 accuracy
    relative to its own values (such a column sends the call to the float64
    recomputation)."""
    rng = np.random.default_rng(71)
    n, S, K = 10, 6, 4
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    psi[:, 1] = tiny * (1 + 1j)  # uniform tiny column
    psi[:, 2] *= tiny            # Gaussian tiny column
    want = oracle.summed_expectation(strings, h, psi)
    got = fp.SummedPauliOp(strings, h).expectation_value(psi)
    for t in range(S):
        assert normwise(got[:, t], want[:, t]) < TOL_C128, t


def test_float64_noise_amplitudes_stay_on_the_double_float_path():
    """Amplitudes of 1e-40 (below 2^-90) beside unit-scale ones: the column's
    largest value sets the df64 range, the tiny ones contribute errors below
    2^-126 each, and the results keep float64 accuracy per column."""
    rng = np.random.default_rng(72)
    n, S = 10, 5
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = rng.standard_normal((P, 3)) + 1j * rng.standard_normal((P, 3))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    for t in range(S):
        psi[rng.choice(1 << n, 64, replace=False), t] = 1e-40 * (1 - 1j)
    for coeffs in (h, np.eye(P, dtype=np.complex128)):
        want = oracle.summed_expectation(strings, coeffs, psi)
        got = fp.SummedPauliOp(strings, coeffs).expectation_value(psi)
        for t in range(S):
            assert normwise(got[:, t], want[:, t]) < TOL_C128, t


@pytest.mark.parametrize("n,S", [(8, 6), (10, 40), (12, 33), (14, 64), (9, 1)])
def test_float64_tile_kernel_all_pairs(n, S):
    """The float64 two-position groups (XX, XY, YX, YY on every pair of
    qubits: the tile kernel's units cover them all): per-string values to
    1e-13 and the summed expectation values to the float64 tolerance against
    the oracle, for even and odd state counts."""
    torch = pytest.importorskip("torch")
    from fast_pauli import _abi

    rng = np.random.default_rng(900 + 10 * n + S)
    strings = [s for s in oracle.calculate_pauli_strings(n, 2) if sum(c in "XY" for c in s) == 2]
    P, K = len(strings), 3
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    L = _abi.lib()
    op = _abi.Operator(strings)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dpsi = torch.from_numpy(psi).cuda()
    ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
    _abi.check(L.fpg_expect_strings(op.handle, dpsi.data_ptr(), ev.data_ptr(), S, _abi.FPG_C128, st))
    torch.cuda.synchronize()
    op.close()
    want = np.stack([oracle.string_expectation(s, psi).real for s in strings])
    assert np.abs(ev.cpu().numpy() - want).max() < 1e-13
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    got = fp.SummedPauliOp(strings, h).expectation_value(dpsi).cpu().numpy()
    assert normwise(got, oracle.summed_expectation(strings, h, psi)) < TOL_C128
