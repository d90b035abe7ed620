"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference sources are present: it calls the reference's
own C++ implementation (qognitive/fast-pauli headers compiled unmodified by
oracle/build_ref.sh into oracle/_ref/libfpref.so) through oracle/ref.py, on
seeded synthetic inputs, and stores inputs and outputs together so the tests
need neither the reference nor a matching RNG stream.

    bash oracle/build_ref.sh && python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from oracle import ref  # noqa: E402


def _s(strings):
    return np.array(strings, dtype="U")


def main() -> None:
    if not ref.available():
        raise SystemExit("oracle/_ref/libfpref.so missing: run oracle/build_ref.sh first")
    out = {}

    # --- sparse patterns: every string of 1..3 qubits plus longer samples -----
    import itertools

    strs = ["".join(p) for k in (1, 2, 3) for p in itertools.product("IXYZ", repeat=k)]
    strs += ["XYZXYZ", "ZZZIII", "XYIZXYZ", "XXIYYIZZ", "ZIXIZYXX", "YYYYYYYYYY"]
    sp = {}
    for s in strs:
        k, m = ref.sparse_repr(s)
        sp[s] = (k, m)
    np.savez_compressed(
        os.path.join(HERE, "sparse_repr.npz"),
        strings=_s(strs),
        **{f"cols_{s}": sp[s][0] for s in strs},
        **{f"vals_{s}": sp[s][1] for s in strs},
    )

    # --- helper ordering -----------------------------------------------------
    helpers = {}
    for n, w in [(2, 1), (3, 2), (4, 2), (5, 3)]:
        helpers[f"max_weight_{n}_{w}"] = _s(ref.pauli_strings_max_weight(n, w))
    for n, w in [(12, 2), (14, 2), (18, 2)]:
        helpers[f"count_{n}_{w}"] = np.array(len(ref.pauli_strings_max_weight(n, w)))
    np.savez_compressed(os.path.join(HERE, "helpers.npz"), **helpers)

    # --- PauliOp.apply, n=10, 64 uniform strings, 1024x100 ----------------------
    rng = np.random.default_rng(1001)
    n, P, S = 10, 64, 100
    strings = oracle.uniform_strings(rng, n, P)
    coeffs = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    res = ref.op_apply(strings, coeffs, psi)
    np.savez_compressed(
        os.path.join(HERE, "pauli_op_apply_n10.npz"),
        strings=_s(strings), coeffs=coeffs, states=psi, out=res,
    )

    # --- small cases of every method ------------------------------------------
    rng = np.random.default_rng(2024)
    n, P, K, S = 6, 24, 5, 10
    strings = oracle.uniform_strings(rng, n, P)
    coeffs = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    psi1 = psi[:, 3].copy()
    data = rng.standard_normal((K, S))
    c = 0.7 - 0.3j
    small = dict(
        strings=_s(strings), coeffs=coeffs, h=h, states=psi, state1=psi1, data=data, c=np.array(c),
        string_apply_2d=ref.string_apply(strings[0], psi, c),
        string_apply_1d=ref.string_apply(strings[0], psi1),
        string_expectation=ref.string_expectation(strings[1], psi, c),
        op_apply=ref.op_apply(strings, coeffs, psi),
        op_expectation=ref.op_expectation(strings, coeffs, psi),
        summed_expectation=ref.summed_expectation(strings, h, psi),
        summed_apply=ref.summed_apply(strings, h, psi),
        summed_apply_weighted=ref.summed_apply_weighted(strings, h, psi, data),
    )
    np.savez_compressed(os.path.join(HERE, "small_methods.npz"), **small)

    # --- SummedPauliOp.expectation_value on weight<=2 strings minus the
    #     identity, n=8, K=20, S=16, h ~ CN(0, 1/P) --------------------------------
    rng = np.random.default_rng(1002)
    n, K, S = 8, 20, 16
    strings = ref.pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) / np.sqrt(2 * P)
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    np.savez_compressed(
        os.path.join(HERE, "summed_expectation_weight2_n8.npz"),
        strings=_s(strings), h=h, states=psi, out=ref.summed_expectation(strings, h, psi),
    )

    # --- SummedPauliOp.square (next row), tiny ------------------------------------
    rng = np.random.default_rng(7)
    strings = ref.pauli_strings_max_weight(3, 1)
    h = rng.standard_normal((len(strings), 2)) + 1j * rng.standard_normal((len(strings), 2))
    sq_strings, sq_h = ref.summed_square(strings, h)
    np.savez_compressed(
        os.path.join(HERE, "summed_square.npz"),
        strings=_s(strings), h=h, sq_strings=_s(sq_strings), sq_h=sq_h,
    )
    # weight <= 2 strings at n = 6 (identity included), K = 3: 154 strings,
    # 1909 squared strings (weight <= 4)
    rng = np.random.default_rng(8)
    strings = ref.pauli_strings_max_weight(6, 2)
    h = rng.standard_normal((len(strings), 3)) + 1j * rng.standard_normal((len(strings), 3))
    sq_strings, sq_h = ref.summed_square(strings, h)
    np.savez_compressed(
        os.path.join(HERE, "summed_square_n6.npz"),
        strings=_s(strings), h=h, sq_strings=_s(sq_strings), sq_h=sq_h,
    )
    # --- PauliOp products (next row): random operators and a self-product
    # with many equal strings; the reference's raw output (its per-thread maps
    # may list a string more than once)
    rng = np.random.default_rng(11)
    a_s = [str(x) for x in oracle.uniform_strings(rng, 5, 12)]
    b_s = [str(x) for x in oracle.uniform_strings(rng, 5, 9)]
    a_c = rng.standard_normal(12) + 1j * rng.standard_normal(12)
    b_c = rng.standard_normal(9) + 1j * rng.standard_normal(9)
    ab_s, ab_c = ref.op_product(a_c, a_s, b_c, b_s)
    w2 = ref.pauli_strings_max_weight(4, 2)
    w_c = rng.standard_normal(len(w2)) + 1j * rng.standard_normal(len(w2))
    ww_s, ww_c = ref.op_product(w_c, w2, w_c, w2)
    np.savez_compressed(
        os.path.join(HERE, "op_product.npz"),
        a_strings=_s(a_s), a_coeffs=a_c, b_strings=_s(b_s), b_coeffs=b_c, ab_strings=_s(ab_s), ab_coeffs=ab_c,
        w_strings=_s(w2), w_coeffs=w_c, ww_strings=_s(ww_s), ww_coeffs=ww_c,
    )
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
