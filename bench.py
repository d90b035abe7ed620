"""Benchmark of the Pauli expectation hot path on GB300.

Default workload (one "step"): SummedPauliOp.expectation_value in float64 at
n = 14 qubits, the 861 strings of weight <= 2 (calculate_pauli_strings_max_weight
minus the identity), K = 1000 operators with coefficients ~ CN(0, 1/861),
16384 x 1024 complex128 unit-norm Gaussian states -> (1000, 1024).  Metric:
amplitude-terms/s = n_strings * 2^n * n_states per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs its own full workload on its own GPU
(weak scaling, no data-path collective); only the timing is reduced (max).
Rank 0 prints one JSON line.

Keys beyond the base contract:
  roofline      the dominant stage (the per-string expectation kernels,
                fpg_expect_strings, timed alone with CUDA events on its
                stream) against its binding roof: float32 FMA-pipe issue.  The
                stage runs its float64 arithmetic as double-float on the
                float32 pipes; achieved = the stage's float64 operations by
                kernel family (fpg_operator_family_stats: 4 multiply-adds per
                row visit plus the sign additions) x the float32 instructions
                each costs in that family's double-float form (DF64_MULADD_OPS,
                DF64_ADD_OPS) / time;
                peak = the float32 FMA rate measured on this GPU
                (fpg_measure_peak).  "streaming_equiv" keeps the
                streaming-equivalent HBM figure (16 B per amplitude-term), and
                "dram_frac" the stage's real DRAM rate (ncu bytes / time).
  cpu_baseline  the CPU oracle port (OpenMP, all host threads) on the whole
                workload (all 861 strings), with the host CPU named.
  e2e           the public API with host numpy states: pinned (value) and
                ordinary pageable memory ("pageable").
  mixed         the complex64 / float32 path on the n = 18 shape (1431 strings,
                K = 1000, 262144 x 512), its throughput and its error against
                the float64 oracle on a column slice.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fast-pauli_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "expval amplitude-terms/s"
UNIT = "amplitude-terms/s"
# float32 FMA-pipe instructions per double-float operation (df64.cuh), by
# the kernel family that performs it (fpg_operator_family_stats):
#  * tile: a product into an offset accumulator (df_fma_offset: 3 fused
#    multiply-adds, 1 more for the rounding error, 2 additions = 6), plus the
#    tile total of each sum, 8 products, into the running sum (1 subtraction +
#    df_add_lazy 8): 6 + 9/8;
#  * marginal, transform: q = conj(a) b formed as df_mul (4) + df_fma (12) per
#    two products: 8;
#  * pair: df_fma, 1 multiply, 3 fused multiply-adds, 8 additions: 12;
#  * direct: native float64 (the float64 pipe): no float32 operations.
# An addition is df_add_lazy (TwoSum and two additions): 8.
DF64_MULADD_OPS = {"tile": 6 + 9 / 8, "marginal": 8, "transform": 8, "pair": 12, "direct": 0}
DF64_ADD_OPS = 8


def host_cpu() -> dict:
    """Host CPU model, logical CPUs and the OpenMP thread setting."""
    import platform

    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"model": model or platform.processor() or platform.machine(), "arch": platform.machine(),
            "nproc": os.cpu_count(), "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS")}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (median SM clock, reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workload
def weight2_problem(n=14, K=1000, S=1024, seed=1002, device="cuda"):
    import numpy as np
    import torch

    import fast_pauli as fp

    strings = [str(s) for s in fp.helpers.calculate_pauli_strings_max_weight(n, 2)][1:]
    P = len(strings)
    rng = np.random.default_rng(seed)
    sd = np.sqrt(1.0 / (2 * P))
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * sd
    g = torch.Generator(device=device).manual_seed(seed)
    D = 1 << n
    psi = torch.complex(torch.randn(D, S, dtype=torch.float64, device=device, generator=g),
                        torch.randn(D, S, dtype=torch.float64, device=device, generator=g))
    psi /= torch.linalg.vector_norm(psi, dim=0, keepdim=True)
    return strings, h, psi


def _stream_handle():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def time_device(fn, steps, warmup):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0 / steps


# ------------------------------------------------------------------ arms
def run_ours(args, rank, world, dist):
    import numpy as np
    import torch

    import fast_pauli as fp
    from fast_pauli import _abi
    from fast_pauli import distributed as fdist

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    n, K, S = 14, 1000, 1024
    strings, h, psi = weight2_problem(n=n, K=K, S=S, seed=1002 + rank)
    P, D = len(strings), 1 << n
    terms = P * D * S
    L = _abi.lib()
    op = _abi.Operator(strings)
    dh = torch.from_numpy(h).cuda()
    out = torch.zeros((K, S), dtype=torch.complex128, device="cuda")
    ev = torch.empty((P, S), dtype=torch.float64, device="cuda")
    stream = _stream_handle()

    def step():
        out.zero_()
        _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, psi.data_ptr(), out.data_ptr(), S,
                                       _abi.FPG_C128, stream))

    def expect_stage():
        _abi.check(L.fpg_expect_strings(op.handle, psi.data_ptr(), ev.data_ptr(), S, _abi.FPG_C128, stream))

    if args.profile:
        # one-shot case for ncu captures: warm-up then a few launches of the stage
        for _ in range(max(1, args.warmup)):
            expect_stage()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize()
        return None

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
        time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = _abi.kernel_launches()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = _abi.kernel_launches() - n0
    t_step = e0.elapsed_time(e1) / 1000.0 / args.steps
    t_step = fdist.max_over_ranks(t_step, dist)
    # dominant stage alone (per-string expectation kernels), same stream
    t_expect = time_device(expect_stage, args.steps, 2)
    clk = clocks.stop() if clocks else None
    if rank != 0:
        return None

    hbm, peak_kind = _peaks()
    fp32_rate = _abi.measure_peak(_abi.FPG_C64, stream)   # float32 FMA lane operations / s
    fp64_rate = _abi.measure_peak(_abi.FPG_C128, stream)  # float64
    nch, visits, adds = op.stats()
    fp64_ops = S * (4 * visits + adds)  # float64 multiply-adds and additions per stage
    fam = op.family_stats()
    fp32_ops = S * sum(4 * v * DF64_MULADD_OPS[f] + (a * DF64_ADD_OPS if DF64_MULADD_OPS[f] else 0)
                       for f, (v, a) in fam.items())
    alg_bytes_expect = terms * 16
    traffic = _ncu_traffic("expect_stage_n14_weight2_fp64.md")
    roof = {
        "bound": "fp32-issue",
        "achieved": fp32_ops / t_expect / 1e12,
        "peak": fp32_rate / 1e12,
        "unit": "T float32 FMA-pipe lane-ops/s",
        "frac": fp32_ops / t_expect / fp32_rate,
        "peak_kind": "measured on this GPU (fpg_measure_peak: independent float32 FMA chains, all SMs)",
        "kernel": "expectation stage (fpg_expect_strings: k_df_split + k_expect_tile + k_expect_marg + k_expect_wht "
                  "+ family reductions)",
        "kernel_ms": t_expect * 1e3,
        "ops_per_launch": fp32_ops,
        "model": "float64 operations of the stage by kernel family (fpg_operator_family_stats: 4 multiply-adds "
                 "per row visit + sign additions) x the float32 instructions that family spends per double-float "
                 "operation: multiply-add 7.125 in the tile kernel (offset accumulators, 6, and the tile "
                 "totals), 8 in the marginal and transform kernels, 12 in the pair kernel; addition 8. "
                 "Loads, index arithmetic, tile maxima and renormalisations are not counted",
        "ops_by_family": {f: S * (4 * v * DF64_MULADD_OPS[f] + (a * DF64_ADD_OPS if DF64_MULADD_OPS[f] else 0))
                          for f, (v, a) in fam.items() if v},
        "traffic": traffic,
        "traffic_source": "ncu DRAM bytes of one stage launch, profiles/expect_stage_n14_weight2_fp64.md "
                          "(captured once, not in this run)",
        "dram_achieved_gbs": traffic / t_expect / 1e9 if traffic else None,
        "dram_frac": traffic / t_expect / 1e9 / hbm if traffic else None,
        "hbm_peak_gbs": hbm,
        "hbm_peak_kind": peak_kind,
        "streaming_equiv": {"bytes_per_launch": alg_bytes_expect, "achieved_gbs": alg_bytes_expect / t_expect / 1e9,
                            "vs_hbm_peak": alg_bytes_expect / t_expect / 1e9 / hbm,
                            "note": "16 B per amplitude-term, the traffic of the reference's per-string streaming; "
                                    "above 1 because the kernels read each amplitude once per kernel family, not "
                                    "once per string"},
        "fp64_pipe": {"ops_per_launch": fp64_ops, "achieved_tflops": 2 * fp64_ops / t_expect / 1e12,
                      "peak_tflops": 2 * fp64_rate / 1e12,
                      "vs_peak": fp64_ops / t_expect / fp64_rate,
                      "note": "the stage's float64 operations per second against the float64 pipe measured on this "
                              "GPU; above 1 because they run as double-float on the float32 pipes"},
    }

    # ---- end to end through the public API, host numpy buffers -----------
    # value: an ordinary (pageable) numpy array, as a drop-in user of the
    # reference passes it; "pinned": the same call on page-locked memory
    e2e = None
    if not args.skip_e2e:
        sop = fp.SummedPauliOp(strings, h)
        pinned = torch.empty((D, S), dtype=torch.complex128, pin_memory=True)
        pinned.copy_(psi.cpu())
        host_pinned = pinned.numpy()
        host_pageable = np.array(host_pinned, copy=True)
        ref_dev = out.cpu().numpy()
        ksteps = max(3, args.steps // 2)

        def e2e_time(host):
            for _ in range(max(3, args.warmup)):  # warm-up (encoding cached, pool buffers mapped)
                res = sop.expectation_value(host)
            t0 = time.perf_counter()
            for _ in range(ksteps):
                res = sop.expectation_value(host)
            t = (time.perf_counter() - t0) / ksteps
            return t, float(np.abs(res - ref_dev).max() / np.abs(ref_dev).max())

        t_pg, err_pg = e2e_time(host_pageable)
        t_pn, err_pn = e2e_time(host_pinned)
        # the same calls with every result kept (each output a fresh numpy
        # allocation, as when a caller collects results)
        kept = []
        t0 = time.perf_counter()
        for _ in range(ksteps):
            kept.append(sop.expectation_value(host_pageable))
        t_kept = (time.perf_counter() - t0) / ksteps
        del kept
        e2e = {"value": world * terms / t_pg, "unit": UNIT,
               "h2d_bytes_per_step": D * S * 16 + P * K * 16, "d2h_bytes_per_step": K * S * 16,
               "ms_per_call": t_pg * 1e3,
               "api": "fast_pauli.SummedPauliOp.expectation_value(numpy array in ordinary pageable host memory)",
               "overlap": "three column chunks of 128, 448 and 448 states: each chunk is copied in while the one "
                          "before it is computed, the chunks' computations alternating between two streams",
               "max_rel_err_vs_device_path": err_pg,
               "results_kept_ms_per_call": t_kept * 1e3,
               "pinned": {"value": world * terms / t_pn, "unit": UNIT, "ms_per_call": t_pn * 1e3,
                          "api": "fast_pauli.SummedPauliOp.expectation_value(numpy array in pinned host memory)",
                          "max_rel_err_vs_device_path": err_pn}}
        del host_pageable, pinned

    # ---- CPU baseline (oracle port, bounded sample) ------------------------
    cpu = None
    if not args.skip_cpu and world == 1:
        cpu = cpu_sample(strings, h, psi, S, n)

    mixed = None
    if not args.skip_mixed:
        mixed = run_mixed(args)

    serve = None
    if not args.skip_serve and world == 1:
        serve = serve_summary()

    line = {
        "metric": METRIC, "value": world * terms / t_step, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128/f64", "data": "synthetic (seeded Gaussian unit-norm states)",
        "config": {"workload": "SummedPauliOp.expectation_value float64: n=14, 861 weight<=2 strings, "
                               "K=1000, states 16384x1024 complex128",
                   "n_qubits": n, "n_strings": P, "n_operators": K, "n_states": S,
                   "l2": "inputs (256 MiB states) larger than L2; no flush",
                   "parallelism": f"replicas x{world} (columns independent, no collective)"},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "launches_per_step": launches / args.steps, "clocks": clk, "mixed": mixed, "serve": serve,
    }
    return line


def cpu_sample(strings, h, psi, S, n):
    """Oracle port (the reference's OpenMP algorithm, all host threads) on the
    whole workload: all 861 strings, K = 1000, all states, one call."""
    import oracle

    host = psi.cpu().numpy()
    oracle.summed_expectation(strings[:2], h[:2], host[:, :8])  # load + warm
    t0 = time.perf_counter()
    oracle.summed_expectation(strings, h, host)
    t = time.perf_counter() - t0
    terms = len(strings) * (1 << n) * S
    return {"value": terms / t, "unit": UNIT, "cores": oracle.max_threads(), "kind": "port",
            "host_cpu": host_cpu(),
            "sample": f"the whole workload: all {len(strings)} strings, K={h.shape[1]}, all {1 << n}x{S} states, "
                      f"one call ({t:.2f} s)"}


def run_profile_c64(args):
    """One-shot complex64 cases for ncu captures (warm-up + args.steps calls)."""
    import numpy as np
    import torch

    import oracle
    from fast_pauli import _abi

    torch.cuda.set_device(0)
    if args.profile == "mixed":
        n, K, S = 18, 1000, 512
        strings, h, psi = weight2_problem(n=n, K=K, S=S, seed=1003)
    else:
        n, K, S = 20, 1, 64
        rng = np.random.default_rng(1006)
        strings = oracle.uniform_strings(rng, n, 1024)
        h = rng.standard_normal((len(strings), K)) + 1j * rng.standard_normal((len(strings), K))
        g = torch.Generator(device="cuda").manual_seed(6)
        psi = torch.complex(torch.randn(1 << n, S, dtype=torch.float64, device="cuda", generator=g),
                            torch.randn(1 << n, S, dtype=torch.float64, device="cuda", generator=g))
        psi /= torch.linalg.vector_norm(psi, dim=0, keepdim=True)
    L = _abi.lib()
    op = _abi.Operator(strings)
    stream = _stream_handle()
    h64 = torch.from_numpy(h).to(torch.complex64).cuda()
    psi64 = psi.to(torch.complex64)
    del psi
    torch.cuda.empty_cache()  # only the complex64 state stays on the device
    out = torch.zeros((K, S), dtype=torch.complex64, device="cuda")
    for _ in range(max(1, args.warmup) + args.steps):
        _abi.check(L.fpg_summed_expect(op.handle, h64.data_ptr(), K, psi64.data_ptr(), out.data_ptr(), S,
                                       _abi.FPG_C64, stream))
    torch.cuda.synchronize()


def run_profile_f64_calls(args):
    """One-shot float64 cases for ncu captures on the n=14 weight<=2
    operators (K=1000): ``apply`` = SummedPauliOp.apply of 256 states
    (fpg_summed_apply: the group-diagonal table and the df64 apply kernel);
    ``chunks`` = fpg_summed_expect of 128 and of 448 states, the widths of
    the host path's column chunks.  Each: warm-up calls, then args.steps."""
    import torch

    from fast_pauli import _abi

    torch.cuda.set_device(0)
    n, K = 14, 1000
    widths = (256,) if args.profile == "apply" else (128, 448)
    L = _abi.lib()
    stream = _stream_handle()
    for S in widths:
        strings, h, psi = weight2_problem(n=n, K=K, S=S, seed=1002)
        op = _abi.Operator(strings)
        dh = torch.from_numpy(h).cuda()
        if args.profile == "apply":
            out = torch.zeros_like(psi)
            call = lambda: _abi.check(L.fpg_summed_apply(op.handle, dh.data_ptr(), K, psi.data_ptr(),
                                                         out.data_ptr(), S, _abi.FPG_C128, stream))
        else:
            out = torch.zeros((K, S), dtype=torch.complex128, device="cuda")
            call = lambda: _abi.check(L.fpg_summed_expect(op.handle, dh.data_ptr(), K, psi.data_ptr(),
                                                          out.data_ptr(), S, _abi.FPG_C128, stream))
        for _ in range(max(1, args.warmup) + args.steps):
            call()
        torch.cuda.synchronize()
        op.close()


def run_profile_batch(args):
    """One-shot case for launch lists: the 256 uneven problems as one batch
    run (default tuning) and one pass of plain per-problem calls."""
    import torch

    from fast_pauli import _abi

    torch.cuda.set_device(0)
    L = _abi.lib()
    stream = _stream_handle()
    g = torch.Generator(device="cuda").manual_seed(4)
    items = []
    for n, strings, c, S in _uneven_problems():
        D = 1 << n
        psi = torch.complex(torch.randn(D, S, device="cuda", generator=g),
                            torch.randn(D, S, device="cuda", generator=g))
        dc = torch.from_numpy(c.reshape(-1, 1)).to(torch.complex64).cuda()
        items.append(dict(n=n, S=S, psi=psi, op=_abi.Operator(strings), c=dc,
                          out=torch.zeros((1, S), dtype=torch.complex64, device="cuda")))
    batch = _abi.Batch(_abi.FPG_C64)
    for it in items:
        batch.add(it["op"], it["c"].data_ptr(), 1, it["psi"].data_ptr(), it["out"].data_ptr(), it["S"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.run(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for it in items:
        _abi.check(L.fpg_summed_expect(it["op"].handle, it["c"].data_ptr(), 1, it["psi"].data_ptr(),
                                       it["out"].data_ptr(), it["S"], _abi.FPG_C64, stream))
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    print(json.dumps({"batch_s": t1 - t0, "plain_s": t2 - t1}), flush=True)


def run_mixed(args):
    """complex64 / float32 path on the n=18 shape: throughput, speed-up over
    the float64 GPU path, and the error against the float64 oracle (on the
    float64 states, before their conversion) over a slice of the columns."""
    import numpy as np
    import torch

    import oracle
    from fast_pauli import _abi

    n, K, S = 18, 1000, 512
    strings, h, psi = weight2_problem(n=n, K=K, S=S, seed=1003)
    P, D = len(strings), 1 << n
    L = _abi.lib()
    op = _abi.Operator(strings)
    stream = _stream_handle()
    h128 = torch.from_numpy(h).cuda()
    h64 = h128.to(torch.complex64)
    psi64 = psi.to(torch.complex64)
    out128 = torch.zeros((K, S), dtype=torch.complex128, device="cuda")
    out64 = torch.zeros((K, S), dtype=torch.complex64, device="cuda")

    def f128():
        out128.zero_()
        _abi.check(L.fpg_summed_expect(op.handle, h128.data_ptr(), K, psi.data_ptr(), out128.data_ptr(), S,
                                       _abi.FPG_C128, stream))

    def f64():
        out64.zero_()
        _abi.check(L.fpg_summed_expect(op.handle, h64.data_ptr(), K, psi64.data_ptr(), out64.data_ptr(), S,
                                       _abi.FPG_C64, stream))

    t128 = time_device(f128, 2, 1)
    steps = max(3, args.steps // 2)
    t64 = time_device(f64, steps, 2)
    ref = out128.cpu().numpy()
    got = out64.cpu().numpy().astype(np.complex128)
    err = np.abs(got - ref)
    den = np.abs(ref).max()
    # the float64 oracle on 32 columns (first 16, last 16)
    cols = np.r_[0:16, S - 16:S]
    psi_slice = psi[:, torch.from_numpy(cols).cuda()].cpu().numpy()
    terms = P * D * S
    del psi, psi64
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    want = oracle.summed_expectation(strings, h, psi_slice)
    t_or = time.perf_counter() - t0
    got_s = got[:, cols]
    err_o = np.abs(got_s - want)
    hbm, _ = _peaks()
    return {"workload": f"n={n}, {P} strings, K={K}, states {D}x{S} complex64", "terms_per_s": terms / t64,
            "ms_per_step": t64 * 1e3, "fp64_ms_per_step": t128 * 1e3, "speedup_vs_fp64": t128 / t64,
            "streaming_equiv_frac_of_hbm": terms * 8 / t64 / 1e9 / hbm,
            "max_normwise_rel_err_vs_oracle": float(err_o.max() / np.abs(want).max()),
            "mean_rel_err_vs_oracle": float(err_o.mean() / np.abs(want).mean()),
            "oracle_sample": f"float64 oracle (C/OpenMP port) on {len(cols)} of {S} columns, all strings and "
                             f"operators ({t_or:.1f} s)",
            "max_normwise_rel_err_vs_fp64_gpu": float(err.max() / den),
            "mean_rel_err_vs_fp64_gpu": float(err.mean() / np.abs(ref).mean())}


def _ncu_traffic(summary: str):
    """DRAM bytes (read + write) of the timed stage from a committed ncu
    summary under profiles/ (the ``traffic_bytes_per_stage:`` line)."""
    import re

    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            m = re.search(r"traffic_bytes_per_stage:\s*([0-9]+)", f.read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


def run_reference(args, rank, world):
    """The reference's own CPU algorithm (oracle/_ref when built from the
    reference sources on this machine, else the C restatement of it) on the
    whole workload every step (all 861 strings, K = 1000, 16384 x 1024
    states), all host threads."""
    if rank != 0:
        return None
    import numpy as np

    import oracle
    from oracle import ref as oref

    n, K, S = 14, 1000, 1024
    rng = np.random.default_rng(1002)
    strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
    P = len(strings)
    h = (rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))) * np.sqrt(1.0 / (2 * P))
    psi = oracle.unit_norm_states(rng, 1 << n, S)
    use_ref = oref.available()
    fn = oref.summed_expectation if use_ref else oracle.summed_expectation
    for _ in range(args.warmup):
        fn(strings, h, psi)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn(strings, h, psi)
    t = (time.perf_counter() - t0) / args.steps
    terms = P * (1 << n) * S
    v = terms / t
    kind = "reference" if use_ref else "port"
    cpu = host_cpu()
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128/f64", "data": "synthetic",
            "config": {"workload": "SummedPauliOp.expectation_value float64: n=14, 861 weight<=2 strings, "
                                   "K=1000, states 16384x1024 complex128",
                       "sample_per_step": "the whole workload (all strings, operators and states)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": oracle.max_threads(), "kind": kind,
                             "host_cpu": cpu,
                             "sample": f"all {P} strings, K={K}, all states, every step"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _uneven_problems(seed=1004, count=256):
    """Uneven batch: n ~ U{8..20}, strings log-uniform in [16, 4096]
    (uniform random strings), states ~ U{1..256}."""
    import numpy as np

    import oracle

    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        n = int(rng.integers(8, 21))
        P = int(np.exp(rng.uniform(np.log(16), np.log(4096))))
        S = int(rng.integers(1, 257))
        strings = oracle.uniform_strings(rng, n, P)
        c = rng.standard_normal(P) + 1j * rng.standard_normal(P)
        probs.append((n, strings, c, S))
    return probs


def run_to_tensor(args):
    """SummedPauliOp.to_tensor: n=12, the 703 weight<=2 strings (identity
    excluded), K=8 operators -> (8, 4096, 4096) complex128 (2.1 GB).  Metric:
    string-rows/s = P * 2^n * K per call (the reference visits each)."""
    import numpy as np
    import torch

    import oracle
    from fast_pauli import _abi

    torch.cuda.set_device(0)
    n, K = 12, 8
    strings, h, _ = weight2_problem(n=n, K=K, S=1, seed=1007)
    P, D = len(strings), 1 << n
    L = _abi.lib()
    op = _abi.Operator(strings)
    stream = _stream_handle()
    dh = torch.from_numpy(h).cuda()
    out = torch.zeros((K, D, D), dtype=torch.complex128, device="cuda")

    def step():
        _abi.check(L.fpg_to_tensor(op.handle, dh.data_ptr(), K, out.data_ptr(), _abi.FPG_C128, stream))

    t = time_device(step, args.steps, args.warmup)
    units = P * D * K
    # parity on a slice: one operator, against the oracle restatement
    out.zero_()
    step()
    torch.cuda.synchronize()
    want0 = oracle.summed_to_tensor(strings[:50], h[:50, :1])
    o2 = torch.zeros((1, D, D), dtype=torch.complex128, device="cuda")
    op2 = _abi.Operator(strings[:50])
    dh2 = torch.from_numpy(np.ascontiguousarray(h[:50, :1])).cuda()
    _abi.check(L.fpg_to_tensor(op2.handle, dh2.data_ptr(), 1, o2.data_ptr(), _abi.FPG_C128, stream))
    err = float(np.abs(o2.cpu().numpy() - want0).max() / np.abs(want0).max())
    tc = time.perf_counter()
    oracle.summed_to_tensor(strings, h[:, :2])
    tc = time.perf_counter() - tc
    return {"metric": "to_tensor string-rows/s", "value": units / t, "unit": "string-rows/s",
            "workload": f"SummedPauliOp.to_tensor float64: n={n}, {P} weight<=2 strings, K={K} -> ({K}, {D}, {D})",
            "ms_per_step": t * 1e3, "steps": args.steps, "warmup": args.warmup,
            "rmw_bytes_per_step": P * D * K * 32, "max_normwise_err_vs_oracle_50_strings": err,
            "cpu_baseline": {"value": P * D * 2 / tc, "unit": "string-rows/s", "cores": oracle.max_threads(),
                             "kind": "port", "sample": f"all {P} strings, 2 of {K} operators ({tc:.2f} s)"}}


def run_square(args):
    """SummedPauliOp.square of the n=14 weight<=2 operator set (861
    weight<=2 strings, K=1000) onto the 91771 strings of weight <= 4.
    Metric: pair-terms/s = P^2 * K per call / time (the reference forms every
    (i, j, k) term)."""
    import numpy as np
    import torch

    import fast_pauli as fp
    import oracle
    from fast_pauli import _abi

    torch.cuda.set_device(0)
    n, K = 14, 1000
    strings, h, _ = weight2_problem(n=n, K=K, S=1, seed=1002)
    sq_strings = [str(s) for s in fp.helpers.calculate_pauli_strings_max_weight(n, 4)]
    P, A = len(strings), len(sq_strings)
    L = _abi.lib()
    op, q = _abi.Operator(strings), _abi.Operator(sq_strings)
    stream = _stream_handle()
    dh = torch.from_numpy(h).cuda()
    out = torch.empty((A, K), dtype=torch.complex128, device="cuda")

    def step():
        _abi.check(L.fpg_summed_square(op.handle, dh.data_ptr(), K, q.handle, out.data_ptr(), _abi.FPG_C128, stream))

    n0 = _abi.kernel_launches()
    t = time_device(step, args.steps, args.warmup)
    launches = (_abi.kernel_launches() - n0) / (args.steps + args.warmup)
    pair_terms = P * P * K
    # end to end: the public API (host coefficients in, host SummedPauliOp out)
    sop = fp.SummedPauliOp(strings, h)
    sop.square()
    t0 = time.perf_counter()
    res = sop.square()
    t_e2e = time.perf_counter() - t0
    e2e_err = float(np.abs(res.coeffs.T - out.cpu().numpy()).max() / np.abs(out.cpu().numpy()).max())
    # CPU baseline: the oracle port of the reference's square on K_s operators
    Ks = 24
    tc = time.perf_counter()
    oracle.summed_square(strings, h[:, :Ks], sq_strings)
    tc = time.perf_counter() - tc
    ref_err = float(np.abs(oracle.summed_square(strings[:200], h[:200, :4], sq_strings)
                           - _square_dev(L, _abi, strings[:200], h[:200, :4], sq_strings, stream)).max())
    return {"metric": "square pair-terms/s", "value": pair_terms / t, "unit": "pair-terms/s",
            "workload": f"SummedPauliOp.square float64: n={n}, {P} weight<=2 strings, K={K} -> {A} strings "
                        "of weight <= 4", "ms_per_step": t * 1e3, "steps": args.steps, "warmup": args.warmup,
            "launches_per_step": launches,
            "e2e": {"value": pair_terms / t_e2e, "unit": "pair-terms/s", "ms": t_e2e * 1e3,
                    "h2d_bytes": P * K * 16, "d2h_bytes": A * K * 16,
                    "api": "fast_pauli.SummedPauliOp.square()", "max_rel_diff_vs_device_call": e2e_err},
            "max_abs_err_vs_oracle_200_strings": ref_err,
            "cpu_baseline": {"value": P * P * Ks / tc, "unit": "pair-terms/s", "cores": oracle.max_threads(),
                             "kind": "port", "sample": f"all {P}^2 pairs, {Ks} of {K} operators ({tc:.2f} s)"}}


def run_product(args):
    """PauliOp @ PauliOp with equal strings merged (fpg_op_product): the
    n=14 weight<=2 operator set (861 strings) times itself
    with seeded complex coefficients, 741321 string pairs -> the distinct
    strings of weight <= 4.  Metric: string pairs/s."""
    import numpy as np
    import torch

    import fast_pauli as fp
    import oracle
    from fast_pauli import _abi

    torch.cuda.set_device(0)
    n = 14
    strings = [str(s) for s in fp.helpers.calculate_pauli_strings_max_weight(n, 2)][1:]
    P = len(strings)
    rng = np.random.default_rng(1005)
    c = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    L = _abi.lib()
    op = _abi.Operator(strings)
    stream = _stream_handle()
    dc = torch.from_numpy(c).cuda()
    N = P * P
    ox = torch.empty(N, dtype=torch.int64, device="cuda")
    oz = torch.empty(N, dtype=torch.int64, device="cuda")
    oc = torch.empty(N, dtype=torch.complex128, device="cuda")
    n_out = ctypes.c_int64(0)

    def step():
        _abi.check(L.fpg_op_product(op.handle, dc.data_ptr(), op.handle, dc.data_ptr(), ox.data_ptr(), oz.data_ptr(),
                                    oc.data_ptr(), ctypes.byref(n_out), stream))

    n0 = _abi.kernel_launches()
    t = time_device(step, args.steps, args.warmup)
    launches = (_abi.kernel_launches() - n0) / (args.steps + args.warmup)
    # end to end: the public API (host coefficients and strings in, host PauliOp out)
    a = fp.PauliOp(list(c), strings)
    a @ a
    t0 = time.perf_counter()
    res = a @ a
    t_e2e = time.perf_counter() - t0
    # CPU baseline and parity: the oracle's restatement of the reference's
    # product, all pairs
    tc = time.perf_counter()
    want = oracle.op_product(c, strings, c, strings)
    tc = time.perf_counter() - tc
    got = dict(zip(res.pauli_strings_as_str, res.coeffs))
    err = max(abs(got[s] - w) for s, w in want.items()) / max(abs(w) for w in want.values())
    same = sorted(got) == sorted(want)
    return {"metric": "product string-pairs/s", "value": N / t, "unit": "string-pairs/s",
            "workload": f"PauliOp @ PauliOp float64: n={n}, {P} x {P} weight<=2 strings -> {n_out.value} distinct",
            "ms_per_step": t * 1e3, "steps": args.steps, "warmup": args.warmup, "launches_per_step": launches,
            "e2e": {"value": N / t_e2e, "unit": "string-pairs/s", "ms": t_e2e * 1e3, "h2d_bytes": P * 16,
                    "d2h_bytes": int(n_out.value) * 32, "api": "fast_pauli.PauliOp.__matmul__"},
            "parity_vs_oracle": {"same_strings": same, "max_rel_err": float(err)},
            "cpu_baseline": {"value": N / tc, "unit": "string-pairs/s", "cores": 1, "kind": "port",
                             "sample": f"all {N} pairs ({tc:.2f} s, one hash map, serial)"}}


def _square_dev(L, _abi, strings, h, sq_strings, stream):
    import torch

    op, q = _abi.Operator(strings), _abi.Operator(sq_strings)
    dh = torch.from_numpy(h).cuda()
    out = torch.empty((len(sq_strings), h.shape[1]), dtype=torch.complex128, device="cuda")
    _abi.check(L.fpg_summed_square(op.handle, dh.data_ptr(), h.shape[1], q.handle, out.data_ptr(), _abi.FPG_C128,
                                   stream))
    res = out.cpu().numpy()
    op.close()
    q.close()
    return res


def run_batch(args):
    """Uneven batch: 256 PauliOp.expectation_value problems in one
    persistent, graph-captured launch (tuning from the autotuner, tuned on the
    problems with n <= 14) versus 256 separate plain launches."""
    import numpy as np
    import torch

    import oracle
    from fast_pauli import _abi

    torch.cuda.set_device(0)
    L = _abi.lib()
    probs = _uneven_problems()
    stream = _stream_handle()
    g = torch.Generator(device="cuda").manual_seed(4)
    items = []
    for n, strings, c, S in probs:
        D = 1 << n
        psi = torch.complex(torch.randn(D, S, device="cuda", generator=g),
                            torch.randn(D, S, device="cuda", generator=g))
        psi /= torch.linalg.vector_norm(psi.to(torch.complex128), dim=0, keepdim=True).to(torch.float32)
        op = _abi.Operator(strings)
        dc = torch.from_numpy(c.reshape(-1, 1)).to(torch.complex64).cuda()
        items.append(dict(n=n, P=len(strings), S=S, psi=psi, op=op, c=dc,
                          out_b=torch.zeros((1, S), dtype=torch.complex64, device="cuda"),
                          out_p=torch.zeros((1, S), dtype=torch.complex64, device="cuda")))
    terms = sum(it["P"] * (1 << it["n"]) * it["S"] for it in items)
    # autotune on the small problems (a proxy: same kernels, a fraction of the time)
    proxy = _abi.Batch(_abi.FPG_C64)
    for it in items:
        if it["n"] <= 14:
            proxy.add(it["op"], it["c"].data_ptr(), 1, it["psi"].data_ptr(), it["out_b"].data_ptr(), it["S"])
    best, best_ms = proxy.autotune(stream)
    proxy.close()
    batch = _abi.Batch(_abi.FPG_C64)
    for it in items:
        batch.add(it["op"], it["c"].data_ptr(), 1, it["psi"].data_ptr(), it["out_b"].data_ptr(), it["S"])
    batch.plan(_abi.BatchTuning(best["threads_per_cta"], best["ctas_per_sm"], best["rows_per_item"],
                                best["tile_mb"]))
    n0 = _abi.kernel_launches()
    t_batch = time_device(lambda: batch.run_graph(stream), args.steps, max(1, args.warmup))
    launches_batch = (_abi.kernel_launches() - n0) / (args.steps + max(1, args.warmup))

    def plain():
        for it in items:
            it["out_p"].zero_()
            _abi.check(L.fpg_summed_expect(it["op"].handle, it["c"].data_ptr(), 1, it["psi"].data_ptr(),
                                           it["out_p"].data_ptr(), it["S"], _abi.FPG_C64, stream))

    n0 = _abi.kernel_launches()
    t_plain = time_device(plain, max(1, args.steps // 2), 1)
    launches_plain = (_abi.kernel_launches() - n0) / (max(1, args.steps // 2) + 1)
    # agreement batch vs plain, and the smallest problems vs the CPU oracle
    err_bp = max(normwise_np(it["out_b"].cpu().numpy(), it["out_p"].cpu().numpy()) for it in items)
    small = sorted(range(len(items)), key=lambda i: items[i]["P"] * (1 << items[i]["n"]) * items[i]["S"])[:6]
    err_or = 0.0
    cpu_terms, cpu_t = 0, 0.0
    for i in small:
        n, strings, c, S = probs[i]
        psi = items[i]["psi"].cpu().numpy().astype(np.complex128)
        t0 = time.perf_counter()
        want = oracle.op_expectation(strings, c, psi)
        cpu_t += time.perf_counter() - t0
        cpu_terms += len(strings) * (1 << n) * S
        err_or = max(err_or, normwise_np(items[i]["out_b"].cpu().numpy()[0], want))
    hbm, _ = _peaks()
    return {"metric": METRIC, "workload": "uneven batch: 256 PauliOp.expectation_value, n~U{8..20}, P log-uniform "
                                          "16..4096 uniform strings, S~U{1..256}, complex64",
            "value": terms / t_batch, "unit": UNIT, "ms_per_step": t_batch * 1e3, "steps": args.steps,
            "plain_value": terms / t_plain, "plain_ms_per_step": t_plain * 1e3, "speedup_vs_plain": t_plain / t_batch,
            "terms": terms, "streaming_equiv_frac_of_hbm": terms * 8 / t_batch / 1e9 / hbm,
            "launches_per_step": launches_batch, "plain_launches_per_step": launches_plain,
            "tuning": best, "autotune_proxy_ms": best_ms,
            "max_normwise_diff_batch_vs_plain": err_bp, "max_normwise_err_vs_oracle_smallest6": err_or,
            "cpu_baseline": {"value": cpu_terms / cpu_t, "unit": UNIT, "cores": oracle.max_threads(),
                             "kind": "port", "sample": "the 6 smallest problems"}}


def normwise_np(got, want):
    import numpy as np

    den = np.abs(want).max()
    return float(np.abs(got - want).max() / den) if den > 0 else float(np.abs(got - want).max())


def _serve_requests(n_req, max_n, seed=1005):
    """Poisson-mix requests (n ~ U{10..max_n}, strings log-uniform 32..2048,
    S ~ U{1..64}, K log-uniform 1..64, 50/50 expectation_value /
    apply_weighted, complex64), with resident operators and device arrays."""
    import numpy as np
    import torch

    import oracle
    from fast_pauli import _abi

    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda").manual_seed(5)
    reqs = []
    for _ in range(n_req):
        n = int(rng.integers(10, max_n + 1))
        P = int(np.exp(rng.uniform(np.log(32), np.log(2048))))
        S = int(rng.integers(1, 65))
        K = int(np.exp(rng.uniform(0, np.log(64))))
        kind = _abi.FPG_REQ_EXPECT if rng.random() < 0.5 else _abi.FPG_REQ_APPLY_WEIGHTED
        strings = oracle.uniform_strings(rng, n, P)
        D = 1 << n
        psi = torch.complex(torch.randn(D, S, device="cuda", generator=g),
                            torch.randn(D, S, device="cuda", generator=g))
        psi /= torch.linalg.vector_norm(psi, dim=0, keepdim=True)
        h = torch.complex(torch.randn(P, K, device="cuda", generator=g), torch.randn(P, K, device="cuda", generator=g))
        data = torch.randn(K, S, device="cuda", generator=g)
        out_shape = (K, S) if kind == _abi.FPG_REQ_EXPECT else (D, S)
        reqs.append(dict(n=n, P=P, S=S, K=K, kind=kind, op=_abi.Operator(strings), psi=psi, h=h, data=data,
                         out=torch.empty(out_shape, dtype=torch.complex64, device="cuda")))
    torch.cuda.synchronize()
    return reqs, rng.exponential(1.0, size=n_req)


def _serve_once(reqs, unit_gaps, n_slots, rate, budget_gb):
    """Submit the requests at Poisson arrival times (unit_gaps / rate) to a
    server with n_slots slots; latency = completion - arrival."""
    import numpy as np

    from fast_pauli import _abi

    gaps = unit_gaps / rate
    srv = _abi.Server(_abi.FPG_C64, n_slots=n_slots, hbm_budget_bytes=budget_gb << 30)
    r0 = min(reqs, key=lambda r: r["P"] << r["n"])  # warm-up: one small request
    srv.wait(srv.submit(r0["kind"], r0["op"], r0["h"].data_ptr(), r0["K"], r0["psi"].data_ptr(),
                        r0["out"].data_ptr(), r0["S"], r0["data"].data_ptr()))
    tickets = []
    t0 = time.perf_counter()
    arrive = t0
    for r, gap in zip(reqs, gaps):
        arrive += gap
        while time.perf_counter() < arrive:
            time.sleep(min(1e-4, max(0.0, arrive - time.perf_counter())))
        tickets.append(srv.submit(r["kind"], r["op"], r["h"].data_ptr(), r["K"], r["psi"].data_ptr(),
                                  r["out"].data_ptr(), r["S"], r["data"].data_ptr()))
    infos = [srv.wait(t) for t in tickets]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([(i["done_us"] - i["submit_us"]) / 1e3 for i in infos])
    return lat, wall, st


def _plain_once(reqs, unit_gaps, rate):
    """The plain per-request path: each request's library call
    (fpg_summed_expect or fpg_summed_apply_weighted, output zeroed first)
    issued on one stream at its arrival, first come first served; completion
    = its event on the stream, read as host time from an event recorded at
    the start while the GPU was idle."""
    import numpy as np
    import torch

    from fast_pauli import _abi

    L = _abi.lib()
    st = torch.cuda.current_stream()
    handle = ctypes.c_void_p(st.cuda_stream)

    def issue(r):
        r["out"].zero_()
        if r["kind"] == _abi.FPG_REQ_EXPECT:
            _abi.check(L.fpg_summed_expect(r["op"].handle, r["h"].data_ptr(), r["K"], r["psi"].data_ptr(),
                                           r["out"].data_ptr(), r["S"], _abi.FPG_C64, handle))
        else:
            _abi.check(L.fpg_summed_apply_weighted(r["op"].handle, r["h"].data_ptr(), r["K"], r["psi"].data_ptr(),
                                                   r["data"].data_ptr(), r["out"].data_ptr(), r["S"], _abi.FPG_C64,
                                                   handle))

    issue(min(reqs, key=lambda r: r["P"] << r["n"]))  # warm-up
    torch.cuda.synchronize()
    gaps = unit_gaps / rate
    e0 = torch.cuda.Event(enable_timing=True)
    done = [torch.cuda.Event(enable_timing=True) for _ in reqs]
    arrivals = []
    t0 = time.perf_counter()
    e0.record(st)
    arrive = t0
    for r, gap, ev in zip(reqs, gaps, done):
        arrive += gap
        while time.perf_counter() < arrive:
            time.sleep(min(1e-4, max(0.0, arrive - time.perf_counter())))
        arrivals.append(arrive - t0)
        issue(r)
        ev.record(st)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    lat = np.array([e0.elapsed_time(ev) - a * 1e3 for ev, a in zip(done, arrivals)])
    return lat, wall


def _service_alone(reqs, budget_gb):
    """GPU service time of every request alone (one slot, one at a time)."""
    import numpy as np

    from fast_pauli import _abi

    alone = []
    srv = _abi.Server(_abi.FPG_C64, n_slots=1, hbm_budget_bytes=budget_gb << 30)
    for r in reqs:
        info = srv.wait(srv.submit(r["kind"], r["op"], r["h"].data_ptr(), r["K"], r["psi"].data_ptr(),
                                   r["out"].data_ptr(), r["S"], r["data"].data_ptr()))
        alone.append((info["done_us"] - info["start_us"]) / 1e3)
    srv.close()
    return np.array(alone)


def _latency_row(lat, ns, alone, wall, terms, n_req, st, slots, target_ms=10.0):
    import numpy as np

    le20 = ns <= 20
    feasible = le20 & (alone < target_ms)
    buckets = {}
    for lo, hi in ((10, 14), (15, 20), (21, 24)):
        m = (ns >= lo) & (ns <= hi)
        if m.any():
            buckets[f"n{lo}-{hi}"] = {"count": int(m.sum()), "p50_ms": float(np.percentile(lat[m], 50)),
                                      "p99_ms": float(np.percentile(lat[m], 99))}
    row = {"slots": slots, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "p99_ms_n_le_20": float(np.percentile(lat[le20], 99)) if le20.any() else None,
           "p99_ms_n_le_20_alone_under_10ms": float(np.percentile(lat[feasible], 99)) if feasible.any() else None,
           "count_n_le_20": int(le20.sum()), "count_n_le_20_alone_under_10ms": int(feasible.sum()),
           "throughput_terms_per_s": terms / wall, "requests_per_s": n_req / wall, "wall_s": wall, "by_n": buckets}
    if st is not None:
        row.update({"peak_running": st["peak_running"], "peak_reserved_gb": st["peak_reserved_bytes"] / 2**30,
                    "merged_runs": st["merged_runs"], "merged_requests": st["merged_requests"]})
    return row


def run_serve(args):
    """Serving: Poisson arrivals of expectation_value / apply_weighted
    requests (n ~ U{10..max_n}, strings log-uniform 32..2048, S ~ U{1..64},
    K log-uniform 1..64, complex64) against the serving loop (continuous
    admission, 8 slots, HBM budget, small expectation requests merged) and
    against the plain per-request path (each request's library call issued on
    one stream at its arrival).  Latency = completion - arrival.  Then a
    burst of small expectation requests at a high rate, both ways."""
    import numpy as np
    import torch

    from fast_pauli import _abi

    torch.cuda.set_device(0)
    n_req = args.requests
    reqs, unit_gaps = _serve_requests(n_req, args.max_n)
    terms = sum(r["P"] * (1 << r["n"]) * r["S"] for r in reqs)
    rates = [float(x) for x in args.rates.split(",")]
    ns = np.array([r["n"] for r in reqs])
    alone = _service_alone(reqs, args.budget_gb)
    le20 = ns <= 20
    out = {"metric": "serving latency ms / amplitude-terms/s",
           "workload": f"serving: {n_req} requests per rate, Poisson rates {rates}/s, n~U{{10..{args.max_n}}}, "
                       "P log-uniform 32..2048 uniform strings, S~U{1..64}, K log-uniform 1..64, "
                       "50/50 expectation_value / apply_weighted, complex64",
           "service_alone_ms": {"p50": float(np.percentile(alone, 50)), "p99": float(np.percentile(alone, 99)),
                                "p99_n_le_20": float(np.percentile(alone[le20], 99)),
                                "sum_s": float(alone.sum()) / 1e3},
           "capacity_requests_per_s": n_req / (float(alone.sum()) / 1e3),
           "sweep": []}
    for rate in rates:
        row = {"rate_per_s": rate}
        lat, wall, st = _serve_once(reqs, unit_gaps, args.slots, rate, args.budget_gb)
        row["served"] = _latency_row(lat, ns, alone, wall, terms, n_req, st, args.slots)
        lat, wall = _plain_once(reqs, unit_gaps, rate)
        row["plain_per_request"] = _latency_row(lat, ns, alone, wall, terms, n_req, None, 1)
        out["sweep"].append(row)
    # a burst of small expectation requests (n <= 14): what merging them into
    # shared launch sequences buys over one call each
    small = [r for r in reqs if r["kind"] == _abi.FPG_REQ_EXPECT and r["n"] <= 14]
    if small:
        burst = [dict(small[i % len(small)]) for i in range(args.burst)]
        for r in burst:
            r["out"] = torch.empty_like(r["out"])  # one output per request in flight
        gaps = np.full(len(burst), 1.0)
        bterms = sum(r["P"] * (1 << r["n"]) * r["S"] for r in burst)
        bns = np.array([r["n"] for r in burst])
        balone = np.zeros(len(burst))
        lat, wall, st = _serve_once(burst, gaps, args.slots, args.burst_rate, args.budget_gb)
        row = {"rate_per_s": args.burst_rate, "requests": len(burst),
               "served": _latency_row(lat, bns, balone, wall, bterms, len(burst), st, args.slots)}
        lat, wall = _plain_once(burst, gaps, args.burst_rate)
        row["plain_per_request"] = _latency_row(lat, bns, balone, wall, bterms, len(burst), None, 1)
        out["small_expectation_burst"] = row
    return out


def serve_summary(n_req=40, rate=4.0, max_n=24, slots=8, budget_gb=64):
    """Short serving run for the default line: one Poisson rate, the same
    request mix as --workload serve, p50 / p99 overall and by qubit count,
    and the p99 over the requests of n <= 20 whose GPU service time alone is
    under 10 ms (the larger ones cannot meet a 10 ms target on one GPU: their
    own work takes longer)."""
    import numpy as np
    import torch

    from fast_pauli import _abi

    reqs, unit_gaps = _serve_requests(n_req, max_n)
    terms = sum(r["P"] * (1 << r["n"]) * r["S"] for r in reqs)
    ns = np.array([r["n"] for r in reqs])
    work = np.array([r["P"] * (1 << r["n"]) * r["S"] for r in reqs], dtype=np.float64)
    alone = _service_alone(reqs, budget_gb)
    lat, wall, st = _serve_once(reqs, unit_gaps, slots, rate, budget_gb)
    row = _latency_row(lat, ns, alone, wall, terms, n_req, st, slots)
    slow = (ns <= 20) & (alone >= 10.0)
    # a burst of small expectation requests arriving faster than they are
    # served: queued ones are merged into shared runs
    burst = None
    small = [r for r in reqs if r["kind"] == _abi.FPG_REQ_EXPECT and r["n"] <= 14]
    if small:
        breqs = [dict(small[i % len(small)]) for i in range(200)]
        for r in breqs:
            r["out"] = torch.empty_like(r["out"])
        gaps = np.full(len(breqs), 1.0)
        blat, bwall, bst = _serve_once(breqs, gaps, slots, 20000.0, budget_gb)
        plat, pwall = _plain_once(breqs, gaps, 20000.0)
        burst = {"requests": len(breqs), "rate_per_s": 20000.0,
                 "served": {"p50_ms": float(np.percentile(blat, 50)), "p99_ms": float(np.percentile(blat, 99)),
                            "requests_per_s": len(breqs) / bwall, "merged_runs": bst["merged_runs"],
                            "merged_requests": bst["merged_requests"]},
                 "plain_per_request": {"p50_ms": float(np.percentile(plat, 50)),
                                       "p99_ms": float(np.percentile(plat, 99)),
                                       "requests_per_s": len(breqs) / pwall}}
        del breqs
    out = {"workload": f"{n_req} requests, Poisson {rate}/s, n~U{{10..{max_n}}}, P log-uniform 32..2048 uniform "
                       "strings, S~U{1..64}, K log-uniform 1..64, 50/50 expectation_value / apply_weighted, "
                       "complex64, 8 slots",
           "rate_per_s": rate, **row,
           "service_alone_ms": {"p50": float(np.percentile(alone, 50)), "p99": float(np.percentile(alone, 99))},
           "n_le_20_over_10ms_alone": {"count": int(slow.sum()),
                                       "min_terms": float(work[slow].min()) if slow.any() else None,
                                       "min_alone_ms": float(alone[slow].min()) if slow.any() else None},
           "small_expectation_burst": burst}
    del reqs
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", nargs="?", const="summed", default=None,
                    choices=["summed", "mixed", "random", "batch", "apply", "chunks"],
                    help="short device-only run for ncu captures: summed = the n=14 weight<=2 workload (float64), "
                         "mixed = the n=18 complex64 shape (tensor-core contraction), "
                         "random = n=20, 1024 uniform random strings, 64 states, complex64, "
                         "batch = the 256 uneven problems: one batch run and one pass of plain calls, "
                         "apply = float64 SummedPauliOp.apply, n=14 weight<=2, 256 states, "
                         "chunks = float64 expectation calls of 128 and 448 states (the host column chunks)")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-mixed", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--workload", default="summed", choices=["summed", "batch", "serve", "square", "to_tensor", "product"],
                    help="summed: the n=14 weight<=2 SummedPauliOp workload (default line); batch: 256 uneven problems; "
                         "serve: the request loop; "
                         "square: SummedPauliOp.square of the n=14 weight<=2 operators")
    ap.add_argument("--requests", type=int, default=60, help="serve: requests per rate")
    ap.add_argument("--rates", default="2,4,8", help="serve: Poisson arrival rates to sweep (requests/s)")
    ap.add_argument("--max-n", type=int, default=24, help="serve: largest qubit count")
    ap.add_argument("--slots", type=int, default=8, help="serve: concurrent request slots")
    ap.add_argument("--budget-gb", type=int, default=64, help="serve: HBM budget for request scratch")
    ap.add_argument("--burst", type=int, default=400, help="serve: small expectation requests in the burst")
    ap.add_argument("--burst-rate", type=float, default=20000.0, help="serve: arrival rate of the burst (1/s)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.profile in ("mixed", "random"):
        run_profile_c64(args)
        return
    if args.profile == "batch":
        run_profile_batch(args)
        return
    if args.profile in ("apply", "chunks"):
        run_profile_f64_calls(args)
        return
    if args.workload != "summed" and args.impl == "ours":
        if rank == 0:
            line = {"batch": run_batch, "serve": run_serve, "square": run_square,
                    "to_tensor": run_to_tensor, "product": run_product}[args.workload](args)
            print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    try:
        line = run_ours(args, rank, world, dist)
        if line is not None and rank == 0:
            print(json.dumps(line), flush=True)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
