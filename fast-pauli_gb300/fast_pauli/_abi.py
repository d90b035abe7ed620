"""ctypes binding of the C ABI in include/fpg.h (libfpg.so).

This is the raw drop-in boundary: plain device pointers, sizes and a stream
handle.  Tests and bench.py call the engine through it with device buffers
(e.g. torch CUDA tensors' ``data_ptr()``); the Python classes in
``fast_pauli`` go through the C++ host API instead.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfpg.so")

FPG_OK = 0
FPG_ERR_INVALID = 1
FPG_ERR_CUDA = 2
FPG_ERR_NOMEM = 3
FPG_ERR_UNSUPPORTED = 4
FPG_ERR_TIMEOUT = 5
FPG_ERR_BUSY = 6

FPG_C128 = 0
FPG_C64 = 1

_lib = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_PI32 = ctypes.POINTER(ctypes.c_int32)
_PI64 = ctypes.POINTER(ctypes.c_int64)

# name -> (restype, argtypes); mirrors include/fpg.h
SIGNATURES = {
    "fpg_abi_version": (ctypes.c_int, []),
    "fpg_last_error": (ctypes.c_char_p, []),
    "fpg_kernel_launches": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint64)]),
    "fpg_device_error": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), _P]),
    "fpg_measure_peak": (ctypes.c_int, [_I32, ctypes.POINTER(ctypes.c_double), _P]),
    "fpg_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "fpg_pointer_is_device": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "fpg_device_alloc": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_size_t, _P]),
    "fpg_device_free": (ctypes.c_int, [_P, _P]),
    "fpg_release_cached_memory": (ctypes.c_int, []),
    "fpg_operator_create": (ctypes.c_int, [ctypes.c_char_p, _I64, _I32, ctypes.POINTER(_P)]),
    "fpg_operator_destroy": (ctypes.c_int, [_P]),
    "fpg_operator_info": (ctypes.c_int, [_P, _PI32, _PI64, _PI64]),
    "fpg_operator_stats": (ctypes.c_int, [_P, _PI64, _PI64, _PI64]),
    "fpg_operator_family_stats": (ctypes.c_int, [_P, _PI64, _PI64]),
    "fpg_sparse_repr": (ctypes.c_int, [ctypes.c_char_p, _I32, _P, _P, _P]),
    "fpg_apply": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I32, _P]),
    "fpg_expect_strings": (ctypes.c_int, [_P, _P, _P, _I64, _I32, _P]),
    "fpg_summed_expect": (ctypes.c_int, [_P, _P, _I64, _P, _P, _I64, _I32, _P]),
    "fpg_summed_apply": (ctypes.c_int, [_P, _P, _I64, _P, _P, _I64, _I32, _P]),
    "fpg_summed_apply_weighted": (ctypes.c_int, [_P, _P, _I64, _P, _P, _P, _I64, _I32, _P]),
    "fpg_op_product": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _PI64, _P]),
    "fpg_summed_square": (ctypes.c_int, [_P, _P, _I64, _P, _P, _I32, _P]),
    "fpg_to_tensor": (ctypes.c_int, [_P, _P, _I64, _P, _I32, _P]),
    "fpg_summed_expect_noalloc": (ctypes.c_int, [ctypes.c_char_p, _I64, _I32, _P, _I64, _P, _P, _I64, _I32, _P]),
    "fpg_batch_create": (ctypes.c_int, [_I32, ctypes.POINTER(_P)]),
    "fpg_batch_add": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64]),
    "fpg_batch_plan": (ctypes.c_int, [_P, _P]),
    "fpg_batch_run": (ctypes.c_int, [_P, _P]),
    "fpg_batch_run_graph": (ctypes.c_int, [_P, _P]),
    "fpg_batch_autotune": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(ctypes.c_double)]),
    "fpg_batch_info": (ctypes.c_int, [_P, _PI64, _PI64, _P]),
    "fpg_batch_destroy": (ctypes.c_int, [_P]),
}


FPG_REQ_EXPECT = 0
FPG_REQ_APPLY_WEIGHTED = 1


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("op", _P), ("coeffs", _P),
                ("n_operators", ctypes.c_int64), ("states", _P), ("data", _P), ("out", _P),
                ("n_states", ctypes.c_int64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("n_slots", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("max_queue", ctypes.c_int64)]


class TicketInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("reserved", ctypes.c_int32), ("scratch_bytes", ctypes.c_int64),
                ("submit_us", ctypes.c_double), ("start_us", ctypes.c_double), ("done_us", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("failed", ctypes.c_int64), ("refused", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("peak_running", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("peak_reserved_bytes", ctypes.c_int64), ("merged_runs", ctypes.c_int64),
                ("merged_requests", ctypes.c_int64)]


SIGNATURES.update({
    "fpg_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "fpg_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "fpg_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(TicketInfo)]),
    "fpg_server_release": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "fpg_server_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    "fpg_server_destroy": (ctypes.c_int, [_P]),
})


class BatchTuning(ctypes.Structure):
    _fields_ = [("threads_per_cta", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("rows_per_item", ctypes.c_int32), ("tile_mb", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {"threads_per_cta": self.threads_per_cta, "ctas_per_sm": self.ctas_per_sm,
                "rows_per_item": self.rows_per_item, "tile_mb": self.tile_mb}


class FpgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fpg error {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def kernel_launches() -> int:
    v = ctypes.c_uint64()
    check(lib().fpg_kernel_launches(ctypes.byref(v)))
    return int(v.value)


def measure_peak(dtype: int, stream=None) -> float:
    """Measured FMA lane operations per second of the current device:
    FPG_C64 = the float32 pipe, FPG_C128 = the float64 pipe."""
    v = ctypes.c_double()
    check(lib().fpg_measure_peak(dtype, ctypes.byref(v), stream))
    return float(v.value)


def check(rc: int) -> None:
    if rc != FPG_OK:
        raise FpgError(rc, lib().fpg_last_error().decode())


class Operator:
    """Owning handle of an fpg_operator (encoded strings on the device)."""

    def __init__(self, strings: list[str]):
        strings = [str(s) for s in strings]
        n = len(strings[0]) if strings else 1
        self.n_qubits = n
        self.n_strings = len(strings)
        self._h = _P()
        check(lib().fpg_operator_create("".join(strings).encode(), len(strings), n, ctypes.byref(self._h)))

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def info(self) -> tuple[int, int, int]:
        n = ctypes.c_int32()
        p = ctypes.c_int64()
        g = ctypes.c_int64()
        check(lib().fpg_operator_info(self._h, ctypes.byref(n), ctypes.byref(p), ctypes.byref(g)))
        return n.value, p.value, g.value

    def stats(self) -> tuple[int, int, int]:
        """(chunks, row visits per column, signed accumulations per column)."""
        c = ctypes.c_int64()
        v = ctypes.c_int64()
        a = ctypes.c_int64()
        check(lib().fpg_operator_stats(self._h, ctypes.byref(c), ctypes.byref(v), ctypes.byref(a)))
        return c.value, v.value, a.value

    FAMILIES = ("direct", "transform", "pair", "marginal", "tile")

    def family_stats(self) -> dict[str, tuple[int, int]]:
        """{family: (row visits per column, signed accumulations per column)}."""
        v = (ctypes.c_int64 * len(self.FAMILIES))()
        a = (ctypes.c_int64 * len(self.FAMILIES))()
        check(lib().fpg_operator_family_stats(self._h, v, a))
        return {f: (v[i], a[i]) for i, f in enumerate(self.FAMILIES)}

    def close(self) -> None:
        if self._h:
            lib().fpg_operator_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Owning handle of an fpg_server (device-resident request loop)."""

    def __init__(self, dtype: int, n_slots: int = 4, hbm_budget_bytes: int = 8 << 30, max_queue: int = 0):
        self._h = _P()
        cfg = ServerConfig(dtype, n_slots, hbm_budget_bytes, max_queue)
        check(lib().fpg_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def submit(self, kind: int, op: "Operator", coeffs_ptr: int, n_operators: int, states_ptr: int, out_ptr: int,
               n_states: int, data_ptr: int = 0) -> int:
        req = Request(kind, 0, op.handle, coeffs_ptr, n_operators, states_ptr, data_ptr or None, out_ptr, n_states)
        t = ctypes.c_uint64()
        check(lib().fpg_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> dict:
        info = TicketInfo()
        check(lib().fpg_server_wait(self._h, ticket, timeout_ms, ctypes.byref(info)))
        return {"status": info.status, "scratch_bytes": info.scratch_bytes, "submit_us": info.submit_us,
                "start_us": info.start_us, "done_us": info.done_us}

    def release(self, ticket: int) -> None:
        check(lib().fpg_server_release(self._h, ticket))

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().fpg_server_stats(self._h, ctypes.byref(s)))
        return {"completed": s.completed, "failed": s.failed, "refused": s.refused, "queued": s.queued,
                "peak_running": s.peak_running, "peak_reserved_bytes": s.peak_reserved_bytes,
                "merged_runs": s.merged_runs, "merged_requests": s.merged_requests}

    def close(self) -> None:
        if self._h:
            lib().fpg_server_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Owning handle of an fpg_batch; keeps the operators (and any arrays the
    caller hands over in ``keep``) alive while the batch exists."""

    def __init__(self, dtype: int):
        self._h = _P()
        self._keep: list = []
        check(lib().fpg_batch_create(dtype, ctypes.byref(self._h)))

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def add(self, op: Operator, coeffs_ptr: int, n_operators: int, states_ptr: int, out_ptr: int, n_states: int,
            keep=()) -> None:
        self._keep.append(op)
        self._keep.extend(keep)
        check(lib().fpg_batch_add(self._h, op.handle, coeffs_ptr, n_operators, states_ptr, out_ptr, n_states))

    def plan(self, tuning: "BatchTuning | None" = None) -> None:
        check(lib().fpg_batch_plan(self._h, ctypes.byref(tuning) if tuning is not None else None))

    def run(self, stream) -> None:
        check(lib().fpg_batch_run(self._h, stream))

    def run_graph(self, stream) -> None:
        check(lib().fpg_batch_run_graph(self._h, stream))

    def autotune(self, stream) -> tuple[dict, float]:
        best = BatchTuning()
        ms = ctypes.c_double()
        check(lib().fpg_batch_autotune(self._h, stream, ctypes.byref(best), ctypes.byref(ms)))
        return best.as_dict(), ms.value

    def info(self) -> tuple[int, int, dict]:
        n = ctypes.c_int64()
        it = ctypes.c_int64()
        t = BatchTuning()
        check(lib().fpg_batch_info(self._h, ctypes.byref(n), ctypes.byref(it), ctypes.byref(t)))
        return n.value, it.value, t.as_dict()

    def close(self) -> None:
        if self._h:
            lib().fpg_batch_destroy(self._h)
            self._h = _P()
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
