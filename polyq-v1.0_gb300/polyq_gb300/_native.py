"""ctypes binding of include/polyq_gb300.h.

This is the Python-side stub a maintainer of the reference would add in place of the
PyO3 module (src/pybind.rs): plain C types only.  Loading fails loudly when the native
library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as ct
import os
import threading

from .build import LIB_PATH

_lock = threading.Lock()
_lib = None

PQ_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "ADMISSION_REFUSED", 4: "TIMEOUT",
                5: "DEVICE", 6: "UNSUPPORTED", 7: "NO_DEVICE", 8: "INTERNAL"}


class PqError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class CircuitDesc(ct.Structure):
    _fields_ = [("num_qubits", ct.c_int32), ("num_gates", ct.c_int32), ("op", ct.POINTER(ct.c_uint8)),
                ("q0", ct.POINTER(ct.c_int32)), ("q1", ct.POINTER(ct.c_int32)), ("phase", ct.POINTER(ct.c_uint32))]


class Stats(ct.Structure):
    _fields_ = [("free_vars", ct.c_int64), ("planes", ct.c_int64), ("lines", ct.c_int64), ("radical", ct.c_int64),
                ("terms", ct.c_int64), ("branch_dim", ct.c_int64), ("pairs", ct.c_int64),
                ("num_branches", ct.c_int64), ("branches_per_amplitude", ct.c_double),
                ("device_bytes", ct.c_int64), ("build_seconds", ct.c_double)]


class Tuning(ct.Structure):
    _fields_ = [("inner_dims", ct.c_int32), ("chunks_per_lane", ct.c_int32), ("block_warps", ct.c_int32),
                ("max_branch_dim", ct.c_int32), ("blocks_per_sm", ct.c_int32), ("unit_chunks", ct.c_int32),
                ("chunk_tables", ct.c_int32)]


class Request(ct.Structure):
    _fields_ = [("sim", ct.c_int32), ("kind", ct.c_int32), ("x", ct.c_uint64 * 2), ("y", ct.c_uint64 * 2),
                ("qubit", ct.c_int32), ("outcome", ct.c_int32), ("tag", ct.c_int64)]


class Result(ct.Structure):
    _fields_ = [("tag", ct.c_int64), ("status", ct.c_int32), ("kind", ct.c_int32), ("re", ct.c_double),
                ("im", ct.c_double), ("errbound", ct.c_double), ("submit_s", ct.c_double), ("done_s", ct.c_double),
                ("level", ct.c_int32), ("pieces", ct.c_int32)]


# name -> (restype, argtypes)
P = ct.c_void_p
u8p, i32p, u64p, f64p, i64p = (ct.POINTER(t) for t in (ct.c_uint8, ct.c_int32, ct.c_uint64, ct.c_double, ct.c_int64))
SIGNATURES = {
    "pq_version": (ct.c_char_p, []),
    "pq_last_error": (ct.c_char_p, []),
    "pq_init": (ct.c_int, [ct.c_int32]),
    "pq_set_default_tuning": (ct.c_int, [ct.POINTER(Tuning)]),
    "pq_get_default_tuning": (ct.c_int, [ct.POINTER(Tuning)]),
    "pq_sim_create": (ct.c_int, [ct.POINTER(CircuitDesc), ct.c_int32, ct.c_int32, ct.POINTER(P)]),
    "pq_analyze": (ct.c_int, [ct.POINTER(CircuitDesc), ct.c_int32, ct.c_int32, ct.POINTER(P)]),
    "pq_sim_destroy": (None, [P]),
    "pq_sim_stats": (ct.c_int, [P, ct.POINTER(Stats)]),
    "pq_amplitudes": (ct.c_int, [P, ct.c_int64, u64p, u64p, f64p, f64p]),
    "pq_probabilities": (ct.c_int, [P, ct.c_int64, u64p, u64p, f64p]),
    "pq_marginal": (ct.c_int, [P, u64p, ct.c_int32, i32p, u8p, f64p]),
    "pq_sample_many": (ct.c_int, [P, u64p, ct.c_int64, ct.c_uint64, u64p]),
    "pq_amplitude_estimate": (ct.c_int, [P, u64p, u64p, ct.c_int64, ct.c_uint64, f64p, f64p]),
    "pq_amplitude_estimate_pairs": (ct.c_int, [P, u64p, u64p, ct.c_int32, ct.c_int64, ct.c_uint64, ct.c_int32, f64p,
                                               f64p]),
    "pq_amplitudes_device": (ct.c_int, [P, ct.c_int64, P, P, P, P, P]),
    "pq_amplitudes_plain": (ct.c_int, [P, ct.c_int64, u64p, u64p, f64p]),
    "pq_amplitudes_fp64": (ct.c_int, [P, ct.c_int64, u64p, u64p, f64p]),
    "pq_amplitudes_noalloc": (ct.c_int, [P, ct.c_int64, P, P, P, P, P]),
    "pq_sim_device_check": (ct.c_int, [P, ct.c_int64, ct.POINTER(ct.c_int32)]),
    "pq_sim_set_resident": (ct.c_int, [P, ct.c_double]),
    "pq_batch_create": (ct.c_int, [ct.c_int32, ct.POINTER(P), i64p, ct.POINTER(P)]),
    "pq_batch_destroy": (None, [P]),
    "pq_batch_run": (ct.c_int, [P, u64p, u64p, f64p, f64p]),
    "pq_batch_run_device": (ct.c_int, [P, P, P, P, P, P]),
    "pq_batch_words": (ct.c_int32, [P]),
    "pq_batch_branches": (ct.c_int64, [P]),
    "pq_server_create": (ct.c_int, [ct.c_int32, ct.POINTER(P), ct.c_int32, ct.c_int64, ct.c_int32, ct.POINTER(P)]),
    "pq_server_destroy": (None, [P]),
    "pq_server_set_pieces": (ct.c_int, [P, ct.c_int32, ct.c_int32]),
    "pq_server_submit": (ct.c_int, [P, ct.c_int64, ct.POINTER(Request)]),
    "pq_server_poll": (ct.c_int64, [P, ct.POINTER(Result), ct.c_int64, ct.c_double]),
    "pq_server_now": (ct.c_double, [P]),
    "pq_server_drain": (ct.c_int, [P, ct.c_double]),
    "pq_sim_kernel_ms": (ct.c_int, [P, ct.c_int64, ct.POINTER(ct.c_float)]),
    "pq_batch_kernel_ms": (ct.c_int, [P, ct.POINTER(ct.c_float)]),
    "pq_sim_launch_items": (ct.c_int64, [P, ct.c_int64]),
    "pq_sim_enumerated": (ct.c_int, [P, ct.c_int64, f64p, f64p]),
    "pq_batch_enumerated": (ct.c_int, [P, f64p]),
    "pq_measure_peaks": (ct.c_int, [f64p]),
    "pq_measure_fma2_rate": (ct.c_int, [f64p]),
    "pq_sim_autotune": (ct.c_int, [P, ct.c_int64, u64p, u64p, ct.c_int32, ct.POINTER(Tuning), f64p]),
    "pq_sim_get_tuning": (ct.c_int, [P, ct.POINTER(Tuning)]),
    "pq_batch_autotune": (ct.c_int, [P, u64p, u64p, ct.c_int32, ct.POINTER(Tuning), f64p]),
    "pq_debug_engine_dump": (ct.c_int64, [P, ct.c_int32, u64p, ct.c_int64]),
    "pq_debug_engine_shape": (ct.c_int, [P, ct.c_int32, i64p]),
    "pq_debug_branch_phases": (ct.c_int32, [P, ct.c_int32, u64p, u64p, u8p]),
    "pq_debug_prepare": (ct.c_int, [P, ct.c_int64, u64p, u64p, u64p]),
}


def lib(build_if_missing: bool = True):
    """Load (building first if needed) the native library."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise OSError("native library not built: %s" % LIB_PATH)
                from .build import build
                build()
            L = ct.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name, None)
                if fn is None:
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status):
    if status != PQ_OK:
        raise PqError(status, lib().pq_last_error().decode())
    return status
