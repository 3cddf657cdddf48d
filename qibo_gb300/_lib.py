"""ctypes binding of ``libqgb300.so`` (declared in ``include/qgb300.h``).

The library is built in-tree (``qibo_gb300/_build.py``).  Loading fails
loudly when it is missing: the package has no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

QGB_OK, QGB_ERR_INVALID, QGB_ERR_OOM, QGB_ERR_CUDA, QGB_ERR_TIMEOUT, QGB_ERR_UNSUPPORTED = range(6)
QGB_C64, QGB_C128 = 0, 1
QGB_PLAN_BLOCKED = 1
QGB_PLAN_STRICT_FP64 = 2
QGB_PLAN_NO_TC = 8
QGB_PLAN_FUSE = 16

vp, i32, i64, u32, u64, f64, sz = C.c_void_p, C.c_int, C.c_int64, C.c_uint32, C.c_uint64, C.c_double, C.c_size_t
ip = C.POINTER(C.c_int)
dp = C.POINTER(C.c_double)
u64p = C.POINTER(C.c_uint64)


class QgbOp(C.Structure):
    """``qgb_op`` record of ``qgb_apply_circuit``."""

    _fields_ = [("k", C.c_int32), ("ncontrols", C.c_int32), ("qubits", C.c_int32 * 5),
                ("controls", C.c_int32 * 8), ("coef_offset", C.c_int64)]


class QgbBatchItem(C.Structure):
    """``qgb_batch_item`` record of ``qgb_batch_run``."""

    _fields_ = [("state", C.c_void_p), ("nqubits", C.c_int32), ("nops", C.c_int32),
                ("ops", C.POINTER(QgbOp)), ("coefs", C.POINTER(C.c_double)), ("init_zero", C.c_int32),
                ("out_kind", C.c_int32), ("nshots", C.c_int64), ("seed", C.c_uint64), ("zmask", C.c_uint64),
                ("out", C.c_void_p)]


QGB_NOT_READY = 6
QGB_PROGRAM_NO_GRAPH = 4
QGB_OUT_STATE, QGB_OUT_SAMPLES, QGB_OUT_ZEXP = 0, 1, 2
QGB_BATCH_MAX_QUBITS = {0: 13, 1: 12}
QGB_PARITY_MAX_TERMS = 256  # include/qgb300.h


# name -> (restype, argtypes)
SIGNATURES = {
    "qgb_last_error": (C.c_char_p, []),
    "qgb_version": (i32, []),
    "qgb_launch_count": (i64, []),
    "qgb_device_init": (i32, [i32, ip]),
    "qgb_mem_info": (i32, [C.POINTER(sz), C.POINTER(sz)]),
    "qgb_malloc": (i32, [C.POINTER(vp), sz]),
    "qgb_free": (i32, [vp]),
    "qgb_memcpy_h2d": (i32, [vp, vp, sz, vp]),
    "qgb_memcpy_d2h": (i32, [vp, vp, sz, vp]),
    "qgb_memcpy_d2d": (i32, [vp, vp, sz, vp]),
    "qgb_memset_zero": (i32, [vp, sz, vp]),
    "qgb_host_alloc": (i32, [C.POINTER(vp), sz]),
    "qgb_host_free": (i32, [vp]),
    "qgb_stream_sync": (i32, [vp]),
    "qgb_state_zero": (i32, [vp, i32, i32, vp]),
    "qgb_state_basis": (i32, [vp, i32, i32, i64, vp]),
    "qgb_state_cast": (i32, [vp, i32, vp, i32, i32, vp]),
    "qgb_state_scale": (i32, [vp, i32, i32, f64, vp]),
    "qgb_apply_gate": (i32, [vp, i32, i32, ip, i32, ip, i32, dp, vp]),
    "qgb_apply_1q": (i32, [vp, i32, i32, i32, dp, vp]),
    "qgb_apply_2q": (i32, [vp, i32, i32, i32, i32, dp, vp]),
    "qgb_apply_phase": (i32, [vp, i32, i32, ip, i32, f64, f64, vp]),
    "qgb_apply_swap": (i32, [vp, i32, i32, i32, i32, ip, i32, vp]),
    "qgb_apply_circuit": (i32, [vp, i32, i32, C.POINTER(QgbOp), i32, dp, i32, vp]),
    "qgb_plan_passes": (i32, [i32, i32, C.POINTER(QgbOp), i32, dp, ip]),
    "qgb_fuse_stats": (i32, [C.POINTER(QgbOp), i32, dp, i32, ip, ip]),
    "qgb_apply_fused5_tc": (i32, [vp, i32, i32, ip, dp, vp]),
    "qgb_tc_status": (i32, [ip]),
    "qgb_probs_scratch_bytes": (sz, [i32, i32]),
    "qgb_probabilities": (i32, [vp, i32, i32, ip, i32, vp, vp, vp]),
    "qgb_norm_scratch_bytes": (sz, []),
    "qgb_norm2": (i32, [vp, i32, i32, vp, vp, vp]),
    "qgb_sample_scratch_bytes": (sz, [i32]),
    "qgb_sample": (i32, [vp, i32, i64, u64, vp, vp, vp, vp]),
    "qgb_philox_fill": (i32, [vp, i64, u32, u32, u32, u32, vp]),
    "qgb_sample_noalloc": (i32, [vp, i32, i64, u64, vp, vp, vp]),
    "qgb_sample_state_scratch_bytes": (sz, [i32]),
    "qgb_sample_state": (i32, [vp, i32, i32, i64, u64, vp, vp, vp]),
    "qgb_parity_counts": (i32, [vp, i64, u64p, i32, vp, vp]),
    "qgb_collapse": (i32, [vp, i32, i32, ip, i32, vp, i32, vp, vp]),
    "qgb_expect_scratch_bytes": (sz, [i32, i32]),
    "qgb_expect_pauli": (i32, [vp, i32, i32, u64p, u64p, dp, i32, vp, vp, vp]),
    "qgb_expect_dense": (i32, [vp, i32, i32, vp, vp, vp, vp]),
    "qgb_apply_pauli_sum": (i32, [vp, vp, i32, i32, u64p, u64p, dp, i32, vp]),
    "qgb_inner_scratch_bytes": (sz, []),
    "qgb_inner": (i32, [vp, vp, i32, i32, vp, vp, vp]),
    "qgb_inner_mixed": (i32, [vp, i32, vp, i32, i32, vp, vp, vp]),
    "qgb_density_scratch_bytes": (sz, []),
    "qgb_density_probabilities": (i32, [vp, i32, i32, ip, i32, vp, vp, vp]),
    "qgb_density_collapse": (i32, [vp, i32, i32, ip, i32, vp, i32, vp, vp]),
    "qgb_density_expect_pauli": (i32, [vp, i32, i32, u64p, u64p, dp, i32, vp, vp, vp]),
    "qgb_state_axpby": (i32, [vp, vp, i32, i32, f64, f64, vp]),
    "qgb_adjoint_scratch_bytes": (sz, [i32]),
    "qgb_adjoint_sweep": (i32, [vp, vp, i32, i32, C.POINTER(QgbOp), i32, dp, ip, C.POINTER(C.c_int64), ip, i32,
                                vp, vp, vp]),
    "qgb_stream_create": (i32, [C.POINTER(vp)]),
    "qgb_stream_destroy": (i32, [vp]),
    "qgb_event_query": (i32, [vp]),
    "qgb_program_create": (i32, [i32, i32, C.POINTER(QgbOp), i32, dp, i32, C.POINTER(vp)]),
    "qgb_program_passes": (i32, [vp, ip]),
    "qgb_program_update": (i32, [vp, C.POINTER(QgbOp), i32, dp, vp]),
    "qgb_program_run": (i32, [vp, vp, vp]),
    "qgb_program_destroy": (i32, [vp]),
    "qgb_batch_create": (i32, [sz, C.POINTER(vp)]),
    "qgb_batch_run": (i32, [vp, C.c_void_p, i32, i32, vp]),
    "qgb_batch_destroy": (i32, [vp]),
    "qgb_event_create": (i32, [C.POINTER(vp)]),
    "qgb_event_destroy": (i32, [vp]),
    "qgb_event_record": (i32, [vp, vp]),
    "qgb_event_elapsed_ms": (i32, [vp, vp, C.POINTER(C.c_float)]),
}


class QgbError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"[qgb status {status}] {msg}")
        self.status = status


class DeviceOutOfMemory(MemoryError):
    """Device allocation failed (mapped to ``RuntimeError`` by
    ``execute_circuit`` as the reference does, backends/abstract.py:2500-2510)."""


class DeviceTimeout(QgbError):
    """A bounded device-side wait gave up."""


_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the shared library (once).  Raises ``ImportError`` if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise ImportError(
                    f"qibo_gb300 CUDA extension not built ({path} missing); "
                    "run `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int):
    if status == QGB_OK:
        return
    msg = _lib.qgb_last_error().decode(errors="replace") if _lib is not None else "?"
    if status == QGB_ERR_OOM:
        raise DeviceOutOfMemory(msg)
    if status == QGB_ERR_TIMEOUT:
        raise DeviceTimeout(status, msg)
    if status == QGB_ERR_INVALID:
        raise ValueError(msg)
    if status == QGB_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise QgbError(status, msg)


def int_array(values):
    values = list(values)
    return (C.c_int * max(1, len(values)))(*values)


def double_array(values):
    values = list(values)
    return (C.c_double * max(1, len(values)))(*values)
