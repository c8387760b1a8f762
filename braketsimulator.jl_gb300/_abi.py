"""ctypes binding of libbraket_gb300.so (the C ABI declared in include/braket_gb300.h).

The library is built in-tree by ``build.build_library()``.  Loading fails loudly
when it is missing: there is no CPU path behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

BS_OK = 0
BS_KIND_SV, BS_KIND_DM = 0, 1
BS_PREC_C128, BS_PREC_C64 = 0, 1
BS_GATE_DIAGONAL = 0x01
BS_GATE_CONJ = 0x02
BS_GATE_SORTED_TARGETS = 0x04
BS_GATE_MSB_FIRST = 0x08
BS_NOISE_REFERENCE = 0x00
BS_NOISE_PHYSICAL = 0x10
BS_ALIAS_EXACT, BS_ALIAS_PARALLEL = 0x0, 0x1
BS_TUNE_TILE_BITS, BS_TUNE_TILE_THREADS, BS_TUNE_TC, BS_TUNE_TC_MIN_BITS, BS_TUNE_TC_COST = 0, 1, 2, 3, 4
BS_TUNE_ADJ_SEGMENTS = 5
BS_FILE_STATE, BS_FILE_PROBABILITIES = 0, 1
BS_ERR_TIMEOUT = 6
BS_ERR_IO = 7
BS_MAX_TARGETS = 10
BS_MAX_CONTROLS = 16

LIB_NAME = "libbraket_gb300.so"
LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build")
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

# every exported entry point and its (restype, argtypes)
_p = C.c_void_p
_i32, _u32, _i64, _u64, _f64 = C.c_int, C.c_uint, C.c_int64, C.c_uint64, C.c_double
_P = C.POINTER


class BsOp(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("flags", C.c_uint32),
        ("n_targets", C.c_int32),
        ("n_controls", C.c_int32),
        ("targets", C.c_int32 * BS_MAX_TARGETS),
        ("controls", C.c_int32 * BS_MAX_CONTROLS),
        ("control_values", C.c_int32 * BS_MAX_CONTROLS),
        ("n_matrices", C.c_int32),
        ("reserved", C.c_int32),
        ("matrix", _P(C.c_double)),
    ]


class BsStats(C.Structure):
    _fields_ = [
        ("sweeps", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("gates", C.c_int64),
        ("bytes_moved", C.c_double),
        ("gpu_ms", C.c_double),
        ("tc_gates", C.c_int64),
        ("tc_launches", C.c_int64),
        ("tc_ms", C.c_double),
    ]


SIGNATURES = {
    "bs_create": (_i32, [_i32, _i32, _i32, _P(_p)]),
    "bs_destroy": (_i32, [_p]),
    "bs_reinit": (_i32, [_p, _i32]),
    "bs_qubit_count": (_i32, [_p, _P(_i32)]),
    "bs_last_error": (C.c_char_p, [_p]),
    "bs_version": (C.c_char_p, []),
    "bs_set_state": (_i32, [_p, _P(_f64), _i64]),
    "bs_get_state": (_i32, [_p, _P(_f64), _i64]),
    "bs_set_state_device": (_i32, [_p, _p, _i64]),
    "bs_get_state_device": (_i32, [_p, _p, _i64]),
    "bs_copy_state": (_i32, [_p, _p]),
    "bs_apply_gate": (_i32, [_p, _P(_f64), _i32, _P(_i32), _i32, _P(_i32), _P(_i32), _u32]),
    "bs_dm_apply_vec_gate": (_i32, [_p, _P(_f64), _i32, _P(_i32), _i32, _P(_i32), _P(_i32), _u32]),
    "bs_apply_kraus": (_i32, [_p, _P(_f64), _i32, _i32, _P(_i32), _u32]),
    "bs_evolve": (_i32, [_p, _P(BsOp), _i64, _u32]),
    # the output buffers as plain addresses (numpy's .ctypes.data): a typed-pointer conversion costs
    # more than the rest of a small run's Python side
    "bs_run_small": (_i32, [_p, _P(BsOp), _i64, _i64, _u64, _p, _p]),
    "bs_last_stats": (_i32, [_p, _P(BsStats)]),
    "bs_probabilities": (_i32, [_p, _P(_f64), _i64]),
    "bs_marginal_probabilities": (_i32, [_p, _i32, _P(_i32), _P(_f64)]),
    "bs_expectation_pauli": (_i32, [_p, _i32, _P(_u64), _P(_u64), _P(_f64), _P(_f64)]),
    "bs_expectation_matrix": (_i32, [_p, _P(_f64), _i32, _P(_i32), _u32, _P(_f64)]),
    "bs_alias_build": (_i32, [_p, _f64, _u32]),
    "bs_alias_build_from": (_i32, [_p, _P(_f64), _i64, _f64]),
    "bs_alias_table": (_i32, [_p, _P(_f64), _P(_i64), _i64]),
    "bs_sample_alias": (_i32, [_p, _P(_i64), _P(_f64), _i64, _P(_i64)]),
    "bs_sample_direct": (_i32, [_p, _P(_f64), _i64, _f64, _P(_i64)]),
    "bs_sample": (_i32, [_p, _u64, _i64, _P(_i64)]),
    "bs_adjoint_gradient": (_i32, [_p, _P(BsOp), _i64, _P(C.c_int32), _P(C.c_int32), _P(_u64), _P(_u64),
                                   _i32, _i32, _P(_u64), _P(_u64), _P(_f64), _P(_f64), _P(_f64)]),
    "bs_expectation_pauli_noalloc": (_i32, [_p, _i32, _i32, _i32, _P(_u64), _P(_u64), _P(_f64), _P(_f64), _p]),
    "bs_run_batch": (_i32, [_i32, _P(_i32), _P(_P(BsOp)), _P(_i64), _i32, _P(_u64), _P(_u64), _i64, _u64, _i32,
                            _P(_f64), _P(_i64), _P(BsStats)]),
    "bs_batch_create": (_i32, [_i32, _P(_i32), _P(_P(BsOp)), _P(_i64), _i32, _P(_u64), _P(_u64), _i64, _u64, _i32,
                               _P(_p)]),
    "bs_batch_set_ops": (_i32, [_p, _P(_P(BsOp)), _P(_i64)]),
    "bs_batch_launch": (_i32, [_p, _P(_f64), _P(_i64), _P(BsStats)]),
    "bs_batch_destroy": (_i32, [_p]),
    "bs_batch_set_tuning": (_i32, [_p, _i32, _P(_i32), _P(_f64)]),
    "bs_set_tuning": (_i32, [_p, _i32, _f64]),
    "bs_get_tuning": (_i32, [_p, _i32, _P(_f64)]),
    "bs_reduced_density_matrix": (_i32, [_p, _i32, _P(_i32), _P(_f64)]),
    "bs_write_result_file": (_i32, [_p, _i32, C.c_char_p, _P(_i64)]),
    "bs_synchronize": (_i32, [_p]),
    "bs_selftest_wait_timeout": (_i32, [_p, _f64]),
    "bs_state_device_ptr": (_i32, [_p, _P(_p)]),
}

_lib = None


class BraketGB300Error(RuntimeError):
    """Raised when an engine call returns a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[bs status {code}] {msg}")
        self.code = code


def lib(path: str | None = None):
    """Load the engine library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or os.environ.get("BRAKET_GB300_LIB", LIB_PATH)
    if not os.path.exists(p):
        raise ImportError(f"{LIB_NAME} not found at {p}; run __graft_entry__.build() (needs nvcc)")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(handle, rc: int):
    if rc != BS_OK:
        msg = lib().bs_last_error(handle)
        raise BraketGB300Error(rc, msg.decode() if msg else "unknown error")


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_int32))


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_int64))


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_uint64))


def cplx_buffer(m: np.ndarray) -> np.ndarray:
    """Row-major interleaved complex128 buffer the engine reads."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).view(np.float64).ravel()
