"""ctypes binding of libgbsv.so, the C ABI declared in include/gbsv.h.

The library is loaded from the in-tree build directory.  If it is missing
the engine raises: there is no CPU or pure-torch fallback for any kernel.
"""
from __future__ import annotations

import ctypes
import threading

from . import build_lib

GBSV_OK = 0
GBSV_ERR_INVALID_ARG = 1
GBSV_ERR_UNSUPPORTED = 2
GBSV_ERR_CUDA = 3
GBSV_ERR_SCRATCH = 4
GBSV_ERR_TIMEOUT = 5

C64, C128, F32, F64 = 0, 1, 2, 3
MAX_DIMS = 8
MAX_DENSE_QUBITS = 12


class GbsvError(RuntimeError):
    """A libgbsv entry point returned a non-zero status."""

    def __init__(self, status: int, what: str, detail: str):
        self.status = status
        super().__init__(f"{what}: {detail} (status {status})")


class Bcast(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("shape", ctypes.c_int64 * MAX_DIMS),
        ("stride_a", ctypes.c_int64 * MAX_DIMS),
        ("stride_b", ctypes.c_int64 * MAX_DIMS),
    ]


class PlanOp(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("contiguous", ctypes.c_int32),
                ("first", ctypes.c_int32), ("count", ctypes.c_int32),
                ("positions", ctypes.c_int32 * 16)]


class Plan(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("used_layouts", ctypes.c_int32),
                ("ops", ctypes.c_void_p), ("max_ops", ctypes.c_int32),
                ("num_ops", ctypes.c_int32),
                ("records", ctypes.c_void_p), ("max_records", ctypes.c_int32),
                ("num_records", ctypes.c_int32),
                ("layouts", ctypes.c_void_p), ("max_layouts", ctypes.c_int32),
                ("num_layouts", ctypes.c_int32),
                ("pool", ctypes.c_void_p), ("max_pool", ctypes.c_int64),
                ("pool_len", ctypes.c_int64)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_SZ = ctypes.c_size_t
_BC = ctypes.POINTER(Bcast)

class MultiStage(ctypes.Structure):
    """gbsv_multi_stage_t"""
    _fields_ = [("state_in", ctypes.c_void_p), ("state_out", ctypes.c_void_p),
                ("gates", ctypes.c_void_p), ("layouts", ctypes.c_void_p),
                ("pool", ctypes.c_void_p), ("num_states", ctypes.c_int64),
                ("in_stride", ctypes.c_int64),
                ("num_layouts", ctypes.c_int32),
                ("contiguous_qubits", ctypes.c_int32),
                ("tile_positions", ctypes.c_int32 * 16)]


# name -> (restype, argtypes); must match include/gbsv.h exactly.
SIGNATURES = {
    "gbsv_abi_version": (_I, []),
    "gbsv_status_string": (ctypes.c_char_p, [_I]),
    "gbsv_last_error": (ctypes.c_char_p, []),
    "gbsv_launch_count": (ctypes.c_uint64, []),
    "gbsv_set_c128_arith": (_I, [_I]),
    "gbsv_get_c128_arith": (_I, []),
    "gbsv_apply_operator": (_I, [_P, _P, _I, _I, _I64, _I64, _P, _I64,
                                 ctypes.POINTER(_I32), _I, _P]),
    "gbsv_apply_all_qubits": (_I, [_P, _P, _I, _I, _I64, _I64, _P, _I64,
                                   _I64, _P]),
    "gbsv_apply_phase": (_I, [_P, _I, _P, _I, _P, _I, _BC, _P]),
    "gbsv_fused_max_tile_qubits": (_I, [_I]),
    "gbsv_run_stage": (_I, [_P, _P, _I, _I, _I64, _I64, _I, _I,
                            ctypes.POINTER(_I32), _P, _I, _P, _P]),
    "gbsv_fused_register_bits": (_I, [_I]),
    "gbsv_run_stage_layouts": (_I, [_P, _P, _I, _I, _I64, _I64, _I, _I,
                                    ctypes.POINTER(_I32), _P, _P, _I, _P,
                                    _P]),
    "gbsv_run_programs": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "gbsv_run_stages_multi": (_I, [_I, _I, _I, _P, _I, _P]),
    "gbsv_run_stage_tc": (_I, [_P, _P, _I, _I, _I64, _I64, _I, _I,
                               ctypes.POINTER(_I32), _P, _I, _P, _P, _P,
                               _P]),
    "gbsv_tc_status": (_I, [ctypes.POINTER(_I), _I]),
    "gbsv_plan": (_I, [_P, _I, _P, _I, _I, _I, _I, _I,
                       ctypes.POINTER(Plan)]),
    "gbsv_operator_grad_scratch_bytes": (_SZ, [_I64, _I, _I, _I]),
    "gbsv_operator_grad": (_I, [_P, _P, _I, _I, _I64, _I64,
                                ctypes.POINTER(_I32), _I, _P, _I, _P, _SZ,
                                _P]),
    "gbsv_pauli_sum_apply": (_I, [_P, _P, _I, _I, _I64, _P, _I, _P]),
    "gbsv_adjoint_scratch_bytes": (_SZ, [_I64, _I]),
    "gbsv_adjoint_rotation_step": (_I, [_P, _P, _I, _I, _I64, _I, _I, _P, _I,
                                        _I64, ctypes.c_double, _P, _I64,
                                        ctypes.c_double, _P, _SZ, _P]),
    "gbsv_permute_qubits": (_I, [_P, _P, _I, _I, _I64,
                                 ctypes.POINTER(_I32), _P]),
    "gbsv_phase_flip": (_I, [_P, _P, _I, _I, _I64, _P, _I, _P]),
    "gbsv_multi_controlled_x": (_I, [_P, _P, _I, _I, _I64,
                                     ctypes.POINTER(_I32), _I, _I, _P]),
    "gbsv_sample_scratch_bytes": (_SZ, [_I64]),
    "gbsv_sample": (_I, [_P, _I, _I64, _I64, ctypes.c_uint64, _P, _P, _SZ,
                         _P]),
    "gbsv_adjoint_stage": (_I, [_P, _P, _I, _I, _I64, _I, _I,
                                ctypes.POINTER(_I32), _P, _I, _P, _P, _I,
                                _I64, _I, _P, _P, _P, _P, _SZ, _P]),
    "gbsv_reduce_scratch_bytes": (_SZ, [_I64, _I64]),
    "gbsv_norm_squared": (_I, [_P, _I, _I64, _I64, _P, _I, _P, _SZ, _P]),
    "gbsv_norm_squared_noalloc": (_I, [_P, _I, _I64, _I64, _P, _I, _P]),
    "gbsv_renormalize": (_I, [_P, _I, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "gbsv_abs_squared": (_I, [_P, _I, _I64, _P, _P]),
    "gbsv_inner_product": (_I, [_P, _P, _I, _BC, _I64, _I64, _I64, _P, _I,
                                _P, _SZ, _P]),
    "gbsv_diag_expectation": (_I, [_P, _I, _P, _I, _BC, _I64, _I64, _I64,
                                   _P, _I, _P, _SZ, _P]),
}

_lock = threading.Lock()
_lib = None


def load(path=None):
    """Load (once) and return the ctypes handle of libgbsv.so."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or build_lib.lib_path()
        if not p.exists():
            raise RuntimeError(
                f"libgbsv.so is not built ({p}); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` or "
                "`python -m qcware_unitair_gb300.build_lib`.  The engine has "
                "no CPU fallback.")
        L = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if path is None:
            _lib = L
        return L


def check(status: int, what: str) -> None:
    if status != GBSV_OK:
        L = load()
        detail = L.gbsv_last_error().decode(errors="replace")
        kind = L.gbsv_status_string(status).decode()
        raise GbsvError(status, what, f"{kind}: {detail}")


def launch_count() -> int:
    return int(load().gbsv_launch_count())


C128_ARITH = {"pairs": 0, "fp64": 1}


def set_complex128_arithmetic(mode: str) -> str:
    """Select the complex128 gate arithmetic for this process: "pairs"
    (double-float pairs on the FP32 pipe, about 47 bits, the default) or
    "fp64" (native FP64).  Returns the previous mode."""
    if mode not in C128_ARITH:
        raise ValueError(f"complex128 arithmetic must be one of "
                         f"{sorted(C128_ARITH)}, not {mode!r}")
    prev = complex128_arithmetic()
    check(load().gbsv_set_c128_arith(C128_ARITH[mode]), "set_c128_arith")
    return prev


def complex128_arithmetic() -> str:
    code = int(load().gbsv_get_c128_arith())
    return {v: k for k, v in C128_ARITH.items()}[code]


def qubit_array(qubits):
    arr = (_I32 * max(len(qubits), 1))(*[int(q) for q in qubits])
    return arr
