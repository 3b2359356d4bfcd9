"""CPU oracle for the unitair hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` (to check its result) and
``bench.py`` (CPU baseline / reference arm) may import this module.  The
engine in ``qcware_unitair_gb300`` never does.

Pinning: ``tests/test_oracle.py`` checks every function here against the
golden vectors in ``tests/golden/`` that ``tests/golden/make_golden.py``
generated by running the reference (unitair 0.3.0) itself, plus the known
answers of its README and tutorial.

Restated reference behaviour (file:line in the unitair project):
  apply_operator        src/unitair/simulation/operations.py:45-148
    batch rules         operations.py:295-329 (op batch rolled to the back and
                        broadcast right-aligned; an unbatched state is
                        expanded to the op batch, :304-309)
  apply_all_qubits      operations.py:332-413
  apply_phase           operations.py:15-42   (exp(-1j*angles) * state)
  abs_squared           src/unitair/states/innerprod.py:4-26
  norm_squared          innerprod.py:29-46
  diag_expectation      innerprod.py:49-59
  inner_product         innerprod.py:62-65
  count_qubits          src/unitair/states/shapes.py:13-27
The gate arithmetic runs in C (``oracle.c``) in complex128; the complex64
variant (float arithmetic, OpenMP) is the timed CPU port.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile oracle.c with gcc (OpenMP) into _build/liboracle.so."""
    src = ORACLE_DIR / "oracle.c"
    BUILD_DIR.mkdir(exist_ok=True)
    if (not force and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime >= src.stat().st_mtime):
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(tmp),
           str(src)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        p, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        for name in ("oracle_apply_c128", "oracle_apply_c64"):
            f = getattr(L, name)
            f.argtypes = [p, p, i64, i32, i64, p, i64, p, i32]
            f.restype = i32
        L.oracle_set_threads.argtypes = [i32]
        L.oracle_get_threads.restype = i32
        L.oracle_norm_squared_c128.argtypes = [p, i64, i64, p]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(lib().oracle_get_threads())


# ----------------------------------------------------------------- shapes --
def count_qubits(length: int) -> int:
    """shapes.py:13-27: log2 of the last dim, which must be a power of 2."""
    n = round(math.log2(length)) if length > 0 else -1
    if n < 0 or 2 ** n != length:
        raise ValueError(f"state length {length} is not a power of 2")
    return n


def broadcast_operator_batch(op_batch: tuple, state_batch: tuple):
    """Output batch shape of apply_operator (operations.py:295-329).

    Returns (out_batch, state_is_expanded).  An unbatched state meets a
    batched operator by expansion (:304-309); otherwise the operator batch
    broadcasts right-aligned onto the state batch, which must not grow.
    """
    if len(op_batch) > 0 and len(state_batch) == 0:
        return tuple(op_batch), True
    extra = len(op_batch) - len(state_batch)
    if extra > 0:
        # extra leading operator dims meet qubit axes in the reference's
        # einsum; size-1 dims broadcast harmlessly, others are rejected
        if any(s != 1 for s in op_batch[:extra]):
            raise ValueError("operator has more batch dims than the state")
        op_batch = op_batch[extra:]
    out = np.broadcast_shapes(tuple(op_batch), tuple(state_batch))
    if tuple(out) != tuple(state_batch):
        raise ValueError("operator batch does not broadcast onto the state "
                         "batch")
    return tuple(state_batch), False


# --------------------------------------------------------- gate arithmetic --
def _c_apply(op: np.ndarray, qubits, state: np.ndarray, fn: str, cdt):
    n = count_qubits(state.shape[-1])
    k = count_qubits(op.shape[-1])
    qubits = [int(q) for q in qubits]
    out_batch, expanded = broadcast_operator_batch(op.shape[:-2],
                                                   state.shape[:-1])
    N = 2 ** n
    d = 2 ** k
    if op.ndim - 2 > len(out_batch):
        op = op.reshape(op.shape[op.ndim - 2 - len(out_batch):])
    ops = np.ascontiguousarray(
        np.broadcast_to(op, out_batch + (d, d)), dtype=cdt)
    if expanded:
        src = np.ascontiguousarray(state.reshape(N), dtype=cdt)
        in_stride = 0
    else:
        src = np.ascontiguousarray(state, dtype=cdt)
        in_stride = N
    B = int(np.prod(out_batch)) if len(out_batch) else 1
    out = np.empty(out_batch + (N,), dtype=cdt)
    q = (ctypes.c_int * max(k, 1))(*qubits)
    rc = getattr(lib(), fn)(src.ctypes.data, out.ctypes.data, B, n,
                            in_stride, ops.ctypes.data, d * d, q, k)
    if rc != 0:
        raise ValueError(f"{fn} rejected n={n} qubits={qubits}")
    return out


def apply_operator(op, qubits, state):
    """complex128 result of apply_operator (operations.py:45-148)."""
    return _c_apply(np.asarray(op), qubits, np.asarray(state),
                    "oracle_apply_c128", np.complex128)


def apply_operator_c64(op, qubits, state):
    """complex64 port: float arithmetic, multi-threaded (timed baseline)."""
    return _c_apply(np.asarray(op), qubits, np.asarray(state),
                    "oracle_apply_c64", np.complex64)


def apply_operator_numpy(op, qubits, state):
    """Independent numpy restatement of operations.py:151-186 / :322.

    Moves the target qubit axes to the front of the tensor layout, contracts
    with einsum exactly as act_first_qubits_tensor does, and moves them
    back.  Used on small cases to cross-check the C oracle.
    """
    op = np.asarray(op, dtype=np.complex128)
    state = np.asarray(state, dtype=np.complex128)
    n = count_qubits(state.shape[-1])
    k = count_qubits(op.shape[-1])
    out_batch, expanded = broadcast_operator_batch(op.shape[:-2],
                                                   state.shape[:-1])
    if expanded:
        state = np.broadcast_to(state, out_batch + state.shape)
    if op.ndim - 2 > len(out_batch):
        op = op.reshape(op.shape[op.ndim - 2 - len(out_batch):])
    nb = len(out_batch)
    t = state.reshape(out_batch + (2,) * n)
    qaxes = [nb + q for q in qubits]
    t = np.moveaxis(t, qaxes, list(range(nb, nb + k)))
    shp = t.shape
    t = t.reshape(out_batch + (2 ** k, 2 ** (n - k)))
    opb = np.broadcast_to(op, out_batch + op.shape[-2:])
    r = np.einsum("...ab,...bc->...ac", opb, t)
    r = r.reshape(shp)
    r = np.moveaxis(r, list(range(nb, nb + k)), qaxes)
    return np.ascontiguousarray(r.reshape(out_batch + (2 ** n,)))


def apply_all_qubits(op, state):
    """operations.py:332-413: the same 2x2 operator on every qubit.

    Single-qubit operators on distinct qubits commute, so applying them in
    qubit order 0..n-1 gives the reference's result up to rounding.
    """
    op = np.asarray(op)
    n = count_qubits(np.asarray(state).shape[-1])
    out = np.asarray(state)
    for q in range(n):
        out = apply_operator(op, [q], out)
    return out


def apply_all_qubits_each(ops, state):
    """Extension: ops[..., q, :, :] acts on qubit q."""
    ops = np.asarray(ops)
    n = count_qubits(np.asarray(state).shape[-1])
    out = np.asarray(state)
    for q in range(n):
        out = apply_operator(ops[..., q, :, :], [q], out)
    return out


def apply_phase(angles, state):
    """operations.py:41-42: exp(-1j * angles) * state, numpy broadcasting.

    torch forms the factor in complex(angles.dtype) -- complex64 for float32
    angles even when the state is complex128 -- so the factor is rounded to
    that precision before the (complex128) product.
    """
    angles = np.asarray(angles)
    state = np.asarray(state)
    fdt = np.complex64 if angles.dtype == np.float32 else np.complex128
    factor = np.exp(-1j * angles.astype(np.float64)).astype(fdt)
    return factor.astype(np.complex128) * state.astype(np.complex128)


# ---------------------------------------------------------------- reductions
def abs_squared(state):
    s = np.asarray(state, dtype=np.complex128)
    return (s.conj() * s).real


def norm_squared(state):
    return abs_squared(state).sum(axis=-1)


def diag_expectation_value(diag, state):
    return (abs_squared(state) * np.asarray(diag, dtype=np.float64)).sum(
        axis=-1)


def inner_product(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return (a.conj() * b).sum(axis=-1)


# ------------------------------------------------------------------ circuits
def run_circuit(gates, state, c64: bool = False):
    """Apply a gate list in order.

    ``gates`` is a sequence of (matrix, qubits) with matrix (*b, d, d).
    complex128 arithmetic unless c64 (the timed float port).
    """
    out = np.asarray(state)
    f = apply_operator_c64 if c64 else apply_operator
    for mat, qubits in gates:
        out = f(mat, qubits, out)
    return out
