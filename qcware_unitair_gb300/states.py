"""Mirror of ``unitair.states``: layout and shape helpers plus the batched
reductions, which run as FP64-accumulating CUDA kernels.

Shape helpers follow src/unitair/states/shapes.py and conversions.py (same
names, arguments and exceptions).  Reductions replace
src/unitair/states/innerprod.py:4-65; they return the same dtypes as
unitair (e.g. float32 norms for complex64 states) but accumulate in double.
"""
from __future__ import annotations

import enum
import math
from typing import List, Tuple, Union

import torch

from . import _core, _lib


class StateLayout(str, enum.Enum):
    VECTOR = "vector"
    TENSOR = "tensor"


class StateShapeError(ValueError):
    """Raised for a state whose shape fits no number of qubits
    (unitair: src/unitair/states/shapes.py:149-182)."""

    def __init__(self, data: torch.Tensor = None,
                 expected_layout: StateLayout = None):
        self.data_size = tuple(data.size()) if data is not None else None
        if expected_layout is not None:
            expected_layout = StateLayout(expected_layout.lower())
        self.layout = expected_layout

    def __str__(self):
        msg = "There is a problem with the shape of a state.\n"
        if self.layout is StateLayout.VECTOR:
            msg += ("Expected VECTOR layout. This means that states are "
                    "specified by a tensor with size "
                    "(*optional_batch_dims, 2^num_qubits)\n")
        if self.layout is StateLayout.TENSOR:
            msg += ("Expected TENSOR layout. This means that states are "
                    "specified by a tensor with size\n"
                    "    (*optional_batch_dims, 2, 2, ..., 2)\n"
                    "where the number of 2's is the number of qubits.\n")
        if self.data_size is not None:
            msg += f"Given state has size {self.data_size}"
        return msg


def _log2_exact(length: int):
    n = round(math.log2(length))
    return n if 2 ** n == length else None


def count_qubits(state: torch.Tensor) -> int:
    """Number of qubits of a vector-layout state (shapes.py:13-27)."""
    length = state.size()[-1]
    n = _log2_exact(length)
    if n is None:
        raise StateShapeError(data=state, expected_layout=StateLayout.VECTOR)
    return n


def count_qubits_gate_matrix(gate: torch.Tensor) -> int:
    """k for a (*batch, 2^k, 2^k) operator (shapes.py:31-47)."""
    length = gate.size()[-1]
    n = _log2_exact(length)
    if n is None:
        raise RuntimeError(f"Given gate matrix has size {gate.size()} which "
                           "is not consistent with any number of qubits.")
    return n


def hilbert_space_dim(state: torch.Tensor) -> int:
    return 2 ** count_qubits(state)


def count_qubits_tensor(state_tensor: torch.Tensor, num_batch_dims: int):
    return state_tensor.dim() - num_batch_dims


def count_batch_dims_tensor(state_tensor: torch.Tensor, num_qubits: int):
    return state_tensor.dim() - num_qubits


def get_qubit_indices(index: Union[int, List[int], Tuple[int, ...],
                                   torch.Tensor],
                      state_tensor: torch.Tensor, num_qubits: int):
    """Qubit index -> torch dim of a tensor-layout state (shapes.py:72-116);
    negative indices are kept as they are."""
    batch_dims = state_tensor.dim() - num_qubits
    msg = ("Expected index in {-num_qubits, ..., num_qubits - 1}.\n"
           f"Num_qubits: {num_qubits}, index: {index}.")
    as_list = not isinstance(index, torch.Tensor)
    idx = torch.tensor(index) if as_list else index
    if (idx >= num_qubits).any() or (idx < -num_qubits).any():
        raise ValueError(msg)
    idx = idx + (idx >= 0) * batch_dims
    return idx.tolist() if as_list else idx


def subset_roll_to_back(tensor: torch.Tensor, subset_num_dims):
    order = list(range(subset_num_dims, tensor.dim())) + list(
        range(subset_num_dims))
    return torch.permute(tensor, order)


def subset_roll_to_front(tensor: torch.Tensor, subset_num_dims):
    start = tensor.dim() - subset_num_dims
    order = list(range(start, tensor.dim())) + list(range(start))
    return torch.permute(tensor, order)


def to_tensor_layout(state: torch.Tensor) -> torch.Tensor:
    """(*b, 2^n) -> (*b, 2, ..., 2) view (conversions.py:5-45)."""
    n = count_qubits(state)
    if not state.is_contiguous():
        state = state.contiguous()
    return state.view(state.size()[:-1] + torch.Size(n * [2]))


def to_vector_layout(state_tensor: torch.Tensor,
                     num_qubits: int) -> torch.Tensor:
    """(*b, 2, ..., 2) -> (*b, 2^n) (conversions.py:48-92)."""
    if not state_tensor.is_contiguous():
        state_tensor = state_tensor.contiguous()
    batch = state_tensor.size()[:-num_qubits] if num_qubits else \
        state_tensor.size()
    return state_tensor.view(batch + torch.Size((2 ** num_qubits,)))


# ------------------------------------------------------------- reductions --
def _scratch(rows: int, dim: int, device) -> tuple:
    nbytes = int(_lib.load().gbsv_reduce_scratch_bytes(rows, dim))
    if nbytes == 0:
        return None, 0
    buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
    return buf, nbytes


def _norm_squared_kernel(state: torch.Tensor, out_dtype=None) -> torch.Tensor:
    dev = _core.require_cuda(state)
    code = _core.complex_code(state.dtype)
    s = state.contiguous()
    rows = s.numel() // s.shape[-1] if s.shape[-1] else 0
    real = _core.real_of(state.dtype) if out_dtype is None else out_dtype
    out = torch.empty(s.shape[:-1], dtype=real, device=dev)
    if rows == 0:
        return out
    if s.shape[-1] == 0:
        return out.zero_()
    buf, nbytes = _scratch(rows, s.shape[-1], dev)
    rc = _lib.load().gbsv_norm_squared(
        s.data_ptr(), code, rows, s.shape[-1], out.data_ptr(),
        _core.real_code(real), buf.data_ptr() if buf is not None else None,
        nbytes, _core.stream_of(dev))
    _lib.check(rc, "norm_squared")
    return out


def _abs_squared_kernel(state: torch.Tensor) -> torch.Tensor:
    dev = _core.require_cuda(state)
    code = _core.complex_code(state.dtype)
    s = state.contiguous()
    out = torch.empty(s.shape, dtype=_core.real_of(state.dtype), device=dev)
    if s.numel() == 0:
        return out
    rc = _lib.load().gbsv_abs_squared(s.data_ptr(), code, s.numel(),
                                      out.data_ptr(), _core.stream_of(dev))
    _lib.check(rc, "abs_squared")
    return out


def _row_broadcast(a: torch.Tensor, b: torch.Tensor):
    """Broadcast two (*batch, dim) tensors over all dims; return the output
    row shape, the descriptor over rows and the inner length/strides."""
    out_shape = torch.broadcast_shapes(a.shape, b.shape)
    sa = _core.broadcast_strides(a, out_shape)
    sb = _core.broadcast_strides(b, out_shape)
    dim = out_shape[-1] if len(out_shape) else 1
    ia = sa[-1] if len(out_shape) else 0
    ib = sb[-1] if len(out_shape) else 0
    desc = _core.bcast_desc(out_shape[:-1], sa[:-1], sb[:-1])
    return tuple(out_shape[:-1]), desc, dim, ia, ib


def _inner_product_kernel(a: torch.Tensor, b: torch.Tensor,
                          out_dtype=None) -> torch.Tensor:
    dev = _core.require_cuda(a, b)
    if a.dtype != b.dtype:
        raise RuntimeError(
            f"expected both states to have one dtype, got {a.dtype} and "
            f"{b.dtype}")
    code = _core.complex_code(a.dtype)
    a = a.contiguous()
    b = b.contiguous()
    rows_shape, desc, dim, ia, ib = _row_broadcast(a, b)
    out_dtype = a.dtype if out_dtype is None else out_dtype
    out = torch.empty(rows_shape, dtype=out_dtype, device=dev)
    rows = out.numel()
    if rows == 0:
        return out
    buf, nbytes = _scratch(rows, dim, dev)
    rc = _lib.load().gbsv_inner_product(
        a.data_ptr(), b.data_ptr(), code, desc, dim, ia, ib, out.data_ptr(),
        _core.complex_code(out_dtype),
        buf.data_ptr() if buf is not None else None, nbytes,
        _core.stream_of(dev))
    _lib.check(rc, "inner_product")
    return out


def _diag_expectation_kernel(diag: torch.Tensor,
                             state: torch.Tensor) -> torch.Tensor:
    dev = _core.require_cuda(diag, state)
    scode = _core.complex_code(state.dtype)
    if diag.is_complex():
        raise NotImplementedError("complex diagonals are not supported; "
                                  "pass the real diagonal")
    dcode = _core.real_code(diag.dtype)
    out_dtype = torch.promote_types(_core.real_of(state.dtype), diag.dtype)
    d = diag.contiguous()
    s = state.contiguous()
    rows_shape, desc, dim, ia, ib = _row_broadcast(d, s)
    out = torch.empty(rows_shape, dtype=out_dtype, device=dev)
    rows = out.numel()
    if rows == 0:
        return out
    buf, nbytes = _scratch(rows, dim, dev)
    rc = _lib.load().gbsv_diag_expectation(
        d.data_ptr(), dcode, s.data_ptr(), scode, desc, dim, ia, ib,
        out.data_ptr(), _core.real_code(out_dtype),
        buf.data_ptr() if buf is not None else None, nbytes,
        _core.stream_of(dev))
    _lib.check(rc, "diag_expectation_value")
    return out


class _NormSquared(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state):
        ctx.save_for_backward(state)
        return _norm_squared_kernel(state)

    @staticmethod
    def backward(ctx, g):
        (state,) = ctx.saved_tensors
        return 2 * g.unsqueeze(-1) * state


class _AbsSquared(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state):
        ctx.save_for_backward(state)
        return _abs_squared_kernel(state)

    @staticmethod
    def backward(ctx, g):
        (state,) = ctx.saved_tensors
        return 2 * g * state


class _InnerProduct(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b):
        ctx.save_for_backward(a, b)
        return _inner_product_kernel(a, b)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        g = g.unsqueeze(-1)
        ga = gb = None
        if ctx.needs_input_grad[0]:
            ga = (g.conj() * b).sum_to_size(a.shape)
        if ctx.needs_input_grad[1]:
            gb = (g * a).sum_to_size(b.shape)
        return ga, gb


class _DiagExpectation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, diag, state):
        ctx.save_for_backward(diag, state)
        return _diag_expectation_kernel(diag, state)

    @staticmethod
    def backward(ctx, g):
        diag, state = ctx.saved_tensors
        g = g.unsqueeze(-1)
        gd = gs = None
        if ctx.needs_input_grad[0]:
            p = (state.conj() * state).real
            gd = (g * p).to(diag.dtype).sum_to_size(diag.shape)
        if ctx.needs_input_grad[1]:
            gs = (2 * g * diag * state).to(state.dtype).sum_to_size(
                state.shape)
        return gd, gs


def abs_squared(state: torch.Tensor) -> torch.Tensor:
    """|x_k|^2 for every amplitude (innerprod.py:4-26)."""
    return _AbsSquared.apply(state)


def norm_squared(state: torch.Tensor) -> torch.Tensor:
    """<state|state> per batch entry (innerprod.py:29-46)."""
    return _NormSquared.apply(state)


def diag_expectation_value(diag_values: torch.Tensor,
                           state: torch.Tensor) -> torch.Tensor:
    """sum_k d_k |x_k|^2 with broadcasting (innerprod.py:49-59)."""
    return _DiagExpectation.apply(diag_values, state)


def inner_product(state_1: torch.Tensor, state_2: torch.Tensor):
    """<state_1|state_2>, conjugate-linear in the left entry
    (innerprod.py:62-65)."""
    return _InnerProduct.apply(state_1, state_2)


def norm_squared_fp64(state: torch.Tensor) -> torch.Tensor:
    """norm_squared returned in float64 (the FP64 accumulator, unrounded)."""
    return _norm_squared_kernel(state, out_dtype=torch.float64)
