"""Host helpers shared by the Python mirror: device checks, dtype codes,
stream handles and broadcast descriptors for the C ABI."""
from __future__ import annotations

import torch

from . import _lib

_COMPLEX = {torch.complex64: _lib.C64, torch.complex128: _lib.C128}
_REAL = {torch.float32: _lib.F32, torch.float64: _lib.F64}


def complex_code(dtype: torch.dtype) -> int:
    try:
        return _COMPLEX[dtype]
    except KeyError:
        raise NotImplementedError(
            f"the GB300 engine computes on complex64/complex128 states; got "
            f"{dtype}") from None


def real_code(dtype: torch.dtype) -> int:
    try:
        return _REAL[dtype]
    except KeyError:
        raise NotImplementedError(
            f"expected a float32/float64 tensor, got {dtype}") from None


def real_of(dtype: torch.dtype) -> torch.dtype:
    return torch.float32 if dtype == torch.complex64 else torch.float64


def require_cuda(*tensors: torch.Tensor) -> torch.device:
    """All tensors must live on one CUDA device; there is no CPU path."""
    dev = None
    for t in tensors:
        if not t.is_cuda:
            raise RuntimeError(
                "qcware_unitair_gb300 runs on CUDA tensors only (no CPU "
                f"fallback); got a tensor on {t.device}")
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise RuntimeError(
                "Expected all tensors to be on the same device, but found at "
                f"least two devices, {dev} and {t.device}!")
    return dev


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def stream_of(device: torch.device) -> int:
    """torch's current CUDA stream on ``device`` as a raw handle.  The
    direct query (a few hundred nanoseconds) matters for small states,
    where a gate's host time is the whole cost; torch.cuda.current_stream
    is the fallback."""
    if _raw_stream is not None and device.index is not None:
        return _raw_stream(device.index)
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def bcast_desc(out_shape, strides_a, strides_b) -> _lib.Bcast:
    """Descriptor over out_shape with per-operand element strides."""
    out_shape = list(out_shape)
    sa = list(strides_a)
    sb = list(strides_b)
    # drop unit dims, then merge dims that are contiguous in both operands
    dims = [(s, a, b) for s, a, b in zip(out_shape, sa, sb) if s != 1]
    merged = []
    for s, a, b in dims:
        if merged:
            ps, pa, pb = merged[-1]
            if pa == a * s and pb == b * s:
                merged[-1] = (ps * s, a, b)
                continue
        merged.append((s, a, b))
    if not merged:
        merged = [(1, 0, 0)]
    if len(merged) > _lib.MAX_DIMS:
        raise NotImplementedError(
            f"broadcast over more than {_lib.MAX_DIMS} non-mergeable dims")
    d = _lib.Bcast()
    d.ndim = len(merged)
    for i, (s, a, b) in enumerate(merged):
        d.shape[i] = s
        d.stride_a[i] = a
        d.stride_b[i] = b
    return d


def broadcast_strides(t: torch.Tensor, out_shape) -> list:
    """Element strides of contiguous t broadcast (right-aligned) to out_shape."""
    nd = len(out_shape)
    shape = [1] * (nd - t.dim()) + list(t.shape)
    strides = [0] * (nd - t.dim()) + list(t.stride())
    return [0 if s == 1 and o != 1 else st
            for s, st, o in zip(shape, strides, out_shape)]


def wide_group_bits(k: int) -> int:
    """log2 of the groups of 2^k amplitudes one tile of the complex64
    wide-operator kernel holds (k = 6..12)."""
    return 7 if k == 6 else 13 - k


def inplace_ok(dtype, k: int, n: int, per_state: bool = False) -> bool:
    """Whether gbsv_apply_operator applies a k-qubit operator in place
    (state_in == state_out) on contiguous n-qubit states; otherwise callers
    go through a temporary.  complex64 operators on 6-12 qubits are in place
    unless they are per-state and a state holds fewer groups than one tile
    of the wide-operator kernel."""
    if k <= (5 if dtype == torch.complex64 else 4):
        return True
    return (dtype == torch.complex64 and k <= 12 and
            (not per_state or n - k >= wide_group_bits(k)))
