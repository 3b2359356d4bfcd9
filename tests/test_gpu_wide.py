"""Operators on 6-12 qubits against the complex128 oracle (unitair's
apply_operator, operations.py:45-148).

complex64 runs the tile kernel (dense_wide_kernel: a CTA holds 2^(13-k)
groups of 2^k amplitudes in shared memory and streams the operator through
it in column chunks); complex128, and per-state complex64 operators on
states smaller than one tile, run the one-output-per-thread kernel.
Covered: shared and per-state operators, tiles that span states or end
early, target 0 among the targets (scalar stores) or not (paired stores),
strided and broadcast inputs, in place, and the bit-identity of the two
kernels (the tile kernel keeps the other's order of fused multiply-adds).

Tolerance: max abs error over the largest output magnitude, 2e-6 for
complex64 (times sqrt(2^k / 64): FP32 sums of 2^k products) and 1e-13 for
complex128.
"""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300 import _core, _lib

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
C64, C128 = torch.complex64, torch.complex128


def _tol(dtype, k):
    if dtype == C64:
        return 2e-6 * max(1.0, (2 ** k / 64) ** 0.5)
    return 1e-13


def _rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _err(got, ref):
    if isinstance(got, torch.Tensor):
        got = got.cpu().numpy()
    return float(np.abs(got - ref).max() / np.abs(ref).max())


@pytest.mark.parametrize("extra", [0, 2])
@pytest.mark.parametrize("k", range(6, 13))
def test_wide_shared_operator(oracle, k, extra):
    """One operator for all states on n = k (one group per state: tiles
    span states and the last tile ends early) and n = k + 2 qubits."""
    rng = np.random.default_rng(100 * k + extra)
    n, B = k + extra, 3
    psi = _rand(rng, (B, 2 ** n))
    op = _rand(rng, (2 ** k, 2 ** k)) / 2 ** (k / 2)
    placements = [[int(q) for q in rng.permutation(n)[:k]]]
    if n > k:  # qubit n-1 (bit 0) left out: paired stores
        placements.append([int(q) for q in rng.permutation(n - 1)[:k]])
    for qubits in placements:
        ref = oracle.apply_operator(op, qubits, psi)
        for dtype in (C64, C128):
            opd = torch.from_numpy(op).to(DEV, dtype)
            st = torch.from_numpy(psi).to(DEV, dtype)
            assert _err(ug.apply_operator(opd, qubits, st), ref) <= _tol(
                dtype, k), (dtype, qubits)
            ug.apply_operator_(opd, qubits, st)
            assert _err(st, ref) <= _tol(dtype, k), (dtype, qubits, "in place")


@pytest.mark.parametrize("k", [6, 8, 12])
def test_wide_per_state_operators(oracle, k):
    """One operator per state: the tile kernel when a state holds a whole
    tile of groups, else the one-output-per-thread kernel (through a
    temporary when in place)."""
    rng = np.random.default_rng(7 + k)
    for n in (k + 1, k + _core.wide_group_bits(k)):
        B = 2
        psi = _rand(rng, (B, 2 ** n))
        op = _rand(rng, (B, 2 ** k, 2 ** k)) / 2 ** (k / 2)
        qubits = [int(q) for q in rng.permutation(n)[:k]]
        ref = oracle.apply_operator(op, qubits, psi)
        opd = torch.from_numpy(op).to(DEV, C64)
        st = torch.from_numpy(psi).to(DEV, C64)
        assert _err(ug.apply_operator(opd, qubits, st), ref) <= _tol(C64, k)
        assert _core.inplace_ok(C64, k, n, True) == (
            n - k >= _core.wide_group_bits(k))
        ug.apply_operator_(opd, qubits, st)
        assert _err(st, ref) <= _tol(C64, k), (n, "in place")


@pytest.mark.parametrize("k", [6, 9])
def test_wide_kernel_bits_match_generic(k):
    """The same operator given once (tile kernel) and repeated per state on
    states smaller than a tile (one-output-per-thread kernel) gives the
    same bits."""
    rng = np.random.default_rng(k)
    n, B = k + 1, 4
    psi = torch.from_numpy(_rand(rng, (B, 2 ** n))).to(DEV, C64)
    op = torch.from_numpy(_rand(rng, (2 ** k, 2 ** k))).to(DEV, C64)
    qubits = [int(q) for q in rng.permutation(n)[:k]]
    a = ug.apply_operator(op, qubits, psi)
    b = ug.apply_operator(op.expand(B, -1, -1).contiguous(), qubits, psi)
    assert torch.equal(a, b)


def test_wide_strided_and_broadcast_inputs(oracle):
    """Through the C ABI: input states further apart than their size (a
    strided batch), one input broadcast to every output (in_stride 0), and
    in place over a strided batch refused."""
    L = _lib.load()
    rng = np.random.default_rng(11)
    k, n, B = 7, 9, 3
    N, stride = 2 ** n, 2 ** n + 6
    buf = _rand(rng, (B * stride,))
    op = _rand(rng, (2 ** k, 2 ** k)) / 2 ** (k / 2)
    qubits = [int(q) for q in rng.permutation(n)[:k]]
    src = torch.from_numpy(buf).to(DEV, C64)
    opd = torch.from_numpy(op).to(DEV, C64)
    out = torch.empty(B, N, dtype=C64, device=DEV)
    st = _core.stream_of(DEV)
    q = _lib.qubit_array(qubits)
    assert L.gbsv_apply_operator(src.data_ptr(), out.data_ptr(), _lib.C64, n,
                                 B, stride, opd.data_ptr(), 0, q, k, st) == 0
    ref = oracle.apply_operator(
        op, qubits, np.stack([buf[s * stride:s * stride + N]
                              for s in range(B)]))
    assert _err(out, ref) <= _tol(C64, k)
    assert L.gbsv_apply_operator(src.data_ptr(), out.data_ptr(), _lib.C64, n,
                                 B, 0, opd.data_ptr(), 0, q, k, st) == 0
    ref0 = oracle.apply_operator(op, qubits, buf[:N])
    assert _err(out, np.broadcast_to(ref0, (B, N))) <= _tol(C64, k)
    assert L.gbsv_apply_operator(src.data_ptr(), src.data_ptr(), _lib.C64, n,
                                 B, stride, opd.data_ptr(), 0, q, k,
                                 st) == _lib.GBSV_ERR_UNSUPPORTED
