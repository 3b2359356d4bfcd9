"""Mirror of ``unitair.simulation`` on the GB300 kernels.

Same function names, argument meaning, validation order and exception
types as src/unitair/simulation/operations.py; every gate application is
one CUDA launch through libgbsv (no permuted copies, no einsum, no CPU path).

Batch rules (operations.py:295-329, checked against the reference):
  * operator batch == state batch           -> one operator per state
  * operator unbatched                      -> shared by every state
  * operator batched, state unbatched       -> the state is broadcast and the
                                               output takes the operator batch
  * operator batch broadcasts right-aligned onto the state batch (dims equal
    or 1)                                   -> operator expanded per state
  * anything else                           -> RuntimeError
Documented divergence: unitair silently broadcasts an operator with MORE
batch dims than a batched state against qubit axes (op (2,3,5) vs state
(3,5)); here leading operator dims of size 1 are dropped and any other
extra dim raises RuntimeError.
"""
from __future__ import annotations

import math
from typing import Iterable, Optional, Sequence, Tuple

import torch

from . import _core, _lib
from .measurement import measure  # noqa: F401  (unitair.simulation.measure)
from .states import (count_qubits, count_qubits_gate_matrix,
                     StateShapeError)  # noqa: F401  (re-exported errors)
from .states import StateLayout, count_batch_dims_tensor, get_qubit_indices


# ----------------------------------------------------------------- helpers --
def _check_dtypes(operator: torch.Tensor, state: torch.Tensor):
    if operator.dtype != state.dtype:
        names = {torch.complex64: "ComplexFloat",
                 torch.complex128: "ComplexDouble",
                 torch.float32: "Float", torch.float64: "Double"}
        raise RuntimeError(
            f"expected scalar type {names.get(state.dtype, state.dtype)} but "
            f"found {names.get(operator.dtype, operator.dtype)}")
    _core.complex_code(state.dtype)


def _prod(shape) -> int:
    p = 1
    for s in shape:
        p *= int(s)
    return p


class _BatchPlan:
    """How a (operator, state) pair maps onto the C ABI's two strides."""

    __slots__ = ("out_batch", "num_states", "in_stride", "ops", "op_stride",
                 "state_expanded", "op_batch_shape")

    def __init__(self, operator, state, n, k):
        d = 2 ** k
        N = 2 ** n
        if operator.dim() < 2:
            raise RuntimeError(
                f"Gate with size {operator.size()} is incorrectly shaped for "
                "an operator batch. Expected size is\n"
                "  (*optional_batch_dims, 2^k, 2^k)\n"
                "with k the number of qubits on which the gate acts.")
        if operator.shape[-2] != d:
            raise RuntimeError(
                f"operator of size {tuple(operator.shape)} is not square")
        state_batch = tuple(state.shape[:-1])
        op_batch = tuple(operator.shape[:-2])
        self.op_batch_shape = op_batch
        self.state_expanded = False
        if op_batch and not state_batch:
            self.out_batch = op_batch
            self.in_stride = 0
            self.state_expanded = True
            self.ops = operator.contiguous()
            self.op_stride = d * d if _prod(op_batch) > 1 else 0
        else:
            extra = len(op_batch) - len(state_batch)
            if extra > 0:
                if any(s != 1 for s in op_batch[:extra]):
                    raise RuntimeError(
                        f"operator batch {op_batch} has more dimensions than "
                        f"the state batch {state_batch}; unitair would "
                        "broadcast the extra dimensions against qubit axes. "
                        "Reshape the operator batch to the state batch.")
                op_batch = op_batch[extra:]
                operator = operator.reshape(op_batch + (d, d))
            for o, s in zip(reversed(op_batch), reversed(state_batch)):
                if o != s and o != 1:
                    raise RuntimeError(
                        f"operator batch {tuple(op_batch)} does not broadcast "
                        f"onto the state batch {state_batch}")
            self.out_batch = state_batch
            self.in_stride = N
            if _prod(op_batch) == 1:
                self.ops = operator.reshape(d, d).contiguous()
                self.op_stride = 0
            elif tuple(op_batch) == state_batch:
                self.ops = operator.contiguous()
                self.op_stride = d * d
            else:
                self.ops = operator.expand(state_batch + (d, d)).contiguous()
                self.op_stride = d * d
        self.num_states = _prod(self.out_batch)


def _launch_apply(ops, op_stride, state_c, in_stride, out, n, qubits,
                  num_states):
    dev = state_c.device
    L = _lib.load()
    rc = L.gbsv_apply_operator(
        state_c.data_ptr(), out.data_ptr(), _core.complex_code(state_c.dtype),
        n, num_states, in_stride, ops.data_ptr(), op_stride,
        _lib.qubit_array(qubits), len(qubits), _core.stream_of(dev))
    _lib.check(rc, "apply_operator")


def _validate_apply(operator, qubits, state):
    """operations.py:126-138 plus the duplicate check of utils.py:26."""
    num_qubits = count_qubits(state)
    qubits = list(qubits)
    if not set(qubits).issubset(range(num_qubits)):
        raise ValueError(
            f"qubits={qubits} is not consistent with state vector with "
            f"{num_qubits} qubits.")
    op_num_qubits = count_qubits_gate_matrix(operator)
    if len(qubits) != op_num_qubits:
        raise ValueError(
            f"Cannot apply operator with {op_num_qubits} to the "
            f"{len(qubits)} qubit sequence {qubits}.")
    if len(set(qubits)) != len(qubits):
        raise ValueError(f"qubits={qubits} contains a repeated qubit.")
    if op_num_qubits > _lib.MAX_DENSE_QUBITS:
        raise NotImplementedError(
            f"operators on more than {_lib.MAX_DENSE_QUBITS} qubits are not "
            "supported by the GB300 engine")
    _core.require_cuda(operator, state)
    _check_dtypes(operator, state)
    return num_qubits, [int(q) for q in qubits], op_num_qubits


def _dagger(ops: torch.Tensor) -> torch.Tensor:
    return ops.conj().transpose(-1, -2).contiguous()


def _apply_forward(operator, state, qubits, n, k):
    """The forward launch; returns (out, plan, contiguous state)."""
    plan = _BatchPlan(operator, state, n, k)
    state_c = state.contiguous()
    out = torch.empty(plan.out_batch + (2 ** n,), dtype=state.dtype,
                      device=state.device)
    if plan.num_states:
        _launch_apply(plan.ops, plan.op_stride, state_c, plan.in_stride,
                      out, n, qubits, plan.num_states)
    return out, plan, state_c


class _ApplyOperator(torch.autograd.Function):
    @staticmethod
    def forward(ctx, operator, state, qubits, n, k):
        out, plan, state_c = _apply_forward(operator, state, qubits, n, k)
        ctx.qubits, ctx.n, ctx.k = qubits, n, k
        ctx.plan = plan
        ctx.op_shape = operator.shape
        ctx.state_shape = state.shape
        ctx.save_for_backward(state_c)
        return out

    @staticmethod
    def backward(ctx, g):
        (state_c,) = ctx.saved_tensors
        plan, n, k, qubits = ctx.plan, ctx.n, ctx.k, ctx.qubits
        g = g.contiguous()
        grad_op = grad_state = None
        if plan.num_states == 0:
            return (torch.zeros(ctx.op_shape, dtype=g.dtype, device=g.device),
                    torch.zeros(ctx.state_shape, dtype=g.dtype,
                                device=g.device), None, None, None)
        if ctx.needs_input_grad[1]:
            gs = torch.empty_like(g)
            _launch_apply(_dagger(plan.ops), plan.op_stride, g, 2 ** n, gs, n,
                          qubits, plan.num_states)
            if plan.state_expanded:
                gs = gs.reshape(-1, 2 ** n).sum(0)
            grad_state = gs.reshape(ctx.state_shape)
        if ctx.needs_input_grad[0]:
            shared = plan.op_stride == 0
            d = 2 ** k
            L = _lib.load()
            nbytes = int(L.gbsv_operator_grad_scratch_bytes(
                plan.num_states, n, k, int(shared)))
            scratch = (torch.empty(nbytes, dtype=torch.uint8, device=g.device)
                       if nbytes else None)
            gop = torch.empty((1 if shared else plan.num_states, d, d),
                              dtype=g.dtype, device=g.device)
            rc = L.gbsv_operator_grad(
                g.data_ptr(), state_c.data_ptr(),
                _core.complex_code(g.dtype), n, plan.num_states,
                plan.in_stride, _lib.qubit_array(qubits), k, gop.data_ptr(),
                int(shared), scratch.data_ptr() if scratch is not None else
                None, nbytes, _core.stream_of(g.device))
            _lib.check(rc, "operator_grad")
            target = tuple(ctx.op_shape)
            if shared:
                grad_op = gop.reshape(target)
            else:
                grad_op = gop.reshape(plan.out_batch + (d, d))
                core = target[len(target) - grad_op.dim():] \
                    if len(target) > grad_op.dim() else target
                grad_op = grad_op.sum_to_size(core).reshape(target)
        return grad_op, grad_state, None, None, None


# ------------------------------------------------------------ public API ---
def apply_operator(operator: torch.Tensor, qubits: Iterable[int],
                   state: torch.Tensor) -> torch.Tensor:
    """Apply a (batch of) k-qubit operator(s) to ``qubits`` of ``state``.

    Drop-in for unitair.simulation.apply_operator (operations.py:45-148):
    operator (*op_batch, 2^k, 2^k), state (*state_batch, 2^n); the first
    listed qubit is the operator's most significant index bit; qubit 0 is
    the most significant bit of the amplitude index.  Returns a new
    contiguous tensor; differentiable with respect to both inputs.
    """
    n, qubits, k = _validate_apply(operator, qubits, state)
    if torch.is_grad_enabled() and (operator.requires_grad or
                                    state.requires_grad):
        return _ApplyOperator.apply(operator, state, tuple(qubits), n, k)
    # no gradient can flow: the same launch without the autograd Function
    # (its bookkeeping is most of a small state's per-gate host time)
    return _apply_forward(operator, state, qubits, n, k)[0]


def apply_operator_(operator: torch.Tensor, qubits: Iterable[int],
                    state: torch.Tensor) -> torch.Tensor:
    """In-place apply_operator for engine use: overwrites ``state``.

    The operator batch must be empty or equal to the state batch (or
    broadcast onto it); no autograd.  ``state`` must be contiguous.
    """
    n, qubits, k = _validate_apply(operator, qubits, state)
    if not state.is_contiguous():
        raise ValueError("apply_operator_ needs a contiguous state")
    plan = _BatchPlan(operator, state, n, k)
    if plan.state_expanded:
        raise ValueError("apply_operator_ cannot broadcast an unbatched "
                         "state over an operator batch")
    if plan.num_states:
        wide = not _core.inplace_ok(state.dtype, k, n, plan.op_stride != 0)
        if wide:  # this operator is not applied in place
            out = torch.empty_like(state)
            _launch_apply(plan.ops, plan.op_stride, state, 2 ** n, out, n,
                          qubits, plan.num_states)
            state.copy_(out)
        else:
            _launch_apply(plan.ops, plan.op_stride, state, 2 ** n, state, n,
                          qubits, plan.num_states)
    return state


def act_first_qubits(operator: torch.Tensor,
                     state: torch.Tensor) -> torch.Tensor:
    """Apply a k-qubit operator to qubits 0..k-1 (operations.py:236-255)."""
    num_qubits = count_qubits(state)
    k = count_qubits_gate_matrix(operator)
    if num_qubits < k:
        raise ValueError(f"Attempted to apply a {k}-qubit gate to "
                         f"{num_qubits} qubit(s).")
    return apply_operator(operator, range(k), state)


def _apply_all_qubits_kernel(operator, state, n, each):
    """One launch per qubit; operator is (*b, 2, 2), or (*b, n, 2, 2) with
    one matrix per qubit when ``each``."""
    plan = _BatchPlan(operator if not each else operator[..., 0, :, :],
                      state, n, 1)
    if each:
        if plan.op_stride:
            ops = operator.expand(plan.out_batch + (n, 2, 2)).contiguous()
            op_stride = n * 4
        else:
            ops = operator.reshape(n, 2, 2).contiguous()
            op_stride = 0
        op_qubit_stride = 4
    else:
        ops, op_stride, op_qubit_stride = plan.ops, plan.op_stride, 0
    state_c = state.contiguous()
    out = torch.empty(plan.out_batch + (2 ** n,), dtype=state.dtype,
                      device=state.device)
    if plan.num_states:
        rc = _lib.load().gbsv_apply_all_qubits(
            state_c.data_ptr(), out.data_ptr(),
            _core.complex_code(state.dtype), n, plan.num_states,
            plan.in_stride, ops.data_ptr(), op_stride, op_qubit_stride,
            _core.stream_of(state.device))
        _lib.check(rc, "apply_all_qubits")
    return out


def apply_all_qubits(operator: torch.Tensor,
                     state: torch.Tensor) -> torch.Tensor:
    """The same single-qubit operator on every qubit
    (operations.py:332-413); batch rules as apply_operator."""
    if count_qubits_gate_matrix(operator) != 1:
        raise ValueError(
            "Expected operator on 1 qubit, found a "
            f"{count_qubits_gate_matrix(operator)} qubit operator.")
    num_qubits = count_qubits(state)
    _core.require_cuda(operator, state)
    _check_dtypes(operator, state)
    if num_qubits < 1:
        raise RuntimeError("apply_all_qubits needs a state of at least one "
                           "qubit")
    if torch.is_grad_enabled() and (operator.requires_grad
                                    or state.requires_grad):
        out = state
        for q in range(num_qubits):
            out = apply_operator(operator, [q], out)
        return out
    return _apply_all_qubits_kernel(operator, state, num_qubits, False)


def apply_each_qubit(operators: torch.Tensor,
                     state: torch.Tensor) -> torch.Tensor:
    """Extension of apply_all_qubits: ``operators`` has shape
    (*op_batch, n, 2, 2) and operators[..., q, :, :] acts on qubit q.

    unitair's apply_all_qubits rejects per-qubit operator batches; this is
    the batched per-qubit rotation layer (e.g. RX(angles) with angles of
    shape (*batch, n)).  Batch rules as apply_operator.
    """
    num_qubits = count_qubits(state)
    if operators.dim() < 3 or operators.shape[-3] != num_qubits or \
            operators.shape[-1] != 2 or operators.shape[-2] != 2:
        raise ValueError(
            f"expected operators of shape (*batch, {num_qubits}, 2, 2), got "
            f"{tuple(operators.shape)}")
    _core.require_cuda(operators, state)
    _check_dtypes(operators, state)
    if torch.is_grad_enabled() and (operators.requires_grad
                                    or state.requires_grad):
        out = state
        for q in range(num_qubits):
            out = apply_operator(operators[..., q, :, :], [q], out)
        return out
    return _apply_all_qubits_kernel(operators, state, num_qubits, True)


class _ApplyPhase(torch.autograd.Function):
    @staticmethod
    def forward(ctx, angles, state):
        out = _phase_kernel(angles, state)
        ctx.save_for_backward(angles, state, out)
        return out

    @staticmethod
    def backward(ctx, g):
        angles, state, out = ctx.saved_tensors
        ga = gs = None
        if ctx.needs_input_grad[1]:
            gs = _phase_kernel(-angles, g.contiguous())
            gs = gs.to(state.dtype).sum_to_size(state.shape)
        if ctx.needs_input_grad[0]:
            # out = exp(-i a) psi  =>  dL/da = Re(i * g * conj(out))
            ga = (1j * g * out.conj()).real.to(angles.dtype)
            ga = ga.sum_to_size(angles.shape)
        return ga, gs


def _phase_kernel(angles: torch.Tensor, state: torch.Tensor) -> torch.Tensor:
    dev = _core.require_cuda(angles, state)
    scode = _core.complex_code(state.dtype)
    if angles.is_complex():
        raise NotImplementedError("apply_phase takes real angles")
    if not angles.is_floating_point():
        angles = angles.to(torch.float32)
    if angles.dtype not in (torch.float32, torch.float64):
        angles = angles.to(torch.float32)
    acode = _core.real_code(angles.dtype)
    out_dtype = torch.complex128 if (angles.dtype == torch.float64 or
                                     state.dtype == torch.complex128) \
        else torch.complex64
    a = angles.contiguous()
    s = state.contiguous()
    out_shape = torch.broadcast_shapes(a.shape, s.shape)
    out = torch.empty(out_shape, dtype=out_dtype, device=dev)
    if out.numel() == 0:
        return out
    desc = _core.bcast_desc(out_shape, _core.broadcast_strides(a, out_shape),
                            _core.broadcast_strides(s, out_shape))
    rc = _lib.load().gbsv_apply_phase(
        a.data_ptr(), acode, s.data_ptr(), scode, out.data_ptr(),
        _core.complex_code(out_dtype), desc, _core.stream_of(dev))
    _lib.check(rc, "apply_phase")
    return out


def apply_phase(angles: torch.Tensor, state: torch.Tensor) -> torch.Tensor:
    """Multiply the k-th amplitude by exp(-i angles_k) with torch
    broadcasting (operations.py:15-42).  float64 angles on a complex64
    state give a complex128 result, as in unitair."""
    return _ApplyPhase.apply(angles, state)


# ------------------------------------------------ permutations and friends --
def _permute(state: torch.Tensor, perm, n: int) -> torch.Tensor:
    _core.require_cuda(state)
    code = _core.complex_code(state.dtype)
    s = state.contiguous()
    out = torch.empty_like(s)
    if s.numel():
        rc = _lib.load().gbsv_permute_qubits(
            s.data_ptr(), out.data_ptr(), code, n, s.numel() >> n,
            _lib.qubit_array(perm), _core.stream_of(s.device))
        _lib.check(rc, "permute_qubits")
    return out


def permute_qubits(permutation: Iterable[int],
                   state_vector: torch.Tensor) -> torch.Tensor:
    """Output qubit j is input qubit permutation[j], batch dims untouched
    (operations.py:600-654)."""
    n = count_qubits(state_vector)
    perm = [int(p) for p in permutation]
    if sorted(perm) != list(range(n)):
        raise RuntimeError(f"permute(): {perm} is not a permutation of the "
                           f"{n} qubit dims")
    return _permute(state_vector, perm, n)


def swap(state: torch.Tensor, qubit_pair: Tuple[int, int]) -> torch.Tensor:
    """Exchange two qubits (operations.py:506-537); negative indices count
    from the last qubit, as in get_qubit_indices."""
    n = count_qubits(state)
    if qubit_pair[0] == qubit_pair[1]:
        return state
    qs = []
    for q in qubit_pair:
        q = int(q)
        if q >= n or q < -n:
            raise ValueError(
                "Expected index in {-num_qubits, ..., num_qubits - 1}.\n"
                f"Num_qubits: {n}, index: {list(qubit_pair)}.")
        qs.append(q % n)
    if qs[0] == qs[1]:
        return state
    perm = list(range(n))
    perm[qs[0]], perm[qs[1]] = qs[1], qs[0]
    return _permute(state, perm, n)


def roll_qubits(state: torch.Tensor, num_steps: int = 1) -> torch.Tensor:
    """Cyclic qubit shift: out[a_0..a_{n-1}] = in[a_k, ..., a_{k-1}] with
    k = num_steps mod n (operations.py:540-597)."""
    n = count_qubits(state)
    k = num_steps % n if n else 0
    if k == 0:
        return state
    perm = [(j - k) % n for j in range(n)]
    return _permute(state, perm, n)


def act_last_qubit(single_qubit_operator: torch.Tensor,
                   state: torch.Tensor) -> torch.Tensor:
    """Deprecated in unitair (operations.py:189-213): the operator on the
    last qubit."""
    import warnings
    warnings.warn(
        "act_last_qubit and act_last_qubit_tensor are outdated. These\n"
        "functions will be removed from Unitair in a later release or may\n"
        "be revised to meet our current standards.\n"
        "Please consider using apply_operator instead.")
    n = count_qubits(state)
    return apply_operator(single_qubit_operator, [n - 1], state)


def apply_to_qubits(operators: Iterable[torch.Tensor], qubits: Iterable[int],
                    state: torch.Tensor) -> torch.Tensor:
    """Single-qubit operators on the listed qubits in order
    (operations.py:416-503).  Operators on the same qubit are multiplied
    first, as unitair does (gates/matrix_algebra.py:6-51); with unbatched
    operators the fused per-qubit gates then run as one fused program."""
    from .gates import fuse_single_qubit_operators
    n = count_qubits(state)
    pairs = list(zip(qubits, operators))
    for q, _ in pairs:
        if not 0 <= int(q) < n:
            raise ValueError(
                "Expected index in {-num_qubits, ..., num_qubits - 1}.\n"
                f"Num_qubits: {n}, index: {int(q)}.")
    fused = fuse_single_qubit_operators([int(q) for q, _ in pairs],
                                        [op for _, op in pairs])
    if not fused:
        return state.contiguous()
    ops = list(fused.items())
    _core.require_cuda(state, *[op for _, op in ops])
    grad = torch.is_grad_enabled() and (
        state.requires_grad or any(op.requires_grad for _, op in ops))
    if grad or any(op.dim() != 2 for _, op in ops):
        out = state
        for q, op in ops:
            out = apply_operator(op, [q], out)
        return out
    for _, op in ops:
        _check_dtypes(op, state)
    from .fusion import Circuit
    circ = Circuit(n)
    for q, op in ops:
        circ.append(op, [q], "dense")
    prog = circ.compile(state.dtype, state.device)
    return prog.run(state.contiguous())


def _mask_of(qubits, n):
    m = 0
    for q in qubits:
        m |= 1 << (n - 1 - int(q))
    return m


def _phase_flip(state: torch.Tensor, masks) -> torch.Tensor:
    n = count_qubits(state)
    _core.require_cuda(state)
    code = _core.complex_code(state.dtype)
    s = state.contiguous()
    out = torch.empty_like(s)
    if s.numel() == 0:
        return out
    host = torch.tensor([int(m) for m in masks] or [0], dtype=torch.int64)
    dev_masks = host.pin_memory().to(s.device, non_blocking=True)
    rc = _lib.load().gbsv_phase_flip(
        s.data_ptr(), out.data_ptr(), code, n, s.numel() >> n,
        dev_masks.data_ptr(), len(masks), _core.stream_of(s.device))
    _lib.check(rc, "phase_flip")
    return out


def multi_cz(qubit_pairs: torch.Tensor, state_vector: torch.Tensor,
             num_bits_memory_cutoff: Optional[int] = None) -> torch.Tensor:
    """CZ on each (control, target) row of ``qubit_pairs`` (shape (2,) or
    (num_pairs, 2)) in one pass (operations.py:657-748).
    ``num_bits_memory_cutoff`` only tuned unitair's temporaries and is
    accepted for compatibility."""
    n = count_qubits(state_vector)
    if qubit_pairs.dim() == 1:
        qubit_pairs = qubit_pairs.view(1, 2)
    if state_vector.device.type != qubit_pairs.device.type:
        raise ValueError(
            "state_vector and qubit_qubit_pairs must have same device.")
    elif qubit_pairs.dim() != 2:
        raise ValueError("qubit_pairs must have size (2,) or (num_pairs, 2).")
    pairs = qubit_pairs.cpu().tolist()
    if any(q >= n for row in pairs for q in row):
        raise ValueError(
            "Control/target indices for CZ gate must be less than num_bits.")
    if any(q < 0 for row in pairs for q in row):
        raise ValueError("Control/target indices must be non-negative.")
    if any(row[0] == row[1] for row in pairs):
        raise ValueError("Control and target qubits are not distinct.")
    return _phase_flip(state_vector, [_mask_of(r, n) for r in pairs])


def multi_controlled_z(qubits: Iterable[int],
                       state_vector: torch.Tensor) -> torch.Tensor:
    """C..CZ on ``qubits``: -1 where all of them are 1
    (operations.py:751-783; unlike unitair, works on CUDA tensors)."""
    n = count_qubits(state_vector)
    qubits = [int(q) for q in qubits]
    if len(set(qubits)) != len(qubits) or any(
            q < 0 or q >= n for q in qubits):
        raise ValueError(f"qubits={qubits} are not distinct qubits of a "
                         f"{n}-qubit state.")
    return _phase_flip(state_vector, [_mask_of(qubits, n)])


def multi_controlled_x(state_vector: torch.Tensor, controls: Iterable[int],
                       target: int) -> torch.Tensor:
    """X on ``target`` where every control is 1 (operations.py:786-805),
    as one exact swap pass instead of H, C..CZ, H."""
    n = count_qubits(state_vector)
    controls = [int(c) for c in controls]
    target = int(target)
    if target < 0 or target >= n or target in controls or len(
            set(controls)) != len(controls) or any(
                c < 0 or c >= n for c in controls):
        raise ValueError(f"bad controls {controls} / target {target} for "
                         f"{n} qubits")
    _core.require_cuda(state_vector)
    code = _core.complex_code(state_vector.dtype)
    s = state_vector.contiguous()
    out = torch.empty_like(s)
    if s.numel():
        rc = _lib.load().gbsv_multi_controlled_x(
            s.data_ptr(), out.data_ptr(), code, n, s.numel() >> n,
            _lib.qubit_array(controls), len(controls), target,
            _core.stream_of(s.device))
        _lib.check(rc, "multi_controlled_x")
    return out


# ------------------------------------------------- tensor-layout variants --
# unitair's *_tensor functions take states in tensor layout, (*batch, 2, ...,
# 2) with one dim per qubit.  That layout is a view of the vector layout, so
# each variant reshapes to (*batch, 2^n), runs the vector function's kernel
# and returns the result viewed in tensor layout.  The pure permutations
# (swap_tensor, roll_qubits_tensor, permute_qubits_tensor without
# contiguous_output) are views in unitair and stay views here: no data moves.
def _as_vector(state_tensor: torch.Tensor, num_qubits: int) -> torch.Tensor:
    if state_tensor.dim() < num_qubits or any(
            d != 2 for d in state_tensor.shape[state_tensor.dim() -
                                               num_qubits:]):
        raise StateShapeError(data=state_tensor,
                              expected_layout=StateLayout.TENSOR)
    batch = state_tensor.shape[:state_tensor.dim() - num_qubits]
    return state_tensor.reshape(batch + torch.Size((2 ** num_qubits,)))


def _as_tensor(state: torch.Tensor, num_qubits: int) -> torch.Tensor:
    return state.view(state.shape[:-1] + torch.Size(num_qubits * [2]))


def _check_gate_qubits(operator: torch.Tensor, given: Optional[int]) -> int:
    k = count_qubits_gate_matrix(operator)
    if given is not None and int(given) != k:
        raise ValueError(f"Operator of size {tuple(operator.shape[-2:])} "
                         f"acts on {k} qubit(s), not {given}.")
    return k


def apply_operator_tensor(operator: torch.Tensor, qubits: Iterable[int],
                          state_tensor: torch.Tensor, num_qubits: int,
                          operator_num_qubits: Optional[int] = None
                          ) -> torch.Tensor:
    """apply_operator on a state in tensor layout (operations.py:151-186);
    contiguous result in tensor layout."""
    _check_gate_qubits(operator, operator_num_qubits)
    out = apply_operator(operator, list(qubits),
                         _as_vector(state_tensor, num_qubits))
    return _as_tensor(out, num_qubits)


def act_first_qubits_tensor(operator: torch.Tensor,
                            state_tensor: torch.Tensor, num_qubits: int,
                            gate_num_qubits: Optional[int] = None
                            ) -> torch.Tensor:
    """A k-qubit operator on qubits 0..k-1 of a tensor-layout state, batch
    rules as act_first_qubits (operations.py:258-329)."""
    k = _check_gate_qubits(operator, gate_num_qubits)
    if num_qubits < k:
        raise ValueError(f"Attempted to apply a {k}-qubit gate to "
                         f"{num_qubits} qubit(s).")
    out = apply_operator(operator, range(k),
                         _as_vector(state_tensor, num_qubits))
    return _as_tensor(out, num_qubits)


def act_last_qubit_tensor(single_qubit_operator: torch.Tensor,
                          state_tensor: torch.Tensor) -> torch.Tensor:
    """A (2, 2) operator contracted with the last dim of the tensor
    (operations.py:216-233, deprecated in unitair): every length-2 fibre of
    the last dim is a one-qubit state."""
    if tuple(single_qubit_operator.shape) != (2, 2):
        raise ValueError("act_last_qubit_tensor takes one (2, 2) operator, "
                         f"got {tuple(single_qubit_operator.shape)}.")
    if state_tensor.dim() < 1 or state_tensor.shape[-1] != 2:
        raise StateShapeError(data=state_tensor,
                              expected_layout=StateLayout.TENSOR)
    out = apply_operator(single_qubit_operator, [0],
                         state_tensor.reshape(-1, 2))
    return out.view(state_tensor.shape)


def apply_all_qubits_tensor(operator: torch.Tensor,
                            state_tensor: torch.Tensor,
                            num_qubits: int) -> torch.Tensor:
    """apply_all_qubits on a tensor-layout state (operations.py:369-413)."""
    out = apply_all_qubits(operator, _as_vector(state_tensor, num_qubits))
    return _as_tensor(out, num_qubits)


def apply_to_qubits_tensor(operators: Iterable[torch.Tensor],
                           qubits: Iterable[int], state_tensor: torch.Tensor,
                           num_qubits: int) -> torch.Tensor:
    """apply_to_qubits on a tensor-layout state (operations.py:449-503)."""
    out = apply_to_qubits(operators, qubits,
                          _as_vector(state_tensor, num_qubits))
    return _as_tensor(out, num_qubits)


def swap_tensor(state_tensor: torch.Tensor, qubit_pair: Tuple[int, int],
                num_qubits: int) -> torch.Tensor:
    """Two qubit dims exchanged, as a view (operations.py:520-537)."""
    if qubit_pair[0] == qubit_pair[1]:
        return state_tensor
    q1, q2 = get_qubit_indices(index=qubit_pair, state_tensor=state_tensor,
                               num_qubits=num_qubits)
    return state_tensor.transpose(q1, q2)


def roll_qubits_tensor(state_tensor: torch.Tensor, num_qubits: int,
                       num_steps: int = 1) -> torch.Tensor:
    """Cyclic shift of the qubit dims by num_steps, as a view
    (operations.py:565-597)."""
    nb = count_batch_dims_tensor(state_tensor, num_qubits)
    num_steps = num_steps % num_qubits
    if num_steps == 0:
        return state_tensor
    ident = list(range(nb, nb + num_qubits))
    perm = ident[-num_steps:] + ident[:-num_steps]
    return state_tensor.permute(list(range(nb)) + perm)


def permute_qubits_tensor(permutation: Iterable[int],
                          state_tensor: torch.Tensor, num_qubits: int,
                          contiguous_output: bool = False) -> torch.Tensor:
    """Qubit dims permuted (output qubit j = input qubit permutation[j]),
    batch dims untouched (operations.py:626-654).  A view, as in unitair;
    with contiguous_output the permuted amplitudes are written by the tiled
    permutation kernel."""
    perm = [int(p) for p in permutation]
    nb = state_tensor.dim() - num_qubits
    if not contiguous_output:
        return torch.permute(state_tensor,
                             tuple(range(nb)) + tuple(p + nb for p in perm))
    if sorted(perm) != list(range(num_qubits)):
        raise RuntimeError(f"permute(): {perm} is not a permutation of the "
                           f"{num_qubits} qubit dims")
    out = _permute(_as_vector(state_tensor, num_qubits), perm, num_qubits)
    return _as_tensor(out, num_qubits)
