"""The engine's core operations as torch.library custom ops (namespace
``gbsv``), so that torch's dispatcher and ``torch.compile`` see them as
single opaque operations rather than tracing into ctypes calls.

    torch.ops.gbsv.apply_operator(operator, qubits, state)
    torch.ops.gbsv.apply_phase(angles, state)
    torch.ops.gbsv.norm_squared(state)
    torch.ops.gbsv.abs_squared(state)
    torch.ops.gbsv.inner_product(state_1, state_2)

Each runs the same CUDA kernels as the functions of ``simulation`` and
``states`` (unitair's apply_operator / apply_phase,
src/unitair/simulation/operations.py:15-148, and the reductions of
src/unitair/states/innerprod.py:4-65).  Each fake implementation derives
the output shape and dtype from the same batch rules without touching
data.  apply_operator and apply_phase are differentiable: their backward
recomputes the forward through the autograd functions of ``simulation``.
"""
from __future__ import annotations

from typing import List

import torch

from . import simulation, states

_real = {torch.complex64: torch.float32, torch.complex128: torch.float64}


# ------------------------------------------------------- apply_operator --
@torch.library.custom_op("gbsv::apply_operator", mutates_args=())
def apply_operator(operator: torch.Tensor, qubits: List[int],
                   state: torch.Tensor) -> torch.Tensor:
    with torch.no_grad():
        return simulation.apply_operator(operator, qubits, state)


@apply_operator.register_fake
def _(operator, qubits, state):
    n, _, k = simulation._validate_apply(operator, qubits, state)
    plan = simulation._BatchPlan(operator, state, n, k)
    return state.new_empty(plan.out_batch + (2 ** n,))


def _apply_operator_setup(ctx, inputs, output):
    operator, qubits, state = inputs
    ctx.qubits = list(qubits)
    ctx.save_for_backward(operator, state)


def _apply_operator_backward(ctx, grad):
    operator, state = ctx.saved_tensors
    want = ctx.needs_input_grad
    with torch.enable_grad():
        op = operator.detach().requires_grad_(want[0])
        st = state.detach().requires_grad_(want[2])
        out = simulation.apply_operator(op, ctx.qubits, st)
        wrt = [x for x in (op, st) if x.requires_grad]
        got = iter(torch.autograd.grad(out, wrt, grad)) if wrt else iter(())
    return (next(got) if want[0] else None, None,
            next(got) if want[2] else None)


apply_operator.register_autograd(_apply_operator_backward,
                                 setup_context=_apply_operator_setup)


# ---------------------------------------------------------- apply_phase --
@torch.library.custom_op("gbsv::apply_phase", mutates_args=())
def apply_phase(angles: torch.Tensor, state: torch.Tensor) -> torch.Tensor:
    with torch.no_grad():
        return simulation.apply_phase(angles, state)


@apply_phase.register_fake
def _(angles, state):
    dtype = (torch.complex128 if angles.dtype == torch.float64
             or state.dtype == torch.complex128 else torch.complex64)
    shape = torch.broadcast_shapes(angles.shape, state.shape)
    return state.new_empty(shape, dtype=dtype)


def _apply_phase_setup(ctx, inputs, output):
    ctx.save_for_backward(*inputs)


def _apply_phase_backward(ctx, grad):
    angles, state = ctx.saved_tensors
    want = ctx.needs_input_grad
    with torch.enable_grad():
        a = angles.detach().requires_grad_(want[0])
        s = state.detach().requires_grad_(want[1])
        out = simulation.apply_phase(a, s)
        wrt = [x for x in (a, s) if x.requires_grad]
        got = iter(torch.autograd.grad(out, wrt, grad)) if wrt else iter(())
    return (next(got) if want[0] else None, next(got) if want[1] else None)


apply_phase.register_autograd(_apply_phase_backward,
                              setup_context=_apply_phase_setup)


# ----------------------------------------------------------- reductions --
@torch.library.custom_op("gbsv::norm_squared", mutates_args=())
def norm_squared(state: torch.Tensor) -> torch.Tensor:
    with torch.no_grad():
        return states.norm_squared(state)


@norm_squared.register_fake
def _(state):
    return state.new_empty(state.shape[:-1], dtype=_real[state.dtype])


@torch.library.custom_op("gbsv::abs_squared", mutates_args=())
def abs_squared(state: torch.Tensor) -> torch.Tensor:
    with torch.no_grad():
        return states.abs_squared(state)


@abs_squared.register_fake
def _(state):
    return state.new_empty(state.shape, dtype=_real[state.dtype])


@torch.library.custom_op("gbsv::inner_product", mutates_args=())
def inner_product(state_1: torch.Tensor,
                  state_2: torch.Tensor) -> torch.Tensor:
    with torch.no_grad():
        return states.inner_product(state_1, state_2)


@inner_product.register_fake
def _(state_1, state_2):
    shape = torch.broadcast_shapes(state_1.shape[:-1], state_2.shape[:-1])
    dtype = torch.promote_types(state_1.dtype, state_2.dtype)
    return state_1.new_empty(shape, dtype=dtype)
