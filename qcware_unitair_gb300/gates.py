"""Gate matrix builders with unitair's conventions
(src/unitair/gates/gates.py:6-213, gate_construction.py:6-38).

  exp_x(a) = e^{-i a X},  exp_y(a) = e^{-i a Y},  exp_z(a) = diag(e^{-ia}, e^{ia})
  so the textbook RX(theta) = exp_x(theta / 2); rx/ry/rz below are those.
Angles may be Python floats (-> (2, 2)) or tensors of any shape
(-> (*angle_shape, 2, 2)), on the angle's device.

Divergence: unitair never forwards ``dtype`` to the builder, so its
rotation gates are complex64 whatever is asked (gate_construction.py:24);
here an explicit ``dtype`` is honoured.  The default is complex64 as in
unitair.  Builders are small torch ops: they produce inputs, they are not
the hot path.
"""
from __future__ import annotations

import functools
import math
from typing import Dict, Iterable, Optional, Union

import torch

Angle = Union[torch.Tensor, float]


def _angles(angle: Angle, dtype: torch.dtype):
    if not isinstance(angle, torch.Tensor):
        angle = torch.tensor(float(angle))
    real = torch.float64 if dtype == torch.complex128 else torch.float32
    return angle.to(real)


def _stack2(a, b, c, d):
    return torch.stack([torch.stack([a, b], -1), torch.stack([c, d], -1)], -2)


def _check_complex(dtype):
    if not dtype.is_complex:
        raise TypeError(f"gate dtype must be complex, got {dtype}")


def exp_x(angle: Angle, dtype: torch.dtype = torch.complex64):
    """e^{-i angle X} (gates.py:6-32)."""
    _check_complex(dtype)
    a = _angles(angle, dtype)
    c = torch.cos(a).to(dtype)
    s = (torch.sin(a) * 1j).to(dtype)
    return _stack2(c, -s, -s, c)


def exp_y(angle: Angle, dtype: torch.dtype = torch.complex64):
    """e^{-i angle Y} (gates.py:35-61)."""
    _check_complex(dtype)
    a = _angles(angle, dtype)
    c = torch.cos(a).to(dtype)
    s = torch.sin(a).to(dtype)
    return _stack2(c, -s, s, c)


def exp_z(angle: Angle, dtype: torch.dtype = torch.complex64):
    """e^{-i angle Z} = diag(e^{-i angle}, e^{i angle}) (gates.py:64-91)."""
    _check_complex(dtype)
    a = _angles(angle, dtype)
    c = torch.cos(a)
    s = torch.sin(a)
    zero = torch.zeros_like(c).to(dtype)
    return _stack2(torch.complex(c, -s).to(dtype), zero, zero,
                   torch.complex(c, s).to(dtype))


def rx(theta: Angle, dtype: torch.dtype = torch.complex64):
    """Standard RX(theta) = exp_x(theta / 2)."""
    return exp_x(_half(theta), dtype)


def ry(theta: Angle, dtype: torch.dtype = torch.complex64):
    """Standard RY(theta) = exp_y(theta / 2)."""
    return exp_y(_half(theta), dtype)


def rz(theta: Angle, dtype: torch.dtype = torch.complex64):
    """Standard RZ(theta) = exp_z(theta / 2)."""
    return exp_z(_half(theta), dtype)


def _half(theta: Angle):
    return theta / 2 if isinstance(theta, torch.Tensor) else float(theta) / 2


def _const(rows, device, dtype):
    t = torch.tensor(rows, dtype=torch.complex128)
    return t.to(device=device or "cpu",
                dtype=dtype if dtype is not None else torch.complex64)


def hadamard(device: Optional[torch.device] = None,
             dtype: Optional[torch.dtype] = None):
    v = 2.0 ** -0.5
    return _const([[v, v], [v, -v]], device, dtype)


def pauli_x(device=None, dtype=None):
    return _const([[0, 1], [1, 0]], device, dtype)


def pauli_y(device=None, dtype=None):
    return _const([[0, -1j], [1j, 0]], device, dtype)


def pauli_z(device=None, dtype=None):
    return _const([[1, 0], [0, -1]], device, dtype)


def s_gate(device=None, dtype=None):
    return _const([[1, 0], [0, 1j]], device, dtype)


def t_gate(device=None, dtype=None):
    w = complex(math.cos(math.pi / 4), math.sin(math.pi / 4))
    return _const([[1, 0], [0, w]], device, dtype)


def cnot(device=None, dtype=None):
    """CNOT with the first listed qubit as control (gates.py:170-188)."""
    return _const([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]],
                  device, dtype)


cx = cnot


def cz(device=None, dtype=None):
    return _const([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, -1]],
                  device, dtype)


def swap(device=None, dtype=None):
    return _const([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],
                  device, dtype)


def fuse_single_qubit_operators(
        qubits: Iterable[int],
        operators: Iterable[torch.Tensor]) -> Dict[int, torch.Tensor]:
    """Per qubit, the product of the single-qubit operators listed for it,
    later operators on the left (gates/matrix_algebra.py:6-51): qubits
    [2, 4, 2, 7] with operators A, B, C, D give {2: C @ A, 4: B, 7: D}.
    Operators are (*batch, 2, 2) and multiply with torch.matmul's batch
    broadcasting; keys keep the order of first appearance."""
    fused: Dict[int, torch.Tensor] = {}
    for q, op in zip(qubits, operators):
        fused[q] = torch.matmul(op, fused[q]) if q in fused else op
    return fused


# ------------------------------------------- gate construction helpers ---
# unitair builds its gates with two decorators and a nested stack
# (gates/gate_construction.py:6-94).  Same behaviour here, without the
# third-party ``decorator`` package: both work bare or with keywords.
def nested_stack(params, roll: bool = False) -> torch.Tensor:
    """A tensor from a nested list of equally sized tensors: [[a, b],
    [c, d]] with a..d of size (5,) -> (2, 2, 5), or (5, 2, 2) with roll
    (the tensors' own dims moved to the front as batch dims)."""
    # every nesting level drops a leading size-1 dim, as unitair's does
    if isinstance(params[0], torch.Tensor):
        out = torch.stack(list(params))
    else:
        out = torch.stack([nested_stack(x) for x in params])
    out = out.squeeze(0)
    if not roll:
        return out
    inner = params
    while not isinstance(inner, torch.Tensor):
        inner = inner[0]
    k = inner.dim()
    d = out.dim()
    return out.permute(list(range(d - k, d)) + list(range(d - k)))


def parameterized_gate(gate_function=None, strictly_complex: bool = False):
    """Decorator: the gate function receives its parameters as a 1-d tensor
    (a float or a 0-d tensor becomes one entry, squeezed away again in the
    result) and returns a tensor or a nested list of tensors, stacked with
    the parameter dims in front.  As in unitair, only the parameters reach
    the gate function."""
    if gate_function is None:
        return functools.partial(parameterized_gate,
                                 strictly_complex=strictly_complex)

    @functools.wraps(gate_function)
    def build(params, *args, **kwargs):
        squeeze = False
        if not isinstance(params, torch.Tensor):
            params = torch.tensor([float(params)], device=torch.device("cpu"))
            squeeze = True
        elif params.dim() == 0:
            params = params.unsqueeze(0)
            squeeze = True
        gate = gate_function(params)
        if not isinstance(gate, torch.Tensor):
            gate = nested_stack(gate, roll=True)
        if squeeze:
            gate = gate.squeeze(0)
        if strictly_complex and not torch.is_complex(gate):
            raise TypeError(
                "This parameterized gate is required to be complex but the\n"
                f"gate ended up having dtype {gate.dtype}. Check the\n"
                "construction of the gate decorated with parameterized_gate,"
                "\nand ensure that it returns a complex Tensor with the given"
                f"\nparameters (which have dtype {params.dtype}).")
        return gate
    return build


def constant_gate(gate_function=None, strictly_complex: bool = False):
    """Decorator: the gate function returns nested lists of numbers; the
    gate is that tensor on ``device`` (CPU by default) in ``dtype``."""
    if gate_function is None:
        return functools.partial(constant_gate,
                                 strictly_complex=strictly_complex)

    @functools.wraps(gate_function)
    def build(device=None, dtype=None):
        gate = torch.tensor(gate_function(),
                            device=device or torch.device("cpu"))
        if dtype is not None:
            gate = gate.to(dtype=dtype)
        if strictly_complex and not torch.is_complex(gate):
            raise TypeError("This gate requires a complex dtype, but it ended "
                            f"up with dtype {gate.dtype}.")
        return gate
    return build
