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
