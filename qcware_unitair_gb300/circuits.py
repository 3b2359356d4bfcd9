"""Synthetic workloads: the canonical random circuit and random states.

Gate set {H, X, Y, Z, S, T, RX, RY, RZ, CNOT, CZ, SWAP}, drawn uniformly;
rotation angles theta ~ U[0, 2 pi) shared across a batch; the qubits of a
gate are uniform and distinct; RX(theta) = exp_x(theta / 2) and likewise
RY, RZ (unitair's exp_* are e^{-i a P}).  Circuits come from
``numpy.random.default_rng(seed)``; states from ``torch.manual_seed(seed)``
exactly like unitair's rand_state (i.i.d. standard-normal complex
amplitudes normalised per state, src/unitair/initializations.py:71-100).

Matrices are built in complex128 from the angles so that a complex128 run
and its oracle use exact gates; a complex64 run rounds them once.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

GATE_SET = ("H", "X", "Y", "Z", "S", "T", "RX", "RY", "RZ", "CNOT", "CZ",
            "SWAP")
TWO_QUBIT = ("CNOT", "CZ", "SWAP")
ROTATIONS = ("RX", "RY", "RZ")
DIAGONAL = ("Z", "S", "T", "RZ", "CZ")

_S2 = 1.0 / math.sqrt(2.0)


def gate_matrix(name: str, theta: Optional[float] = None) -> np.ndarray:
    """complex128 matrix of a gate of the canonical set."""
    if name == "H":
        return np.array([[_S2, _S2], [_S2, -_S2]], dtype=np.complex128)
    if name == "X":
        return np.array([[0, 1], [1, 0]], dtype=np.complex128)
    if name == "Y":
        return np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    if name == "Z":
        return np.array([[1, 0], [0, -1]], dtype=np.complex128)
    if name == "S":
        return np.array([[1, 0], [0, 1j]], dtype=np.complex128)
    if name == "T":
        return np.array([[1, 0], [0, np.exp(1j * math.pi / 4)]],
                        dtype=np.complex128)
    if name in ROTATIONS:
        a = theta / 2.0
        c, s = math.cos(a), math.sin(a)
        if name == "RX":
            return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)
        if name == "RY":
            return np.array([[c, -s], [s, c]], dtype=np.complex128)
        return np.array([[complex(c, -s), 0], [0, complex(c, s)]],
                        dtype=np.complex128)
    if name == "CNOT":
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = [[0, 1], [1, 0]]
        return m
    if name == "CZ":
        return np.diag([1, 1, 1, -1]).astype(np.complex128)
    if name == "SWAP":
        m = np.zeros((4, 4), dtype=np.complex128)
        m[0, 0] = m[1, 2] = m[2, 1] = m[3, 3] = 1
        return m
    raise ValueError(f"unknown gate {name}")


@dataclass(frozen=True)
class Gate:
    name: str
    qubits: Tuple[int, ...]
    theta: Optional[float] = None

    def matrix(self) -> np.ndarray:
        return gate_matrix(self.name, self.theta)

    @property
    def diagonal(self) -> bool:
        return self.name in DIAGONAL


def random_circuit(num_qubits: int, num_gates: int, seed: int = 0,
                   gate_set: Sequence[str] = GATE_SET) -> List[Gate]:
    """Uniform gates from ``gate_set`` on uniform distinct qubits."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(num_gates):
        name = gate_set[int(rng.integers(len(gate_set)))]
        if name in TWO_QUBIT:
            if num_qubits < 2:
                name = "H"
                qs = (int(rng.integers(num_qubits)),)
            else:
                qs = tuple(int(q) for q in rng.choice(num_qubits, size=2,
                                                      replace=False))
        else:
            qs = (int(rng.integers(num_qubits)),)
        theta = float(rng.uniform(0.0, 2.0 * math.pi)) \
            if name in ROTATIONS else None
        gates.append(Gate(name, qs, theta))
    return gates


def random_states(num_qubits: int, batch_dims: Sequence[int] = (),
                  dtype: torch.dtype = torch.complex64, seed: int = 0,
                  device="cpu") -> torch.Tensor:
    """rand_state with a seed: randn complex, normalised per state."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    size = tuple(batch_dims) + (2 ** num_qubits,)
    s = torch.randn(size, dtype=dtype, device=device, generator=g)
    norm = (s.conj() * s).real.sum(-1, keepdim=True).sqrt()
    return s / norm


def zero_state(num_qubits: int, batch_dims: Sequence[int] = (),
               dtype: torch.dtype = torch.complex64,
               device="cpu") -> torch.Tensor:
    s = torch.zeros(tuple(batch_dims) + (2 ** num_qubits,), dtype=dtype,
                    device=device)
    s[..., 0] = 1
    return s


def circuit_ops(gates: Sequence[Gate], dtype=torch.complex64,
                device="cpu") -> List[Tuple[torch.Tensor, Tuple[int, ...]]]:
    """(matrix tensor, qubits) pairs ready for apply_operator."""
    return [(torch.from_numpy(g.matrix()).to(dtype=dtype, device=device),
             g.qubits) for g in gates]
