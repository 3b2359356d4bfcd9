"""State constructors with unitair's signatures
(src/unitair/initializations.py:10-128).  They build inputs with torch on
the requested device; normalisation uses the engine's norm kernel when the
device is CUDA."""
from __future__ import annotations

from typing import Optional, Sequence, Union

import torch

from . import states


def unit_vector_from_bitstring(bitstring, device=torch.device("cpu"),
                               dtype=torch.complex64):
    try:
        bits = torch.tensor(bitstring)
    except TypeError:
        bits = torch.tensor([int(i) for i in bitstring])
    n = bits.size()[0]
    powers = torch.tensor([2 ** k for k in reversed(range(n))])
    return unit_vector(index=int((powers * bits).sum()), num_qubits=n,
                       device=device, dtype=dtype)


def unit_vector(index: int, num_qubits: Optional[int] = None,
                dim: Optional[int] = None, device=torch.device("cpu"),
                dtype=torch.complex64):
    if dim is None:
        if num_qubits is None:
            raise TypeError("To specify a unit vector, provide either "
                            "`num_qubits` or  `dim`.")
        dim = 2 ** num_qubits
    elif num_qubits is not None:
        raise TypeError("Unit vector can be specified by `dim` or "
                        "`num_qubits` but not both.")
    v = torch.zeros(dim, device=device, dtype=dtype)
    v[index] = 1
    return v


def rand_state(num_qubits: int, batch_dims: Optional[Sequence] = None,
               device=torch.device("cpu"), dtype=torch.complex64,
               requires_grad: bool = False) -> torch.Tensor:
    size = (torch.Size(batch_dims) if batch_dims is not None
            else torch.Size()) + torch.Size((2 ** num_qubits,))
    s = torch.randn(size, device=device, dtype=dtype)
    if s.is_cuda and s.is_complex():
        norm = states.norm_squared(s).sqrt()
    else:
        norm = (s.conj() * s).real.sum(-1).sqrt() if s.is_complex() else \
            (s * s).sum(-1).sqrt()
    s /= norm.view(norm.size() + (1,))
    return s.requires_grad_(requires_grad)


def uniform_superposition(num_qubits: int,
                          batch_dims: Optional[Sequence] = None,
                          device=torch.device("cpu"), dtype=torch.complex64,
                          requires_grad: bool = False):
    s = 2 ** (-num_qubits / 2.0) * torch.ones(2 ** num_qubits, device=device,
                                              dtype=dtype)
    if batch_dims is not None:
        s = s.repeat(torch.Size(batch_dims) + (1,))
    return s.requires_grad_(requires_grad)
