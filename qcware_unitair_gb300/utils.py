"""Small host helpers of unitair's public API: qubit permutations as lists
(utils.py:5-47), integers as bit vectors (utils.py:50-77) and the batch shape
of an operator batch (simulation/utils.py:4-36)."""
from __future__ import annotations

from typing import List

import torch


def permutation_to_front(n: int, entries: List[int]) -> List[int]:
    """The permutation of n elements that moves ``entries`` to the front in
    their order and keeps the rest in order: (5, [2, 1]) -> [2, 1, 0, 3, 4]
    (utils.py:5-27).  Entry j of the result is the element placed in slot
    j, torch.permute's convention."""
    front = list(entries)
    rest = [i for i in range(n) if i not in set(front)]
    return front + rest


def inverse_list_permutation(perm: List[int]) -> List[int]:
    """inverse[perm[j]] = j: [1, 2, 3, 4, 0] -> [4, 0, 1, 2, 3]
    (utils.py:30-47)."""
    inverse = [None] * len(perm)
    for slot, element in enumerate(perm):
        inverse[element] = slot
    return inverse


def bool_to_strings(bool_data) -> str:
    """[True, False, False, True] -> '1001' (utils.py:70-77)."""
    return "".join(str(int(b.item() if isinstance(b, torch.Tensor) else b))
                   for b in bool_data)


def int_to_bin(x: int, num_bits: int, str_output: bool = False,
               device: torch.device = torch.device("cpu")):
    """x as num_bits bits, most significant first: a bool tensor, or a
    '0'/'1' string with str_output (utils.py:50-67)."""
    if x >= 2 ** num_bits:
        raise ValueError(f"Insufficient bits to store integer {x}.")
    if x < 0:
        raise ValueError(f"Expected a nonnegative integer, found {x}.")
    bits = [(x >> (num_bits - 1 - j)) & 1 for j in range(num_bits)]
    out = torch.tensor(bits, dtype=torch.bool, device=device)
    return bool_to_strings(out) if str_output else out


def count_gate_batch_dims(gate: torch.Tensor) -> int:
    """Batch dims of an operator batch (*batch, 2^k, 2^k)
    (simulation/utils.py:4-23)."""
    out = gate.dim() - 2
    if out < 0:
        raise RuntimeError(
            f"Gate with size {gate.size()} is incorrectly shaped for an "
            "operator batch. Expected size is\n"
            "  (*optional_batch_dims, 2^k, 2^k)\n"
            "with k the number of qubits on which the gate acts.")
    return out


def gate_batch_size(gate: torch.Tensor) -> torch.Size:
    """The batch shape of an operator batch (simulation/utils.py:26-36)."""
    return gate.size()[:count_gate_batch_dims(gate)]
