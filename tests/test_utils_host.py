"""unitair's small host helpers (utils.py, simulation/utils.py,
gates/gate_construction.py): the known answers of their docstrings and
the gate-construction behaviour."""
import math

import pytest
import torch

from qcware_unitair_gb300 import gates as G
from qcware_unitair_gb300 import utils as U


def test_permutation_helpers():
    assert U.permutation_to_front(5, [2]) == [2, 0, 1, 3, 4]
    assert U.permutation_to_front(5, [2, 1]) == [2, 1, 0, 3, 4]
    assert U.inverse_list_permutation([1, 2, 3, 4, 0]) == [4, 0, 1, 2, 3]
    p = U.permutation_to_front(7, [5, 0, 3])
    inv = U.inverse_list_permutation(p)
    assert [p[inv[j]] for j in range(7)] == list(range(7))


def test_int_to_bin_and_strings():
    assert U.int_to_bin(5, 4).tolist() == [False, True, False, True]
    assert U.int_to_bin(5, 4, str_output=True) == "0101"
    assert U.int_to_bin(0, 3, str_output=True) == "000"
    assert U.bool_to_strings([True, False, False, True]) == "1001"
    with pytest.raises(ValueError):
        U.int_to_bin(8, 3)
    with pytest.raises(ValueError):
        U.int_to_bin(-1, 3)


def test_gate_batch_helpers():
    g = torch.zeros(6, 5, 4, 4)
    assert U.count_gate_batch_dims(g) == 2
    assert U.gate_batch_size(g) == torch.Size([6, 5])
    assert U.gate_batch_size(torch.zeros(2, 2)) == torch.Size([])
    with pytest.raises(RuntimeError):
        U.count_gate_batch_dims(torch.zeros(4))


def test_nested_stack():
    a, b, c, d = (torch.full((5,), float(i)) for i in range(4))
    assert G.nested_stack([[a, b], [c, d]]).shape == (2, 2, 5)
    r = G.nested_stack([[a, b], [c, d]], roll=True)
    assert r.shape == (5, 2, 2)
    assert r[3].tolist() == [[0.0, 1.0], [2.0, 3.0]]
    x = torch.zeros(6, 9, 8)
    assert G.nested_stack([[x, x], [x, x]], roll=True).shape == (6, 9, 8, 2,
                                                                  2)
    # a length-1 level is squeezed away at every depth
    assert G.nested_stack([[[a, b], [c, d]]]).shape == (2, 2, 5)


def test_parameterized_and_constant_gates():
    @G.parameterized_gate(strictly_complex=True)
    def rot(theta):
        c = torch.cos(theta).to(torch.complex64)
        s = torch.sin(theta).to(torch.complex64)
        return [[[c, -1j * s], [-1j * s, c]]]

    m = rot(0.5)
    assert m.shape == (2, 2) and m.dtype == torch.complex64
    assert abs(m[0, 0].real.item() - math.cos(0.5)) < 1e-6
    assert rot(torch.tensor([0.1, 0.2, 0.3])).shape == (3, 2, 2)
    assert rot(torch.tensor(0.1)).shape == (2, 2)

    @G.parameterized_gate(strictly_complex=True)
    def real_only(theta):
        return [[[torch.cos(theta), torch.sin(theta)],
                 [torch.sin(theta), torch.cos(theta)]]]
    with pytest.raises(TypeError):
        real_only(0.3)

    @G.parameterized_gate
    def bare(theta):
        return [[[theta, theta], [theta, theta]]]
    assert bare(1.0).shape == (2, 2)

    @G.constant_gate
    def hadamard_like():
        s = 1 / math.sqrt(2)
        return [[s, s], [s, -s]]
    h = hadamard_like()
    assert h.shape == (2, 2) and h.dtype == torch.float32
    assert hadamard_like(dtype=torch.complex128).dtype == torch.complex128

    @G.constant_gate(strictly_complex=True)
    def real_const():
        return [[1.0, 0.0], [0.0, 1.0]]
    with pytest.raises(TypeError):
        real_const()
    assert real_const(dtype=torch.complex64).dtype == torch.complex64
