"""The reference's own property tests (tests/test_operations.py:23-201,
tests/test_unitary.py:10-127), restated on the CUDA path with seeded random
inputs in place of Hypothesis draws (Hypothesis is not installed on every
machine the tests run on): normalised states of 1-8 qubits with up to two
batch dims, random non-unitary operators, the three batch structures."""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300 import simulation as sim
from qcware_unitair_gb300.states import to_tensor_layout

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
CASES = [(1, ()), (2, (3,)), (3, (2, 3)), (5, ()), (6, (3,)), (8, (2,))]


def _state(rng, n, batch, dtype=torch.complex64):
    a = rng.uniform(-1, 1, size=batch + (2 ** n,)) + 1j * rng.uniform(
        -1, 1, size=batch + (2 ** n,))
    a /= np.linalg.norm(a, axis=-1, keepdims=True)
    return torch.from_numpy(a).to(dtype).to(DEV)


def _op(rng, k, batch=(), dtype=torch.complex64):
    d = 2 ** k
    a = rng.uniform(-1, 1, size=batch + (d, d)) + 1j * rng.uniform(
        -1, 1, size=batch + (d, d))
    return torch.from_numpy(a).to(dtype).to(DEV)


def _close(a, b, tol):
    return torch.allclose(a.to(torch.complex128), b.to(torch.complex128),
                          atol=tol, rtol=0)


@pytest.mark.parametrize("n,batch", CASES)
def test_apply_operator_matches_act_first_qubits(n, batch):
    rng = np.random.default_rng(n)
    psi = _state(rng, n, batch)
    for k in range(1, min(n, 2) + 1):
        op = _op(rng, k)
        assert torch.equal(ug.apply_operator(op, list(range(k)), psi),
                           sim.act_first_qubits(op, psi))


@pytest.mark.parametrize("n,batch", [c for c in CASES if c[1]])
def test_batched_entries_equal_unbatched_calls(n, batch):
    """Equal batches, an unbatched operator, and a batched operator on an
    unbatched state: each entry equals the call on that entry alone."""
    rng = np.random.default_rng(10 + n)
    psi = _state(rng, n, batch)
    k = min(n, 2)
    qubits = [int(q) for q in rng.choice(n, size=k, replace=False)]
    ops = _op(rng, k, batch)
    out = ug.apply_operator(ops, qubits, psi)
    shared = _op(rng, k)
    out_shared = ug.apply_operator(shared, qubits, psi)
    for idx in np.ndindex(*batch):
        assert _close(out[idx], ug.apply_operator(ops[idx], qubits, psi[idx]),
                      1e-6)
        assert _close(out_shared[idx],
                      ug.apply_operator(shared, qubits, psi[idx]), 1e-6)
    one = psi[(0,) * len(batch)]
    out_b = ug.apply_operator(ops, qubits, one)
    assert out_b.shape == batch + (2 ** n,)
    for idx in np.ndindex(*batch):
        assert _close(out_b[idx], ug.apply_operator(ops[idx], qubits, one),
                      1e-6)
    # apply_all_qubits follows the same rules
    op1 = _op(rng, 1, batch)
    out = ug.apply_all_qubits(op1, psi)
    for idx in np.ndindex(*batch):
        assert _close(out[idx], ug.apply_all_qubits(op1[idx], psi[idx]),
                      1e-5)


@pytest.mark.parametrize("n,batch", CASES)
def test_apply_phase_inverse_and_formula(n, batch):
    rng = np.random.default_rng(20 + n)
    psi = _state(rng, n, batch)
    ang = torch.from_numpy(rng.uniform(0, 2 * np.pi, size=batch + (2 ** n,))
                           ).float().to(DEV)
    there = ug.apply_phase(ang, psi)
    assert _close(ug.apply_phase(-ang, there), psi, 1e-4)
    manual = torch.complex(psi.real * torch.cos(ang) + psi.imag *
                           torch.sin(ang),
                           psi.imag * torch.cos(ang) - psi.real *
                           torch.sin(ang))
    assert _close(there, manual, 1e-5)


@pytest.mark.parametrize("n,batch", [c for c in CASES if c[0] >= 2])
def test_swap_properties(n, batch):
    rng = np.random.default_rng(30 + n)
    psi = _state(rng, n, batch)
    a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
    s = ug.swap(psi, (a, b))
    assert torch.equal(ug.swap(s, (a, b)), psi)          # involution
    assert torch.equal(ug.swap(psi, (b, a)), s)          # symmetric
    perm = list(range(n))
    perm[a], perm[b] = b, a
    assert torch.equal(sim.permute_qubits(perm, psi), s)
    nb = len(batch)
    manual = to_tensor_layout(psi).transpose(nb + a, nb + b).reshape(
        psi.shape)
    assert torch.equal(s, manual)


@pytest.mark.parametrize("n,batch", CASES)
def test_apply_to_qubits_equals_apply_all(n, batch):
    rng = np.random.default_rng(40 + n)
    psi = _state(rng, n, batch)
    op = _op(rng, 1)
    a = ug.apply_to_qubits([op] * n, list(range(n)), psi)
    b = ug.apply_all_qubits(op, psi)
    scale = float(b.abs().max()) + 1.0
    assert _close(a, b, 1e-5 * scale)


@pytest.mark.parametrize("n,batch", CASES)
def test_act_last_qubit(n, batch):
    rng = np.random.default_rng(50 + n)
    psi = _state(rng, n, batch)
    op = _op(rng, 1)
    with pytest.warns(UserWarning):
        last = sim.act_last_qubit(op, psi)
    assert torch.equal(last, ug.apply_operator(op, [n - 1], psi))
