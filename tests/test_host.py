"""Host-side logic of the drop-in, on CPU: validation order and exception
types, and the batch-broadcast plan, against what the reference did for
the same shapes (tests/golden/cases.json, recorded from unitair)."""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300 import simulation as sim
from qcware_unitair_gb300 import states as S
from qcware_unitair_gb300._core import bcast_desc, broadcast_strides
from conftest import golden_data

G = golden_data()
DT = {"c64": torch.complex64, "c128": torch.complex128}
EXC = {"ValueError": ValueError, "RuntimeError": RuntimeError,
       "StateShapeError": S.StateShapeError}


def _inputs(spec):
    op = torch.ones(spec["op_shape"], dtype=DT[spec["op_dtype"]])
    st = torch.ones(spec["state_shape"], dtype=DT[spec["state_dtype"]])
    return op, st


@pytest.mark.parametrize("spec", G.errors, ids=lambda s: str(s))
def test_error_and_shape_parity_host(spec):
    """Shape/qubit validation runs before any device work, so CPU tensors
    reach the same exception as unitair; the batch plan gives unitair's
    output shape or a RuntimeError where unitair raised one."""
    op, st = _inputs(spec)
    fn = spec["fn"]
    if "error" in spec:
        exc = EXC[spec["error"]]
        with pytest.raises(exc):
            if fn == "apply_all_qubits":
                ug.apply_all_qubits(op, st)
            else:
                n, qs, k = _validate_shapes(op, spec["qubits"], st)
                sim._check_dtypes(op, st)
                sim._BatchPlan(op, st, n, k)
    else:
        n, qs, k = _validate_shapes(op, spec["qubits"], st)
        plan = sim._BatchPlan(op, st, n, k)
        assert list(plan.out_batch) + [2 ** n] == spec["ok"]


def _validate_shapes(op, qubits, st):
    try:
        return sim._validate_apply(op, qubits, st)
    except RuntimeError as e:
        if "CUDA" not in str(e):
            raise
        return (S.count_qubits(st), list(qubits),
                S.count_qubits_gate_matrix(op))


def test_batch_plan_strides():
    st = torch.ones(3, 5, 16, dtype=torch.complex64)
    p = sim._BatchPlan(torch.ones(2, 2, dtype=torch.complex64), st, 4, 1)
    assert (p.num_states, p.in_stride, p.op_stride) == (15, 16, 0)
    p = sim._BatchPlan(torch.ones(5, 2, 2, dtype=torch.complex64), st, 4, 1)
    assert (p.num_states, p.op_stride) == (15, 4)
    assert p.ops.shape == (3, 5, 2, 2)
    p = sim._BatchPlan(torch.ones(7, 4, 4, dtype=torch.complex64),
                       torch.ones(16, dtype=torch.complex64), 4, 2)
    assert (p.out_batch, p.in_stride, p.op_stride) == ((7,), 0, 16)
    # operator batch of ones is a shared operator
    p = sim._BatchPlan(torch.ones(1, 1, 2, 2, dtype=torch.complex64), st, 4, 1)
    assert p.op_stride == 0


def test_quirk_divergence_raises():
    """unitair broadcasts an op with more batch dims than a batched state
    against qubit axes; the engine raises instead (documented)."""
    with pytest.raises(RuntimeError, match="more dimensions"):
        sim._BatchPlan(torch.ones(2, 3, 5, 2, 2, dtype=torch.complex64),
                       torch.ones(3, 5, 16, dtype=torch.complex64), 4, 1)


def test_bcast_desc_merges_contiguous_dims():
    out = (4, 3, 16)
    a = torch.ones(16)
    b = torch.ones(4, 3, 16)
    d = bcast_desc(out, broadcast_strides(a, out), broadcast_strides(b, out))
    assert d.ndim == 2
    assert list(d.shape)[:2] == [12, 16]
    assert list(d.stride_a)[:2] == [0, 1]
    assert list(d.stride_b)[:2] == [16, 1]
    d = bcast_desc(out, broadcast_strides(b, out), broadcast_strides(b, out))
    assert d.ndim == 1 and d.shape[0] == 4 * 3 * 16


def test_shape_helpers_match_reference_semantics():
    assert S.count_qubits(torch.ones(3, 32)) == 5
    with pytest.raises(S.StateShapeError):
        S.count_qubits(torch.ones(6))
    with pytest.raises(RuntimeError):
        S.count_qubits_gate_matrix(torch.ones(3, 3))
    t = S.to_tensor_layout(torch.arange(16.).reshape(2, 8))
    assert t.shape == (2, 2, 2, 2)
    assert S.to_vector_layout(t, 3).shape == (2, 8)
    assert S.get_qubit_indices([1, 0], torch.rand(500, 17, 2, 2, 2), 3) == \
        [3, 2]
    assert S.get_qubit_indices([-1, 0], torch.rand(500, 17, 2, 2, 2), 3) == \
        [-1, 2]
    x = torch.rand(4, 5, 6, 7, 8, 9)
    assert S.subset_roll_to_back(x, 2).shape == (6, 7, 8, 9, 4, 5)
    assert S.subset_roll_to_front(x, 2).shape == (8, 9, 4, 5, 6, 7)


def test_gate_builders_match_reference_values():
    import numpy as np
    np.testing.assert_allclose(ug.gates.exp_x(0.5).numpy(),
                               G["kat_expx/out"], atol=1e-7)
    t = torch.from_numpy(G["kat_expx_batch/t"])
    assert ug.gates.exp_x(t).shape == (len(t), 2, 2)
    assert ug.gates.exp_x(0.3).dtype == torch.complex64
    assert ug.gates.exp_z(torch.zeros(3, 4)).shape == (3, 4, 2, 2)
    np.testing.assert_allclose(ug.gates.rx(1.0).numpy(),
                               ug.gates.exp_x(0.5).numpy())


def test_circuit_generator_is_deterministic():
    from qcware_unitair_gb300.circuits import GATE_SET, random_circuit
    a = random_circuit(30, 1000, seed=0)
    b = random_circuit(30, 1000, seed=0)
    assert a == b
    names = {g.name for g in a}
    assert names == set(GATE_SET)
    for g in a:
        assert len(set(g.qubits)) == len(g.qubits)
        assert all(0 <= q < 30 for q in g.qubits)


def test_fuse_single_qubit_operators():
    """Per qubit, later operators multiply on the left
    (gates/matrix_algebra.py:6-51), with torch batch broadcasting."""
    from qcware_unitair_gb300.gates import fuse_single_qubit_operators
    g = torch.Generator().manual_seed(0)
    A, B, C, D = (torch.randn(2, 2, dtype=torch.complex128, generator=g)
                  for _ in range(4))
    out = fuse_single_qubit_operators([2, 4, 2, 7], [A, B, C, D])
    assert list(out) == [2, 4, 7]
    assert torch.equal(out[2], C @ A)
    assert out[4] is B and out[7] is D
    E = torch.randn(5, 2, 2, dtype=torch.complex128, generator=g)
    out = fuse_single_qubit_operators(iter([1, 1, 1]), iter([A, E, B]))
    assert out[1].shape == (5, 2, 2)
    assert torch.allclose(out[1], B @ (E @ A))
    assert fuse_single_qubit_operators([], []) == {}


def test_public_names_of_unitair_present():
    """Every name unitair exports from unitair, unitair.simulation,
    unitair.states and unitair.gates (their __init__ files) exists here."""
    from qcware_unitair_gb300 import gates as G
    sim_names = ["apply_phase", "apply_operator", "apply_to_qubits",
                 "apply_all_qubits", "act_last_qubit", "swap", "multi_cz",
                 "multi_controlled_x", "multi_controlled_z",
                 "act_first_qubits", "measure"]
    state_names = ["StateLayout", "StateShapeError", "count_qubits",
                   "count_qubits_tensor", "count_qubits_gate_matrix",
                   "hilbert_space_dim", "count_batch_dims_tensor",
                   "subset_roll_to_back", "subset_roll_to_front",
                   "to_tensor_layout", "to_vector_layout", "inner_product",
                   "norm_squared", "abs_squared", "diag_expectation_value"]
    top_names = ["states", "simulation", "StateLayout", "unit_vector",
                 "uniform_superposition", "rand_state", "count_qubits",
                 "hilbert_space_dim", "diag_expectation_value",
                 "inner_product", "norm_squared", "abs_squared",
                 "VECTOR_LAYOUT", "TENSOR_LAYOUT"]
    gate_names = ["exp_x", "exp_y", "exp_z", "cnot", "cx", "cz", "hadamard",
                  "pauli_x", "pauli_y", "pauli_z",
                  "fuse_single_qubit_operators"]
    for mod, names in ((sim, sim_names), (S, state_names), (ug, top_names),
                       (G, gate_names)):
        missing = [n for n in names if not hasattr(mod, n)]
        assert not missing, (mod.__name__, missing)


def test_tensor_layout_permutations_are_views():
    """swap_tensor, roll_qubits_tensor and permute_qubits_tensor (without
    contiguous_output) are views, as in unitair (operations.py:520-654):
    no data moves and the result aliases the input."""
    n = 4
    x = torch.arange(3 * 2 ** n, dtype=torch.float32).view(3, *(n * [2]))
    a = x.numpy()
    s = sim.swap_tensor(x, (0, 3), n)
    assert s.data_ptr() == x.data_ptr()
    assert np.array_equal(s.numpy(), np.swapaxes(a, 1, 4))
    assert np.array_equal(sim.swap_tensor(x, (1, -1), n).numpy(),
                          np.swapaxes(a, 2, 4))
    assert sim.swap_tensor(x, (2, 2), n) is x
    with pytest.raises(ValueError):
        sim.swap_tensor(x, (0, n), n)
    # psi_rolled[a_0, ..., a_{n-1}] = psi[a_k, ..., a_{n-1}, a_0, ..., a_{k-1}]
    r = sim.roll_qubits_tensor(x, n, 1)
    assert r.data_ptr() == x.data_ptr()
    idx = (1, 0, 1, 1)
    k = 1
    src = idx[k:] + idx[:k]
    assert r[(2,) + idx] == x[(2,) + src]
    assert sim.roll_qubits_tensor(x, n, n) is x
    p = sim.permute_qubits_tensor([2, 0, 3, 1], x, n)
    assert p.data_ptr() == x.data_ptr()
    assert np.array_equal(p.numpy(), np.transpose(a, (0, 3, 1, 4, 2)))


def test_tensor_layout_shape_checks():
    with pytest.raises(S.StateShapeError):
        sim._as_vector(torch.zeros(4, 3, 2), 2)
    with pytest.raises(ValueError):
        sim.act_last_qubit_tensor(torch.zeros(4, 4, dtype=torch.complex64),
                                  torch.zeros(2, 2, dtype=torch.complex64))
    with pytest.raises(ValueError):
        sim._check_gate_qubits(torch.zeros(2, 2), 2)
