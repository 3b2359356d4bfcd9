"""Host-side pieces of the adjoint API on CPU: Pauli term encoding,
checkpoint segments and the ansatz layout."""
import numpy as np
import pytest

from qcware_unitair_gb300.adjoint import (ParamCircuit, PauliSum,
                                          hardware_efficient_ansatz)


def test_pauli_term_encoding():
    H = PauliSum(3).z(0).xx(0, 1, 0.5).add(0.3, {2: "Y"})
    t = H.term_array()
    # qubit q is bit n-1-q
    assert (int(t[0]["x"]), int(t[0]["z"])) == (0, 4)
    assert (int(t[1]["x"]), int(t[1]["z"])) == (6, 0)
    assert (int(t[2]["x"]), int(t[2]["z"])) == (1, 1)
    assert t[2]["re"] == 0 and t[2]["im"] == pytest.approx(0.3)  # c * i


def test_pauli_dense_is_hermitian_sum():
    H = PauliSum(2).z(0).xx(0, 1, 0.5).add(2.0, {1: "Y"})
    D = H.dense()
    assert np.allclose(D, D.conj().T)
    z0 = np.kron(np.diag([1, -1]), np.eye(2))
    assert np.allclose(np.diag(D).real, np.diag(z0))


def test_checkpoint_segments_every_sqrt_layers():
    pc = hardware_efficient_ansatz(20, 12)
    assert len(pc.ops) == 12 * (40 + 20)
    segs = pc.segments()
    assert segs == [(0, 240), (240, 480), (480, 720)]  # every 4 layers
    flat = ParamCircuit(3, 1)
    for _ in range(10):
        flat.rx(0, 0)
    s = flat.segments()
    assert s[0] == (0, 4) and s[-1][1] == 10


def test_param_validation():
    pc = ParamCircuit(2, 3)
    with pytest.raises(ValueError):
        pc.rx(0, 3)
    with pytest.raises(ValueError):
        pc.ry(2, 0)
    with pytest.raises(ValueError):
        PauliSum(2).add(1.0, {0: "Q"})


def _cmp_backward_plans(pc, m, dtype):
    """The backward-stage plan built by the C++ planner equals the one the
    Python planner builds: same stage order, bit positions, adjoint
    operation records, fixed-gate records, matrices and parameter slots."""
    import torch
    from qcware_unitair_gb300.adjoint import (_adjop_dtype, _plan_backward,
                                              _plan_backward_native)
    cpu = torch.device("cpu")
    A = _plan_backward(pc, 0, len(pc.ops), dtype, cpu, m)
    B = _plan_backward_native(pc, 0, len(pc.ops), dtype, cpu, m)
    assert len(A) == len(B)
    AD = _adjop_dtype()
    for (ka, ea), (kb, eb) in zip(A, B):
        assert ka == kb
        if ka != "stage":
            assert ea is eb or ea == eb
            continue
        assert ea["c"] == eb["c"]
        assert list(ea["positions"]) == list(eb["positions"])
        xa, xb = ea["ops"].numpy().view(AD), eb["ops"].numpy().view(AD)
        for f in ("kind", "gen", "bit", "slot", "pidx", "scale"):
            assert np.array_equal(xa[f], xb[f]), f
        fixed = xa["kind"] == 1
        ga, gb = xa["g"][fixed], xb["g"][fixed]
        for f in ("kind", "nq", "b0", "b1", "cmask", "cval", "mat_bstride"):
            assert np.array_equal(ga[f], gb[f]), f
        pa, pb = ea["pool"].numpy(), eb["pool"].numpy()
        for ia, ib in zip(ga, gb):
            k = (16 if ia["kind"] == 1 else
                 (1 << ia["nq"] if ia["kind"] == 2 else 4))
            assert np.array_equal(pa[ia["mat"]:ia["mat"] + k],
                                  pb[ib["mat"]:ib["mat"] + k])
        assert torch.equal(ea["slot_param"], eb["slot_param"])
        assert torch.equal(ea["slot_scale"], eb["slot_scale"])


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_native_backward_plan_matches_python(dtype):
    import torch
    from qcware_unitair_gb300 import serve as S
    dt = getattr(torch, dtype)
    for n, layers in ((8, 3), (20, 4)):
        _cmp_backward_plans(hardware_efficient_ansatz(n, layers),
                            min(12, n), dt)
    for req in S.make_trace(6, rate=100.0, seed=0, qubits=(10, 20),
                            depth=(50, 300)):
        pc, _, _ = S._grad_circuit(req)
        _cmp_backward_plans(pc, min(12, req.num_qubits), dt)
