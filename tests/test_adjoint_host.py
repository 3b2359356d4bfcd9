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
