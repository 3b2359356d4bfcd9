"""complex128 gates in both arithmetic modes against the complex128 oracle:

* "pairs" (double-float pairs on the FP32 pipe, the default): every gate
  kind within 1e-13 of the oracle per gate (a few 2^-47 relative);
* "fp64" (native FP64): within 1e-15;
* the kinds without arithmetic (permutations, entries 0, +-1, +-i) give the
  same bits in both modes;
* amplitudes or entries outside the pair range ([2^-40, 2^60]) fall back to
  FP64 per thread and keep their relative accuracy.
"""
import math

import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300.circuits import gate_matrix

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


@pytest.fixture
def arith():
    prev = ug.complex128_arithmetic()
    yield ug.set_complex128_arithmetic
    ug.set_complex128_arithmetic(prev)


def _state(n, batch, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=(batch, 2 ** n)) + 1j * rng.normal(size=(batch,
                                                                  2 ** n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    return psi * scale


def _unitary(k, seed):
    rng = np.random.default_rng(seed)
    d = 2 ** k
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d,
                                                                       d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _ctrl(u):
    m = np.eye(4, dtype=np.complex128)
    m[2:, 2:] = u
    return m


def _apply_ref(oracle, m, qubits, psi):
    return oracle.run_circuit([(m, tuple(qubits))], psi)


OPS_1Q = {
    "X": gate_matrix("X"), "Y": gate_matrix("Y"), "Z": gate_matrix("Z"),
    "S": gate_matrix("S"), "H": gate_matrix("H"), "T": gate_matrix("T"),
    "RX": gate_matrix("RX", 0.7), "RY": gate_matrix("RY", 1.1),
    "RZ": gate_matrix("RZ", 0.3), "U": _unitary(1, 5),
    "iX": 1j * gate_matrix("X"), "diag_real": np.diag([0.6, -0.8]) + 0j,
    "diag_imag": np.diag([0.6j, -0.8j]),
    "anti_full": np.array([[0, np.exp(0.3j)], [np.exp(-1.2j), 0]]),
}
OPS_2Q = {
    "CNOT": gate_matrix("CNOT"), "CZ": gate_matrix("CZ"),
    "SWAP": gate_matrix("SWAP"), "U4": _unitary(2, 7),
    "CRY": _ctrl(gate_matrix("RY", 0.9)), "CU": _ctrl(_unitary(1, 8)),
    "diag4": np.diag(np.exp(1j * np.array([0.1, 0.2, -0.4, 1.3]))),
    "perm_iswap": np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0],
                            [0, 0, 0, 1]]),
}
EXACT = {"X", "Y", "Z", "S", "iX", "CNOT", "CZ", "SWAP", "perm_iswap"}


def _run(m, qubits, psi):
    out = ug.apply_operator(torch.from_numpy(m).to(DEV), list(qubits),
                            torch.from_numpy(psi).to(DEV))
    return out.cpu().numpy()


@pytest.mark.parametrize("mode,tol", [("pairs", 1e-13), ("fp64", 1e-15)])
@pytest.mark.parametrize("name", sorted(OPS_1Q))
@pytest.mark.parametrize("q", [0, 5, 9, 10])
def test_one_qubit_kinds(oracle, arith, mode, tol, name, q):
    arith(mode)
    n = 11
    psi = _state(n, 2, seed=q)
    got = _run(OPS_1Q[name], [q], psi)
    ref = _apply_ref(oracle, OPS_1Q[name], [q], psi)
    assert float(np.abs(got - ref).max()) <= tol


@pytest.mark.parametrize("mode,tol", [("pairs", 1e-13), ("fp64", 1e-15)])
@pytest.mark.parametrize("name", sorted(OPS_2Q))
@pytest.mark.parametrize("qubits", [(0, 7), (3, 10), (10, 9), (9, 2)])
def test_two_qubit_kinds(oracle, arith, mode, tol, name, qubits):
    arith(mode)
    n = 11
    psi = _state(n, 2, seed=sum(qubits))
    got = _run(OPS_2Q[name], qubits, psi)
    ref = _apply_ref(oracle, OPS_2Q[name], qubits, psi)
    assert float(np.abs(got - ref).max()) <= tol


@pytest.mark.parametrize("name", sorted(EXACT))
def test_exact_kinds_same_bits_in_both_modes(arith, name):
    m = OPS_1Q.get(name, OPS_2Q.get(name))
    qubits = [4] if m.shape[0] == 2 else [1, 8]
    psi = _state(10, 3, seed=11)
    arith("pairs")
    a = _run(m, qubits, psi)
    arith("fp64")
    b = _run(m, qubits, psi)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)) or \
        np.array_equal(a, b)


@pytest.mark.parametrize("scale", [1e-30, 2.0 ** -45, 1e25, 1e100, 1e-200])
@pytest.mark.parametrize("name", ["H", "RX", "U"])
def test_out_of_pair_range_states_fall_back(oracle, arith, scale, name):
    """Amplitudes far outside [2^-40, 2^60] take FP64 in their thread:
    the relative error stays at the FP64 level."""
    arith("pairs")
    psi = _state(10, 1, seed=3, scale=scale)
    got = _run(OPS_1Q[name], [6], psi)
    ref = _apply_ref(oracle, OPS_1Q[name], [6], psi)
    assert float(np.abs(got - ref).max()) <= 1e-15 * scale


def test_mixed_range_state(oracle, arith):
    """One state whose first half is tiny: threads over the tiny half fall
    back, the rest run in pairs; the result is accurate everywhere
    relative to each half's own scale."""
    arith("pairs")
    n = 12
    psi = _state(n, 1, seed=4)
    psi[:, : 2 ** (n - 1)] *= 1e-20
    m = OPS_1Q["U"]
    got = _run(m, [11], psi)
    ref = _apply_ref(oracle, m, [11], psi)
    half = 2 ** (n - 1)
    assert float(np.abs(got[:, :half] - ref[:, :half]).max()) <= 1e-35
    assert float(np.abs(got[:, half:] - ref[:, half:]).max()) <= 1e-13


@pytest.mark.parametrize("entry_scale", [1e-20, 1e30])
def test_out_of_range_operator_falls_back(oracle, arith, entry_scale):
    arith("pairs")
    m = OPS_1Q["U"] * entry_scale
    psi = _state(9, 2, seed=5)
    got = _run(m, [3], psi)
    ref = _apply_ref(oracle, m, [3], psi)
    assert float(np.abs(got - ref).max()) <= 1e-15 * entry_scale


def test_zero_state_and_zero_entries(arith):
    arith("pairs")
    psi = np.zeros((1, 2 ** 9), dtype=np.complex128)
    psi[0, 5] = 1.0
    m = np.array([[0.6, 0.0], [0.0, 0.8j]])  # real and imaginary diagonal
    got = _run(m, [8], psi)
    want = psi.copy()
    want[0, 5] = 0.8j  # index 5 has bit 0 (qubit 8) set
    # zeros stay exactly zero; 0.8 carries the pairs' few 2^-47
    assert np.count_nonzero(got) == 1
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-15)


@pytest.mark.parametrize("mode", ["pairs", "fp64"])
def test_deep_circuit_norm_drift(arith, mode):
    """2,000 gates alternating H and RY(pi/3) on one qubit: repeated real
    entries are the form in which a systematically biased product would
    drift the norm fastest."""
    arith(mode)
    n = 12
    psi = torch.from_numpy(_state(n, 1, seed=9)).to(DEV)
    h = torch.from_numpy(gate_matrix("H")).to(DEV)
    ry = torch.from_numpy(gate_matrix("RY", math.pi / 3)).to(DEV)
    for _ in range(1000):
        psi = ug.apply_operator(h, [3], psi)
        psi = ug.apply_operator(ry, [3], psi)
    drift = float((ug.states.norm_squared_fp64(psi) - 1).abs().max())
    assert drift <= 1e-12


def test_mode_round_trip(arith):
    arith("fp64")
    assert ug.complex128_arithmetic() == "fp64"
    arith("pairs")
    assert ug.complex128_arithmetic() == "pairs"
    with pytest.raises(ValueError):
        ug.set_complex128_arithmetic("fp32")


@pytest.mark.parametrize("mode", ["pairs", "fp64"])
def test_fused_circuit_in_both_modes(oracle, arith, mode):
    """1,000 random gates through fused register stages (14 qubits, two
    states): within 1e-12 of the oracle and the norm within 1e-12."""
    from qcware_unitair_gb300 import states as S
    from qcware_unitair_gb300.circuits import random_circuit, random_states
    from qcware_unitair_gb300.fusion import Circuit
    arith(mode)
    n = 14
    gates = random_circuit(n, 1000, seed=7)
    prog = Circuit.from_gates(n, gates).compile(torch.complex128, DEV)
    psi0 = random_states(n, (2,), torch.complex128, seed=7)
    out = prog.run(psi0.to(DEV))
    ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in gates],
                             psi0.numpy())
    err = float(np.abs(out.cpu().numpy() - ref).max())
    drift = float((S.norm_squared_fp64(out) - 1).abs().max())
    print(f"{mode}: passes={prog.num_passes} max|err| {err:.2e} "
          f"drift {drift:.2e}")
    assert err <= 1e-12
    assert drift <= 1e-12


def test_fused_pairs_match_fp64(arith):
    """The same fused program in both modes agrees to pair precision."""
    from qcware_unitair_gb300.circuits import random_circuit, random_states
    from qcware_unitair_gb300.fusion import Circuit
    n = 16
    gates = random_circuit(n, 300, seed=8)
    prog = Circuit.from_gates(n, gates).compile(torch.complex128, DEV)
    psi0 = random_states(n, (1,), torch.complex128, seed=8).to(DEV)
    arith("pairs")
    a = prog.run(psi0).cpu().numpy()
    arith("fp64")
    b = prog.run(psi0).cpu().numpy()
    assert float(np.abs(a - b).max()) <= 1e-13


@pytest.mark.parametrize("mode", ["pairs", "fp64"])
@pytest.mark.parametrize("name,qubits", [("U", [2]), ("H", [7]),
                                         ("U4", [1, 6]), ("CRY", [7, 0])])
def test_in_place_matches_functional(arith, mode, name, qubits):
    """apply_operator_ (in place, the streaming kernel reading and writing
    one buffer) gives the same bits as the functional form."""
    arith(mode)
    m = OPS_1Q.get(name, OPS_2Q.get(name))
    psi = torch.from_numpy(_state(9, 3, seed=13)).to(DEV)
    op = torch.from_numpy(m).to(DEV)
    want = ug.apply_operator(op, qubits, psi)
    got = psi.clone()
    ug.apply_operator_(op, qubits, got)
    assert torch.equal(got, want)


@pytest.mark.parametrize("n", [7, 8])
@pytest.mark.parametrize("name", ["U", "H", "U4", "SWAP"])
def test_smallest_streamed_states(oracle, arith, n, name):
    """n = 7 is one warp step per state; every target position."""
    arith("pairs")
    m = OPS_1Q.get(name, OPS_2Q.get(name))
    k = int(np.log2(m.shape[0]))
    psi = _state(n, 2, seed=n)
    for q0 in range(n):
        qubits = [q0] if k == 1 else [q0, (q0 + 3) % n]
        got = _run(m, qubits, psi)
        ref = _apply_ref(oracle, m, qubits, psi)
        assert float(np.abs(got - ref).max()) <= 1e-13


def test_monomial_with_phases(oracle, arith):
    """A permutation matrix whose entries are arbitrary phases: the
    permutation is exact, the phases go through the pairs."""
    ph = np.exp(1j * np.array([0.3, -1.1, 2.0, 0.7]))
    m = np.zeros((4, 4), dtype=np.complex128)
    for r, c in enumerate([2, 0, 3, 1]):
        m[r, c] = ph[r]
    for mode, tol in (("pairs", 1e-13), ("fp64", 1e-15)):
        arith(mode)
        psi = _state(10, 2, seed=5)
        got = _run(m, [4, 8], psi)
        ref = _apply_ref(oracle, m, [4, 8], psi)
        assert float(np.abs(got - ref).max()) <= tol


@pytest.mark.parametrize("mode,tol", [("pairs", 1e-13), ("fp64", 1e-15)])
@pytest.mark.parametrize("k,qubits", [(3, [0, 5, 9]), (3, [10, 2, 7]),
                                      (4, [1, 4, 8, 10]), (4, [9, 0, 6, 3])])
def test_three_and_four_qubit_operators(oracle, arith, mode, tol, k,
                                        qubits):
    """The group kernel: one group per thread, each output a compensated
    dot product of pairs (df_rowD)."""
    arith(mode)
    m = _unitary(k, 30 + k)
    psi = _state(11, 2, seed=k)
    got = _run(m, qubits, psi)
    ref = _apply_ref(oracle, m, qubits, psi)
    assert float(np.abs(got - ref).max()) <= tol


@pytest.mark.parametrize("mode,tol", [("pairs", 2e-14), ("fp64", 1e-15)])
@pytest.mark.parametrize("scale", [1.0, 100.0, 1e5])
def test_apply_phase_double_angles(arith, mode, tol, scale):
    """apply_phase with float64 angles: the phase factor in pairs
    (df_sincos: Cody-Waite reduction, Taylor series) or FP64, against
    numpy's exp(-1j * angles) * state in complex128."""
    arith(mode)
    n = 12
    rng = np.random.default_rng(int(scale))
    ang = rng.uniform(-scale, scale, size=(2, 2 ** n))
    ang[0, :64] = np.arange(-32, 32) * (np.pi / 2)  # exact-cancellation cases
    ang[1, :8] = [0.0, 1e-300, -1e-12, 2.0 ** 19, 3e6, -3e6, np.pi, 1e-40]
    psi = _state(n, 2, seed=3)
    got = ug.apply_phase(torch.from_numpy(ang).to(DEV),
                         torch.from_numpy(psi).to(DEV)).cpu().numpy()
    want = np.exp(-1j * ang) * psi
    assert float(np.abs(got - want).max()) <= tol * np.abs(psi).max() * 100


def test_apply_phase_double_angles_on_complex64(arith):
    """float64 angles on a complex64 state: complex128 output, the phase
    in pairs."""
    arith("pairs")
    n = 10
    rng = np.random.default_rng(4)
    ang = rng.uniform(-10, 10, size=2 ** n)
    psi = _state(n, 1, seed=4).astype(np.complex64)
    got = ug.apply_phase(torch.from_numpy(ang).to(DEV),
                         torch.from_numpy(psi).to(DEV))
    assert got.dtype == torch.complex128
    want = np.exp(-1j * ang) * psi.astype(np.complex128)
    assert float(np.abs(got.cpu().numpy() - want).max()) <= 1e-15
