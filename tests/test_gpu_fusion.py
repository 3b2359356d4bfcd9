"""Fused stages on the GPU against the complex128 oracle (tolerances as in
test_gpu_parity: 1e-5 for complex64, 1e-12 for complex128, max abs)."""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300 import states as S
from qcware_unitair_gb300.circuits import (gate_matrix, random_circuit,
                                           random_states, zero_state)
from qcware_unitair_gb300.fusion import Circuit

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def oracle_run(oracle, circ: Circuit, psi0: np.ndarray):
    gates = [(g.matrix.detach().cpu().numpy(), g.qubits) for g in circ.gates]
    return oracle.run_circuit(gates, psi0.astype(np.complex128))


def max_err(a, b):
    return float(np.abs(a.astype(np.complex128) - b).max())


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
@pytest.mark.parametrize("n,m,cmin,batch", [(10, 4, 2, 3), (12, 12, 4, 2),
                                             (14, 8, 3, 2), (16, 13, 4, 1),
                                             (5, 3, 1, 4), (2, 2, 1, 2),
                                             (18, 10, 4, 1)])
def test_fused_random_circuits(oracle, dtype, tol, n, m, cmin, batch):
    circ = Circuit.from_gates(n, random_circuit(n, 300, seed=n + m))
    psi0 = random_states(n, (batch,), dtype, seed=n)
    prog = circ.compile(dtype, DEV, tile_qubits=m, min_contiguous=cmin)
    assert prog.num_passes < len(circ)
    out = prog.run(psi0.to(DEV))
    ref = oracle_run(oracle, circ, psi0.numpy())
    assert max_err(out.cpu().numpy(), ref) <= tol
    # in place gives the same bits as out of place
    st = psi0.to(DEV).clone()
    prog.run(st, inplace=True)
    assert torch.equal(st, out)


def test_unfused_program_equals_apply_operator_loop():
    n = 11
    gates = random_circuit(n, 120, seed=5)
    circ = Circuit.from_gates(n, gates)
    psi = random_states(n, (3,), torch.complex64, seed=1).to(DEV)
    plain = circ.compile(torch.complex64, DEV, fuse=False)
    assert plain.num_passes == len(gates)
    got = plain.run(psi)
    ref = psi
    for g in gates:
        m = torch.from_numpy(g.matrix()).to(DEV, torch.complex64)
        ref = ug.apply_operator(m, g.qubits, ref)
    assert torch.equal(got, ref)


def test_controls_and_diagonals_outside_tile(oracle):
    """Tile of 3 bits on 8 qubits: CNOT/CZ/RZ with qubits outside the tile
    become per-tile conditions and factors."""
    n = 8
    circ = Circuit(n)
    rng = np.random.default_rng(3)
    for _ in range(60):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        op = int(rng.integers(5))
        if op == 0:
            circ.cnot(a, b)
        elif op == 1:
            circ.cz(a, b)
        elif op == 2:
            circ.rz(a, float(rng.uniform(0, 6.28)))
        elif op == 3:
            circ.t(b)
        else:
            circ.h(b)
    psi0 = random_states(n, (2,), torch.complex128, seed=4)
    prog = circ.compile(torch.complex128, DEV, tile_qubits=3,
                        min_contiguous=1)
    out = prog.run(psi0.to(DEV))
    assert max_err(out.cpu().numpy(), oracle_run(oracle, circ,
                                                 psi0.numpy())) < 1e-12


def test_per_state_gates(oracle):
    """Gates with a (B, d, d) batch: state b sees gate[b]."""
    n, B = 9, 5
    rng = np.random.default_rng(8)
    circ = Circuit(n)
    for layer in range(4):
        th = torch.from_numpy(rng.uniform(0, 6.28, size=(B,)))
        for q in range(n):
            circ.rx(q, th)
            circ.rz(q, th * 0.5)
        for q in range(n - 1):
            circ.cnot(q, q + 1)
    psi0 = random_states(n, (B,), torch.complex128, seed=2)
    out = circ.compile(torch.complex128, DEV, tile_qubits=6,
                       min_contiguous=2).run(psi0.to(DEV))
    ref = np.stack([
        oracle.run_circuit([((g.matrix[b] if g.matrix.dim() == 3
                              else g.matrix).numpy(), g.qubits)
                            for g in circ.gates],
                           psi0[b].numpy().astype(np.complex128))
        for b in range(B)])
    assert max_err(out.cpu().numpy(), ref) < 1e-12


def test_wide_gate_between_stages(oracle):
    n = 9
    rng = np.random.default_rng(1)
    circ = Circuit.from_gates(n, random_circuit(n, 40, seed=9))
    u = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    circ.append(torch.from_numpy(u), [4, 0, 7])
    for g in random_circuit(n, 40, seed=10):
        circ._named(g.name, list(g.qubits), g.theta)
    psi0 = random_states(n, (2,), torch.complex128, seed=3)
    prog = circ.compile(torch.complex128, DEV, tile_qubits=5,
                        min_contiguous=2)
    assert prog.num_plain == 1
    out = prog.run(psi0.to(DEV))
    assert max_err(out.cpu().numpy(), oracle_run(oracle, circ,
                                                 psi0.numpy())) < 1e-11


def test_30q_fused_matches_plain():
    """Full size: the fused program and the one-kernel-per-gate program give
    the same 30-qubit state (complex64 rounding) with >= 3x fewer passes."""
    if torch.cuda.mem_get_info()[0] < 20 * 2 ** 30:
        pytest.skip("needs 20 GiB free")
    n = 30
    circ = Circuit.from_gates(n, random_circuit(n, 300, seed=0))
    fused = circ.compile(torch.complex64, DEV)
    plain = circ.compile(torch.complex64, DEV, fuse=False)
    assert fused.num_passes * 3 <= plain.num_passes
    a = zero_state(n, (), torch.complex64, DEV)
    fused.run(a, inplace=True)
    b = zero_state(n, (), torch.complex64, DEV)
    plain.run(b, inplace=True)
    diff = float((a - b).abs().max())
    norm = float(S.norm_squared_fp64(a))
    del a, b
    torch.cuda.empty_cache()
    assert diff < 1e-5
    assert abs(norm - 1) < 1e-5


def _haar(rng, d):
    z = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
@pytest.mark.parametrize("n", [9, 12, 14])
def test_general_two_qubit_ops_in_stages(oracle, dtype, tol, n):
    """Dense 4x4 unitaries, non-SWAP/CNOT permutations and two-qubit
    diagonals inside register layouts (the run-time-indexed paths)."""
    rng = np.random.default_rng(100 + n)
    circ = Circuit(n)
    perms = [[0, 3, 1, 2], [1, 0, 3, 2], [3, 2, 1, 0], [2, 0, 3, 1]]
    for i in range(150):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        kind = i % 5
        if kind == 0:
            circ.append(_haar(rng, 4), [a, b], "dense")
        elif kind == 1:
            p = perms[int(rng.integers(len(perms)))]
            circ.append(np.eye(4)[p].astype(complex), [a, b], "dense")
        elif kind == 2:
            ph = np.exp(1j * rng.uniform(0, 2 * np.pi, 4))
            circ.append(np.diag(ph), [a, b], "diag")
        elif kind == 3:
            circ.h(a)
        else:
            circ.append(_haar(rng, 2), [a], "dense")
    psi0 = random_states(n, (2,), dtype, seed=n)
    prog = circ.compile(dtype, DEV, tile_qubits=min(n, 12))
    assert prog.num_passes < len(circ)
    out = prog.run(psi0.to(DEV))
    ref = oracle_run(oracle, circ, psi0.numpy())
    assert max_err(out.cpu().numpy(), ref) <= tol


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_x_and_swap_heavy_stages(oracle, dtype, tol, seed):
    """X and SWAP on register bits only relabel registers; every other
    operation after them (dense, controlled, permutation, diagonal) must
    see the relabelled bits."""
    rng = np.random.default_rng(seed)
    n = 10
    circ = Circuit(n)
    for _ in range(150):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        k = int(rng.integers(10))
        if k == 0:
            circ.x(a)
        elif k == 1:
            circ.swap(a, b)
        elif k == 2:
            circ.cnot(a, b)
        elif k == 3:
            circ.append(_haar(rng, 2), [a], "dense")
        elif k == 4:
            circ.append(_haar(rng, 4), [a, b], "dense")
        elif k == 5:
            circ.append(np.diag(np.exp(1j * rng.uniform(0, 6, 4))), [a, b],
                        "diag")
        elif k == 6:
            circ.append(gate_matrix("RZ", float(rng.uniform(0, 6))), [a],
                        "diag")
        elif k == 7:
            circ.h(a)
        elif k == 8:
            circ.y(a)
        else:
            circ.append(np.eye(4)[[1, 3, 0, 2]].astype(complex), [a, b],
                        "dense")
    psi0 = random_states(n, (2,), dtype, seed=seed)
    prog = circ.compile(dtype, DEV, tile_qubits=10)
    out = prog.run(psi0.to(DEV))
    ref = oracle_run(oracle, circ, psi0.numpy())
    assert max_err(out.cpu().numpy(), ref) <= tol


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
def test_single_qubit_runs_merged(oracle, dtype, tol):
    """Runs of single-qubit gates on one register bit (per-state rotations,
    a diagonal, shared gates) are multiplied into one 2x2 per state."""
    rng = np.random.default_rng(7)
    n, B = 11, 3
    circ = Circuit(n)
    for _ in range(2):
        for q in range(n):
            for name in ("RX", "RY", "RZ"):
                th = rng.uniform(0, 2 * np.pi, B)
                mats = np.stack([gate_matrix(name, float(t)) for t in th])
                circ.append(mats, [q], "diag" if name == "RZ" else "dense")
            circ.t(q)
            circ.h(q)
        for q in range(n - 1):
            circ.cnot(q, q + 1)
    psi0 = random_states(n, (B,), dtype, seed=1)
    prog = circ.compile(dtype, DEV, tile_qubits=11)
    out = prog.run(psi0.to(DEV))
    psi = psi0.numpy().astype(np.complex128)
    for g in circ.gates:
        psi = oracle.apply_operator(g.matrix.detach().cpu().numpy(),
                                    list(g.qubits), psi)
    assert max_err(out.cpu().numpy(), psi) <= tol


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
def test_stage_beyond_resident_limits(oracle, dtype, tol):
    """A stage with more operations than stay resident per CTA (chunked
    decode) and one with more layouts than the per-CTA table (per-layout
    rebuild), both against the oracle."""
    rng = np.random.default_rng(11)
    n = 10
    many_ops = Circuit(n)
    for i in range(150):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        if i % 3 == 0:
            many_ops.append(gate_matrix("RZ", float(rng.uniform(0, 6))), [a],
                            "diag")
        elif i % 3 == 1:
            many_ops.cz(a, b)
        else:
            many_ops.t(a)
    many_ops.h(9)
    many_ops.h(8)
    many_layouts = Circuit(n)
    for _ in range(120):
        many_layouts.h(int(rng.integers(2, n)))
    for circ in (many_ops, many_layouts):
        psi0 = random_states(n, (2,), dtype, seed=4)
        prog = circ.compile(dtype, DEV, tile_qubits=8)
        out = prog.run(psi0.to(DEV))
        ref = oracle_run(oracle, circ, psi0.numpy())
        assert max_err(out.cpu().numpy(), ref) <= tol


def test_program_with_wide_gate_in_place(oracle):
    """A 6-qubit gate between stages of an in-place program."""
    rng = np.random.default_rng(8)
    n = 10
    circ = Circuit(n)
    for q in range(n):
        circ.h(q)
    circ.append(_haar(rng, 64), [0, 3, 4, 6, 8, 9], "dense")
    for q in range(n):
        circ.t(q)
    psi0 = random_states(n, (2,), torch.complex64, seed=8)
    st = psi0.to(DEV).clone()
    circ.compile(torch.complex64, DEV).run(st, inplace=True)
    ref = oracle_run(oracle, circ, psi0.numpy())
    assert max_err(st.cpu().numpy(), ref) <= 1e-5
