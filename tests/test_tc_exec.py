"""Tensor-core stage programs executed on the CPU from their records.

A tensor-core stage is described by its tile positions, one 64-byte record
per block (swizzled shared-memory offsets of the register and thread bits,
the image index, the post-diagonals) and the fp16 block images.  This test
runs exactly what the kernel is given: the tile in swizzled order, each
block's 128 x 32 gather through the XOR offset tables, the real 64 x 64
matrix the image stands for, the post-diagonals from thread, register and
outside bits, and the scatter back.  The result must match the complex128
oracle running the circuit gate by gate, for random circuits, wide gates,
all-diagonal circuits and batches; a corrupted record must be caught.  The
GPU tests check that the kernel executes the same records.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from qcware_unitair_gb300 import tcplan
from qcware_unitair_gb300.circuits import random_circuit
from qcware_unitair_gb300.fusion import Circuit
from qcware_unitair_gb300.tcplan import BLOCK_DTYPE, DIAG_DTYPE, tc_swz

SWZ = np.array([tc_swz(l) for l in range(4096)])


def _apply_plain(psi, mat, qubits, n):
    return O.apply_operator_numpy(mat, list(qubits), psi)


def run_tc_records(prog, psi, blocks=None):
    """psi (B, 2^n) complex128 -> the program's result, from its records."""
    n = prog.n
    blocks_l, diags_l, images_l, factors_l = prog.tc_records
    factors = np.concatenate(factors_l) if factors_l else np.zeros(0)
    blocks = np.stack(blocks_l) if blocks is None else blocks
    diags = np.stack(diags_l) if diags_l else np.zeros(0, DIAG_DTYPE)
    psi = psi.copy()
    Bn = psi.shape[0]
    r = np.arange(128)
    i = np.arange(32)
    for op in prog.ops:
        if op[0] == "plain":
            psi = _apply_plain(psi, op[1].cpu().numpy().astype(np.complex128),
                               op[2], n)
            continue
        _, c, positions, first, count = op
        order = list(positions)
        # state axes: axis a <-> position n-1-a; tile local bit b <->
        # position order[b]; outside positions first (ascending), then the
        # tile bits from local bit 11 down to 0
        outside = sorted(set(range(n)) - set(order))
        axes = [n - 1 - p for p in reversed(outside)] + \
            [n - 1 - order[b] for b in range(11, -1, -1)]
        t = psi.reshape((Bn,) + (2,) * n).transpose([0] + [1 + a for a in axes])
        T = t.reshape(Bn, 2 ** (n - 12), 4096)
        S = np.empty_like(T)
        S[..., SWZ] = T
        # outside-position bits of each tile: tile index bit j <-> outside[j]
        tiles = np.arange(2 ** (n - 12))
        for blk in blocks[first:first + count]:
            sb = np.zeros(128, dtype=np.int64)
            for j in range(7):
                sb ^= np.where((r >> j) & 1, int(blk["tspo"][j]), 0)
            ro = np.zeros(32, dtype=np.int64)
            for k in range(5):
                ro ^= np.where((i >> k) & 1, int(blk["rspo"][k]), 0)
            addr = sb[:, None] ^ ro[None, :]                 # (128, 32)
            assert sorted(addr.reshape(-1)) == list(range(4096))
            A = S[:, :, addr]                                 # (B, t, 128, 32)
            Bm = tcplan.image_matrix(images_l[int(blk["mat"])])
            Ar = np.stack([A.real, A.imag], -1).reshape(A.shape[:-1] + (64,))
            Y = Ar @ Bm
            Y = Y[..., 0::2] + 1j * Y[..., 1::2]
            fac = int(blk["fac"])
            if fac >= 0:  # per-thread factor table, indexed by outside bits
                p = np.zeros(len(tiles), dtype=np.int64)
                for k in range(int(blk["nout"])):
                    pos = int(blk["opos"][k])
                    p |= ((tiles >> outside.index(pos)) & 1) << k
                f = factors[fac + p[:, None] * 128 + r[None, :]]
                Y = Y * f[None, :, :, None]
            f0, nd = int(blk["first_diag"]), int(blk["num_diag"])
            for dg in diags[f0:f0 + nd]:
                idx = np.zeros((len(tiles), 128, 32), dtype=np.int64)
                for u in range(int(dg["nq"])):
                    en = int(dg["enc"][u])
                    if en < 0:
                        p = -1 - en
                        bit = (tiles >> outside.index(p)) & 1
                        bit = bit[:, None, None]
                    elif en < 5:
                        bit = ((i >> en) & 1)[None, None, :]
                    else:
                        bit = ((r >> (en - 5)) & 1)[None, :, None]
                    idx = (idx << 1) | bit
                d = dg["d"].astype(np.float64)
                vals = d[0::2] + 1j * d[1::2]
                Y = Y * vals[idx][None]
            S[:, :, addr] = Y
        T = S[..., SWZ]
        inv = np.argsort([0] + [1 + a for a in axes])
        psi = T.reshape((Bn,) + (2,) * n).transpose(inv).reshape(Bn, 2 ** n)
    return psi


def _oracle(gates, psi0):
    return O.run_circuit([(g.matrix(), g.qubits) for g in gates], psi0)


def _states(n, batch, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(batch, 2 ** n)) + 1j * rng.normal(size=(batch, 2 ** n))
    return x / np.linalg.norm(x, axis=1, keepdims=True)


@pytest.mark.parametrize("n,depth,seed", [(12, 150, 0), (13, 200, 1),
                                          (14, 200, 2), (15, 120, 3)])
def test_tc_records_random_circuits(n, depth, seed):
    gates = random_circuit(n, depth, seed=seed)
    prog = Circuit.from_gates(n, gates).compile(device="cpu")
    assert prog.tensor_cores and prog.num_stages >= 1
    psi0 = _states(n, 2, seed)
    got = run_tc_records(prog, psi0)
    want = _oracle(gates, psi0)
    assert np.abs(got - want).max() < 2e-6


def test_tc_records_wide_and_diagonal_gates():
    """3- and 4-qubit dense operators join blocks; long runs of diagonals
    on qubits outside the tile become post-diagonals."""
    n = 14
    rng = np.random.default_rng(7)
    circ = Circuit(n)
    ref = []
    for step in range(60):
        k = int(rng.integers(1, 5))
        qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
        if step % 3 == 0:
            ph = np.exp(1j * rng.uniform(0, 2 * np.pi, size=2 ** min(k, 2)))
            m = np.diag(ph)
            qs = qs[:min(k, 2)]
        else:
            a = rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(
                size=(2 ** k, 2 ** k))
            m, _ = np.linalg.qr(a)
        circ.append(torch.from_numpy(m), qs)
        ref.append((m, qs))
    prog = circ.compile(device="cpu", tensor_cores=True)
    psi0 = _states(n, 3, 5)
    got = run_tc_records(prog, psi0)
    want = O.run_circuit(ref, psi0)
    assert np.abs(got - want).max() < 2e-6


def test_tc_records_all_diagonal_circuit():
    n = 13
    circ = Circuit(n)
    rng = np.random.default_rng(3)
    ref = []
    for _ in range(40):
        q = int(rng.integers(0, n))
        circ.rz(q, float(rng.uniform(0, 6)))
        ref.append((circ.gates[-1].matrix.numpy(), [q]))
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        circ.cz(a, b)
        ref.append((circ.gates[-1].matrix.numpy(), [a, b]))
    prog = circ.compile(device="cpu", tensor_cores=True)
    psi0 = _states(n, 1, 9)
    got = run_tc_records(prog, psi0)
    assert np.abs(got - O.run_circuit(ref, psi0)).max() < 2e-6


def test_tc_image_split_is_exact_integer_plus_residual():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    U, _ = np.linalg.qr(a)
    img = tcplan.block_image(U)
    bh = img[tcplan._IMG_IDX[64:]].astype(np.float64)
    assert np.all(bh == np.rint(bh)) and np.abs(bh).max() <= 1024
    # column L1 norms of the real form stay within the exactness bound
    B = tcplan.image_matrix(img)
    assert np.abs(B).sum(axis=0).max() <= 8.0 + 1e-9
    Ur = np.empty((64, 64))
    Ur[0::2, 0::2] = U.real.T
    Ur[1::2, 0::2] = -U.imag.T
    Ur[0::2, 1::2] = U.imag.T
    Ur[1::2, 1::2] = U.real.T
    assert np.abs(B - Ur).max() < 2 ** -21


def test_tc_corrupted_record_is_caught():
    n = 13
    gates = random_circuit(n, 80, seed=11)
    prog = Circuit.from_gates(n, gates).compile(device="cpu")
    psi0 = _states(n, 1, 1)
    want = _oracle(gates, psi0)
    blocks = np.stack(prog.tc_records[0]).copy()
    assert np.abs(run_tc_records(prog, psi0, blocks) - want).max() < 2e-6
    blocks[0]["rspo"][[0, 1]] = blocks[0]["rspo"][[1, 0]]
    assert np.abs(run_tc_records(prog, psi0, blocks) - want).max() > 1e-3


def test_tc_plan_thread_bits_cover_banks():
    """Every block's lowest lane bits hit distinct shared-memory banks:
    16 lanes (8-byte accesses) or 8 lanes (16-byte pair accesses)."""
    n = 20
    gates = random_circuit(n, 400, seed=4)
    prog = Circuit.from_gates(n, gates).compile(device="cpu")
    for blk in prog.tc_records[0]:
        pairs = int(blk["flags"]) & tcplan.TC_PAIRS
        lanes = 8 if pairs else 16
        addr = np.zeros(lanes, dtype=np.int64)
        r = np.arange(lanes)
        for j in range(7):
            addr ^= np.where((r >> j) & 1, int(blk["tspo"][j]), 0)
        unit = (addr >> 1) & 7 if pairs else addr & 15
        # a few blocks cannot avoid a 2-way conflict (all free bits in one
        # bank class); none may do worse
        assert len(set(unit.tolist())) >= lanes // 2
