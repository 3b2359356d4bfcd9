"""Fused programs executed on the CPU from their records.

A compiled Program holds, per stage, the tile's state bit positions and a
list of gate records (kind, bits, condition, matrix offset); with register
layouts, each layout names the tile bits its register bits stand for.  This
test decodes every record back into a matrix on state bit positions (plus
its condition) and applies it with numpy, then compares the result with the
complex128 oracle running the circuit gate by gate.  It checks on the CPU
that both planners (Python and C++) encode the circuit faithfully: the
gate order, bit mapping, control conditions and matrix values.  The GPU
tests check that the kernels execute the same records.
"""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300.circuits import random_circuit
from qcware_unitair_gb300.fusion import (FG_DTYPE, LAYOUT_DTYPE, Circuit,
                                         FG_ANTI1, FG_CANTI1, FG_CDENSE1,
                                         FG_DENSE1, FG_DENSE2, FG_DIAG,
                                         FG_PERM2, FG_RDIAG, FG_REAL1)


def _apply(psi, mat, pos, n, cmask=0, cval=0):
    """mat (d x d, matrix index bit k-1-j <-> state bit pos[j]) on every
    state of psi (B, 2^n), where (index & cmask) == cval."""
    k = len(pos)
    idx = np.arange(2 ** n)
    tmask = sum(1 << p for p in pos)
    base = idx[(idx & tmask) == 0]
    base = base[(base & cmask) == cval]
    offs = [sum(((r >> (k - 1 - j)) & 1) << pos[j] for j in range(k))
            for r in range(2 ** k)]
    group = base[:, None] + np.array(offs)[None, :]      # (G, d)
    vals = psi[:, group]                                  # (B, G, d)
    psi[:, group] = np.einsum("rc,bgc->bgr", mat, vals)


def _run_records(prog, psi):
    n, rb = prog.n, prog.rb
    raw = prog.gate_records.cpu().numpy()  # a placeholder when empty
    recs = raw[:raw.size - raw.size % FG_DTYPE.itemsize].view(FG_DTYPE)
    lays = (prog.layout_records.cpu().numpy().view(LAYOUT_DTYPE)
            if prog.num_layouts else None)
    pool = prog.pool.cpu().numpy().astype(np.complex128)

    def values(r, count):
        return pool[int(r["mat"]):int(r["mat"]) + count]

    for op in prog.ops:
        if op[0] == "plain":
            mat = op[1].cpu().numpy().astype(np.complex128)
            _apply(psi, mat, [n - 1 - q for q in op[2]], n)
            continue
        positions = list(op[2])
        if op[0] == "stage":  # shared-memory stage: bits are tile bits
            for r in recs[op[3]:op[3] + op[4]]:
                def tp(b):
                    return positions[b] if b >= 0 else -1 - b
                kind = int(r["kind"])
                cm, cv = int(r["cmask"]), int(r["cval"])
                if kind == FG_DIAG:
                    nq = int(r["nq"])
                    ps = [tp(int(r["b0"]))] + (
                        [tp(int(r["b1"]))] if nq == 2 else [])
                    _apply(psi, np.diag(values(r, 2 ** nq)), ps, n)
                elif kind == FG_DENSE1:
                    _apply(psi, values(r, 4).reshape(2, 2),
                           [tp(int(r["b0"]))], n, cm, cv)
                else:
                    assert kind == FG_DENSE2
                    _apply(psi, values(r, 16).reshape(4, 4),
                           [tp(int(r["b0"])), tp(int(r["b1"]))], n, cm, cv)
            continue
        assert op[0] == "layouts"
        for li in range(op[3], op[3] + op[4]):
            lay = lays[li]
            rbits = [int(b) for b in lay["rb"][:rb]]

            def reg(k):
                return positions[rbits[k]]

            def enc(e):  # register bit, thread (tile) bit, or outside
                if e < 0:
                    return -1 - e
                return reg(e) if e < rb else positions[e - rb]

            first, count = int(lay["first_gate"]), int(lay["num_gates"])
            for r in recs[first:first + count]:
                kind = int(r["kind"])
                cm, cv = int(r["cmask"]), int(r["cval"])
                if kind in (FG_DENSE1, FG_REAL1, FG_ANTI1):
                    _apply(psi, values(r, 4).reshape(2, 2),
                           [reg(int(r["b0"]))], n, cm, cv)
                elif kind in (FG_CDENSE1, FG_CANTI1):
                    c = 1 << positions[int(r["b1"])]
                    _apply(psi, values(r, 4).reshape(2, 2),
                           [reg(int(r["b0"]))], n, cm | c, cv | c)
                elif kind in (FG_DENSE2, FG_PERM2):
                    _apply(psi, values(r, 16).reshape(4, 4),
                           [reg(int(r["b0"])), reg(int(r["b1"]))], n, cm, cv)
                else:
                    assert kind == FG_RDIAG, kind
                    nq = int(r["nq"])
                    ps = [enc(int(r["b0"]))] + (
                        [enc(int(r["b1"]))] if nq == 2 else [])
                    _apply(psi, np.diag(values(r, 2 ** nq)), ps, n)
    return psi


@pytest.mark.parametrize("native", [True, False])
@pytest.mark.parametrize("layouts", [True, False])
@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("n,m,gates", [(8, 6, 120), (10, 7, 200),
                                        (9, 5, 150)])
def test_records_reproduce_the_circuit(oracle, native, layouts, dtype, n, m,
                                       gates):
    circ_gates = random_circuit(n, gates, seed=n * 7 + m)
    circ = Circuit.from_gates(n, circ_gates)
    prog = circ.compile(dtype, "cpu", tile_qubits=m, min_contiguous=2,
                        layouts=layouts, native=native)
    assert prog.native == native
    rng = np.random.default_rng(n + m)
    psi0 = rng.normal(size=(2, 2 ** n)) + 1j * rng.normal(size=(2, 2 ** n))
    psi0 /= np.linalg.norm(psi0, axis=1, keepdims=True)
    got = _run_records(prog, psi0.copy())
    ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in circ_gates],
                             psi0)
    # the pool holds the matrices in the program's precision
    tol = 2e-5 if dtype == torch.complex64 else 1e-12
    assert np.abs(got - ref).max() <= tol


def _unitary(rng, d):
    q, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q


def _general_circuit(n, num, seed):
    """Dense 4x4 unitaries, controlled 2x2 unitaries (diag(I, U)) and
    dense / diagonal single-qubit gates on random qubits."""
    rng = np.random.default_rng(seed)
    circ = Circuit(n)
    listing = []
    for _ in range(num):
        kind = rng.integers(4)
        q = [int(x) for x in rng.choice(n, size=2 if kind < 2 else 1,
                                         replace=False)]
        if kind == 0:
            mat, tag = _unitary(rng, 4), "dense"
        elif kind == 1:
            mat = np.eye(4, dtype=complex)
            mat[2:, 2:] = _unitary(rng, 2)
            tag = "ctrl"
        elif kind == 2:
            mat, tag = _unitary(rng, 2), "dense"
        else:
            mat, tag = np.diag(np.exp(1j * rng.normal(size=2))), "diag"
        circ.append(torch.from_numpy(mat), q, tag)
        listing.append((mat, q))
    return circ, listing


@pytest.mark.parametrize("native", [True, False])
@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_records_general_two_qubit_gates(oracle, native, dtype):
    """Dense two-qubit records and controls on thread bits (CDENSE1)."""
    n, m = 9, 6
    circ, listing = _general_circuit(n, 160, seed=4)
    prog = circ.compile(dtype, "cpu", tile_qubits=m, min_contiguous=2,
                        native=native)
    kinds = set(prog.gate_records.cpu().numpy().view(FG_DTYPE)["kind"])
    assert {FG_DENSE2, FG_CDENSE1} <= {int(k) for k in kinds}
    rng = np.random.default_rng(1)
    psi0 = rng.normal(size=(1, 2 ** n)) + 1j * rng.normal(size=(1, 2 ** n))
    psi0 /= np.linalg.norm(psi0)
    got = _run_records(prog, psi0.copy())
    ref = oracle.run_circuit(listing, psi0)
    tol = 2e-5 if dtype == torch.complex64 else 1e-12
    assert np.abs(got - ref).max() <= tol


def test_executor_detects_a_wrong_record(oracle):
    """The check has teeth: one record moved to another register bit gives
    a different state."""
    n, m = 8, 6
    circ_gates = random_circuit(n, 80, seed=11)
    prog = Circuit.from_gates(n, circ_gates).compile(
        torch.complex128, "cpu", tile_qubits=m, min_contiguous=2)
    recs = prog.gate_records.cpu().numpy().view(FG_DTYPE)
    dense = np.flatnonzero(np.isin(recs["kind"], [FG_DENSE1, FG_REAL1]))
    assert len(dense)
    raw = prog.gate_records.cpu().numpy().copy()
    bad = raw.view(FG_DTYPE)
    j = dense[0]
    bad["b0"][j] = (bad["b0"][j] + 1) % prog.rb
    prog.gate_records = torch.from_numpy(raw)
    rng = np.random.default_rng(2)
    psi0 = rng.normal(size=(1, 2 ** n)) + 1j * rng.normal(size=(1, 2 ** n))
    psi0 /= np.linalg.norm(psi0)
    got = _run_records(prog, psi0.copy())
    ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in circ_gates],
                             psi0)
    assert np.abs(got - ref).max() > 1e-3


def test_planners_on_random_circuits_and_tiles(oracle):
    """Property search over circuits and tile parameters (both planners,
    layouts on and off): the records always reproduce the circuit."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from qcware_unitair_gb300 import _lib
    L = _lib.load()

    @hyp.settings(max_examples=60, deadline=None)
    @hyp.given(n=st.integers(2, 9), seed=st.integers(0, 10 ** 6),
               num=st.integers(1, 60), native=st.booleans(),
               layouts=st.booleans(), c128=st.booleans(),
               general=st.booleans(), data=st.data())
    def run(n, seed, num, native, layouts, c128, general, data):
        dtype = torch.complex128 if c128 else torch.complex64
        code = _lib.C128 if c128 else _lib.C64
        m = data.draw(st.integers(min(n, 2), min(n, int(
            L.gbsv_fused_max_tile_qubits(code)))))
        cmin = data.draw(st.integers(0 if c128 else 1, m))
        if general:
            circ, listing = _general_circuit(n, num, seed)
        else:
            gates = random_circuit(n, num, seed=seed)
            circ = Circuit.from_gates(n, gates)
            listing = [(g.matrix(), g.qubits) for g in gates]
        prog = circ.compile(dtype, "cpu", tile_qubits=m, min_contiguous=cmin,
                            layouts=layouts, native=native)
        rng = np.random.default_rng(seed)
        psi0 = rng.normal(size=(1, 2 ** n)) + 1j * rng.normal(
            size=(1, 2 ** n))
        psi0 /= np.linalg.norm(psi0)
        got = _run_records(prog, psi0.copy())
        ref = oracle.run_circuit(listing, psi0)
        tol = 1e-4 if dtype == torch.complex64 else 1e-11
        assert np.abs(got - ref).max() <= tol

    run()
