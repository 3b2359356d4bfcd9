"""The C++ planner (gbsv_plan) produces exactly what the Python planner
in fusion.py produces: the same passes, gate records, layouts and pool."""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300.circuits import gate_matrix, random_circuit
from qcware_unitair_gb300.fusion import Circuit


def _cmp(circ, dtype, **kw):
    kw.setdefault("tensor_cores", False)  # the register-stage planners
    a = circ.compile(dtype, "cpu", native=True, **kw)
    b = circ.compile(dtype, "cpu", native=False, **kw)
    assert a.native and not b.native
    assert [o[0] for o in a.ops] == [o[0] for o in b.ops]
    for x, y in zip(a.ops, b.ops):
        if x[0] == "plain":
            assert torch.equal(x[1], y[1]) and x[2] == y[2]
        else:
            assert x[1] == y[1] and list(x[2]) == list(y[2])
            assert x[3:] == y[3:]
    assert torch.equal(a.gate_records[:b.gate_records.numel()],
                       b.gate_records)
    assert torch.equal(a.layout_records[:b.layout_records.numel()],
                       b.layout_records)
    assert torch.equal(a.pool, b.pool)
    return a


@pytest.mark.parametrize("n,m,cmin", [(30, 12, 4), (30, 13, 4), (20, 12, 4),
                                      (12, 12, 4), (9, 5, 2), (6, 4, 1)])
@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_native_matches_python(n, m, cmin, dtype):
    circ = Circuit.from_gates(n, random_circuit(n, 300, seed=n * m))
    _cmp(circ, dtype, tile_qubits=m, min_contiguous=cmin)
    _cmp(circ, dtype, tile_qubits=m, min_contiguous=cmin, layouts=False)
    _cmp(circ, dtype, fuse=False)


def test_native_per_state_and_wide_gates():
    rng = np.random.default_rng(0)
    n, B = 9, 4
    c = Circuit(n)
    th = torch.from_numpy(rng.uniform(0, 6, size=(B,)))
    for q in range(n):
        c.rx(q, th)
        c.rz(q, th)
        c.ry(q, th * 0.3)
    for q in range(n - 1):
        c.cnot(q, q + 1)
        c.cz(q, n - 1 - q) if q != n - 1 - q else None
    u = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    c.append(torch.from_numpy(u), [4, 0, 7])
    c.swap(2, 6)
    c.append(torch.from_numpy(gate_matrix("Y")), [3])
    for m in (4, 6, 9):
        _cmp(c, torch.complex64, tile_qubits=m, min_contiguous=2)
