"""Fusion planner on CPU: every gate lands in exactly one pass, in order,
each stage's tile holds the bits its gates need, and the canonical
30-qubit circuit needs far fewer passes than gates."""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300.circuits import random_circuit
from qcware_unitair_gb300.fusion import (CTRL, DENSE, DIAG, Circuit, _needs,
                                         classify, plan)


def test_classify_structures():
    from qcware_unitair_gb300.circuits import gate_matrix
    t = lambda n, th=None: torch.from_numpy(gate_matrix(n, th))
    assert classify(t("RZ", 0.3)) == DIAG
    assert classify(t("CZ")) == DIAG
    assert classify(t("CNOT")) == CTRL
    assert classify(t("SWAP")) == DENSE
    assert classify(t("H")) == DENSE
    batched = torch.stack([t("RZ", 0.1), t("RZ", 0.2)])
    assert classify(batched) == DIAG


@pytest.mark.parametrize("n,m,cmin", [(30, 13, 4), (20, 12, 4), (10, 4, 2),
                                      (12, 12, 4), (6, 3, 1)])
def test_plan_covers_gates_in_order(n, m, cmin):
    c = Circuit.from_gates(n, random_circuit(n, 400, seed=n))
    ops = plan(c.gates, n, m, cmin)
    seen = []
    for kind, item in ops:
        if kind == "plain":
            seen.append(item)
            continue
        assert len(item.tile) == m
        assert set(range(min(cmin, m))) <= item.tile
        for g in item.gates:
            assert _needs(g, n) <= item.tile
        seen.extend(item.gates)
    assert [id(g) for g in seen] == [id(g) for g in c.gates]


def test_canonical_30q_pass_reduction():
    """At least 3x fewer HBM passes than one kernel per gate (measured
    planner output: 55 passes for 1000 gates at 13 tile qubits)."""
    c = Circuit.from_gates(30, random_circuit(30, 1000, seed=0))
    ops = plan(c.gates, 30, 13, 4)
    assert len(ops) * 3 <= 1000
    assert len(ops) <= 60


def test_wide_gates_run_unfused():
    c = Circuit(6)
    c.h(0)
    c.append(torch.eye(8, dtype=torch.complex128), [0, 1, 2])
    c.h(5)
    ops = plan(c.gates, 6, 4, 2)
    assert [k for k, _ in ops] == ["stage", "plain", "stage"]


def test_circuit_validation():
    c = Circuit(3)
    with pytest.raises(ValueError):
        c.append(torch.eye(2), [3])
    with pytest.raises(ValueError):
        c.append(torch.eye(4), [1, 1])
    with pytest.raises(ValueError):
        c.append(torch.eye(2), [0, 1])
