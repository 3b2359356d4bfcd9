"""Pin the CPU oracle to the reference's own outputs (golden vectors that
tests/golden/make_golden.py recorded by running unitair), to the known
answers of unitair's README / tutorial, and to an independent numpy
restatement."""
import math

import numpy as np
import pytest

from conftest import golden_data

G = golden_data()


def _tol(arr):
    return 2e-5 if arr.dtype in (np.complex64, np.float32) else 1e-12


@pytest.mark.parametrize("case", G.of_kind("apply"), ids=lambda c: c["name"])
def test_oracle_apply_matches_reference(oracle, case):
    op = G[case["name"] + "/op"]
    st = G.state_of(case)
    ref = G[case["name"] + "/out"]
    got = oracle.apply_operator(op, case["qubits"], st)
    assert got.shape == ref.shape
    scale = max(1.0, np.abs(ref).max())
    np.testing.assert_allclose(got, ref, atol=_tol(ref) * scale * 4, rtol=0)
    # independent numpy restatement agrees with the C oracle to rounding
    np.testing.assert_allclose(oracle.apply_operator_numpy(op, case["qubits"],
                                                           st), got,
                               atol=1e-12 * scale, rtol=0)


@pytest.mark.parametrize("case", G.of_kind("all_qubits"),
                         ids=lambda c: c["name"])
def test_oracle_all_qubits(oracle, case):
    ref = G[case["name"] + "/out"]
    got = oracle.apply_all_qubits(G[case["name"] + "/op"],
                                  G[case["name"] + "/state"])
    scale = max(1.0, np.abs(ref).max())
    np.testing.assert_allclose(got, ref, atol=_tol(ref) * scale * 8, rtol=0)


@pytest.mark.parametrize("case", G.of_kind("phase"), ids=lambda c: c["name"])
def test_oracle_phase(oracle, case):
    ref = G[case["name"] + "/out"]
    ang, st = G[case["name"] + "/angles"], G[case["name"] + "/state"]
    got = oracle.apply_phase(ang, st)
    assert got.shape == ref.shape
    single = ang.dtype == np.float32 or st.dtype == np.complex64
    tol = 2e-6 if single else 1e-12
    np.testing.assert_allclose(got, ref, atol=tol * np.abs(st).max(), rtol=0)


def test_oracle_reductions(oracle):
    for c in G.of_kind("inner"):
        ref = G[c["name"] + "/out"]
        got = oracle.inner_product(G[c["name"] + "/a"], G[c["name"] + "/b"])
        np.testing.assert_allclose(got, ref, rtol=1e-5 if ref.dtype ==
                                   np.complex64 else 1e-12)
    for c in G.of_kind("norm"):
        st = G[c["name"] + "/state"]
        np.testing.assert_allclose(oracle.norm_squared(st),
                                   G[c["name"] + "/out"], rtol=1e-5)
        if c["name"] + "/abs2" in G.arrays.files:
            np.testing.assert_allclose(oracle.abs_squared(st),
                                       G[c["name"] + "/abs2"], rtol=1e-6)
    for c in G.of_kind("diag"):
        ref = G[c["name"] + "/out"]
        got = oracle.diag_expectation_value(G[c["name"] + "/diag"],
                                            G[c["name"] + "/state"])
        np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-4)


def test_oracle_circuits(oracle):
    from qcware_unitair_gb300.circuits import random_circuit
    for c in G.of_kind("circuit"):
        gates = [(g.matrix(), g.qubits)
                 for g in random_circuit(c["n"], c["depth"], seed=c["seed"])]
        st = G[c["name"] + "/state"].astype(np.complex128)
        got = oracle.run_circuit(gates, st)
        ref = G[c["name"] + "/out"]
        tol = 2e-5 if ref.dtype == np.complex64 else 1e-12
        assert np.abs(got - ref).max() < tol, c["name"]


def test_known_answers(oracle):
    """README.rst:153-224 and docs/tutorial/first_example.rst:271-333."""
    s = 1 / math.sqrt(2)
    h = np.array([[s, s], [s, -s]])
    np.testing.assert_allclose(G["kat_h0/out"], [s, s], atol=1e-6)
    np.testing.assert_allclose(oracle.apply_operator(h, [0], [1, 0]),
                               [s, s], atol=1e-15)
    cnot = np.eye(4)[[0, 1, 3, 2]]
    bell = oracle.apply_operator(cnot, [0, 1],
                                 oracle.apply_operator(h, [0], [1, 0, 0, 0]))
    np.testing.assert_allclose(bell, [s, 0, 0, s], atol=1e-15)
    np.testing.assert_allclose(G["kat_bell/out"], bell, atol=1e-6)
    np.testing.assert_allclose(G["kat_expx/out"],
                               [[0.8776, -0.4794j], [-0.4794j, 0.8776]],
                               atol=1e-4)
    t = G["kat_expx_batch/t"].astype(np.float64)
    ops = np.stack([np.stack([np.cos(t), -1j * np.sin(t)], -1),
                    np.stack([-1j * np.sin(t), np.cos(t)], -1)], -2)
    got = oracle.apply_operator(ops, [0], np.array([1, 0]))
    np.testing.assert_allclose(got, G["kat_expx_batch/out"], atol=1e-6)
    # the batch ends near -|0> (first_example.rst:283-333)
    assert abs(got[-1, 0] + 1) < 1e-3


def test_oracle_c64_port_tracks_c128(oracle):
    rng = np.random.default_rng(7)
    for n, qs in ((6, [5]), (9, [0, 8]), (7, [3, 1, 6])):
        k = len(qs)
        st = (rng.normal(size=(3, 2 ** n)) + 1j * rng.normal(size=(3, 2 ** n)))
        op = rng.normal(size=(3, 2 ** k, 2 ** k)) + 0j
        a = oracle.apply_operator(op, qs, st)
        b = oracle.apply_operator_c64(op, qs, st)
        assert b.dtype == np.complex64
        np.testing.assert_allclose(b, a, atol=1e-4 * np.abs(a).max())


def test_oracle_rejects_bad_qubits(oracle):
    with pytest.raises(ValueError):
        oracle.apply_operator(np.eye(2), [3], np.ones(8))
    with pytest.raises(ValueError):
        oracle.apply_operator(np.eye(4), [1, 1], np.ones(8))


@pytest.mark.parametrize("k", [9, 10, 11, 12])
def test_oracle_wide_operators_match_numpy(oracle, k):
    """Operators on 9-12 qubits (too large for golden files): the C oracle
    against the independent einsum restatement, shared and per-state
    operators, targets in a scrambled order."""
    rng = np.random.default_rng(500 + k)
    n = k + 1
    qubits = [int(q) for q in rng.permutation(n)[:k]]
    st = rng.standard_normal((2, 2 ** n)) + 1j * rng.standard_normal((2, 2 ** n))
    for shape in ((2 ** k, 2 ** k), (2, 2 ** k, 2 ** k)):
        op = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) \
            / 2 ** (k / 2)
        got = oracle.apply_operator(op, qubits, st)
        ref = oracle.apply_operator_numpy(op, qubits, st)
        scale = max(1.0, np.abs(ref).max())
        np.testing.assert_allclose(got, ref, atol=1e-12 * scale, rtol=0)
