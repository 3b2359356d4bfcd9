"""Parity of the CUDA path (through the C ABI) with the reference's golden
outputs and with the CPU oracle.

Tolerances (max abs error, scaled by the largest magnitude involved):
complex64 1e-5, complex128 1e-12 for gate application; reductions are
FP64-accumulated and compared at 1e-6 (c64 inputs) / 1e-12 (c128).
"""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300 import _lib, states as S
from qcware_unitair_gb300.circuits import (random_circuit, random_states,
                                           zero_state)
from conftest import golden_data

pytestmark = pytest.mark.gpu
G = golden_data()
DEV = torch.device("cuda:0")
DT = {"c64": torch.complex64, "c128": torch.complex128}
EXC = {"ValueError": ValueError, "RuntimeError": RuntimeError,
       "StateShapeError": S.StateShapeError}


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def tol_of(dtype):
    return 1e-5 if dtype in (np.complex64, torch.complex64) else 1e-12


def assert_close(got, ref, tol):
    got = got.detach().cpu().numpy() if isinstance(got, torch.Tensor) else got
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    scale = max(1.0, float(np.abs(ref).max()) if ref.size else 1.0)
    err = float(np.abs(got.astype(np.complex128) - ref).max()) if ref.size \
        else 0.0
    assert err <= tol * scale, f"max abs err {err:.3e} > {tol * scale:.3e}"


# ------------------------------------------------------------ golden ------
@pytest.mark.parametrize("case", G.of_kind("apply"), ids=lambda c: c["name"])
def test_apply_operator_golden(case):
    op = G[case["name"] + "/op"]
    st = G.state_of(case)
    ref = G[case["name"] + "/out"]
    got = ug.apply_operator(cu(op), case["qubits"], cu(st))
    assert got.dtype == torch.from_numpy(ref).dtype
    assert_close(got, ref, 4 * tol_of(ref.dtype))


@pytest.mark.parametrize("case", G.of_kind("all_qubits"),
                         ids=lambda c: c["name"])
def test_apply_all_qubits_golden(case):
    ref = G[case["name"] + "/out"]
    got = ug.apply_all_qubits(cu(G[case["name"] + "/op"]),
                              cu(G[case["name"] + "/state"]))
    assert_close(got, ref, 8 * tol_of(ref.dtype))


@pytest.mark.parametrize("case", G.of_kind("phase"), ids=lambda c: c["name"])
def test_apply_phase_golden(case):
    ang, st = G[case["name"] + "/angles"], G[case["name"] + "/state"]
    ref = G[case["name"] + "/out"]
    got = ug.apply_phase(cu(ang), cu(st))
    assert got.dtype == torch.from_numpy(ref).dtype
    single = ang.dtype == np.float32 or st.dtype == np.complex64
    assert_close(got, ref, 2e-6 if single else 1e-12)


def test_reductions_golden():
    for c in G.of_kind("inner"):
        ref = G[c["name"] + "/out"]
        got = ug.inner_product(cu(G[c["name"] + "/a"]), cu(G[c["name"] + "/b"]))
        assert got.dtype == torch.from_numpy(ref).dtype
        assert_close(got, ref, 1e-5 if ref.dtype == np.complex64 else 1e-12)
    for c in G.of_kind("norm"):
        st = G[c["name"] + "/state"]
        ref = G[c["name"] + "/out"]
        got = ug.norm_squared(cu(st))
        assert got.dtype == torch.from_numpy(ref).dtype
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-5)
        # FP64 accumulation: the float64 result matches the oracle tightly
        exact = np.sum(np.abs(st.astype(np.complex128)) ** 2, -1)
        np.testing.assert_allclose(S.norm_squared_fp64(cu(st)).cpu().numpy(),
                                   exact, rtol=1e-12)
        if c["name"] + "/abs2" in G.arrays.files:
            np.testing.assert_allclose(ug.abs_squared(cu(st)).cpu().numpy(),
                                       G[c["name"] + "/abs2"], rtol=1e-6)
    for c in G.of_kind("diag"):
        ref = G[c["name"] + "/out"]
        got = ug.diag_expectation_value(cu(G[c["name"] + "/diag"]),
                                        cu(G[c["name"] + "/state"]))
        assert got.dtype == torch.from_numpy(ref).dtype
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-4,
                                   atol=1e-4)


@pytest.mark.parametrize("case", G.of_kind("grad"), ids=lambda c: c["name"])
def test_autograd_golden(case):
    op = cu(G[case["name"] + "/op"]).requires_grad_()
    st = cu(G[case["name"] + "/state"]).requires_grad_()
    w = cu(G[case["name"] + "/w"])
    out = ug.apply_operator(op, case["qubits"], st)
    assert_close(out, G[case["name"] + "/out"], 1e-12)
    loss = (out * w).real.sum() + (out.conj() * out).real.sum()
    loss.backward()
    assert_close(op.grad, G[case["name"] + "/gop"], 1e-11)
    assert_close(st.grad, G[case["name"] + "/gstate"], 1e-11)


def test_known_answers():
    s = 2 ** -0.5
    h = ug.gates.hadamard(device=DEV)
    out = ug.apply_operator(h, [0], ug.unit_vector(0, 1, device=DEV))
    assert_close(out, [s, s], 1e-7)
    bell = ug.apply_operator(ug.gates.cnot(device=DEV), [0, 1],
                             ug.apply_operator(h, [0],
                                               ug.unit_vector(0, 2, device=DEV)))
    assert_close(bell, G["kat_bell/out"], 1e-7)
    t = cu(G["kat_expx_batch/t"])
    out = ug.apply_operator(ug.gates.exp_x(t), [0],
                            ug.unit_vector(0, 1, device=DEV))
    assert_close(out, G["kat_expx_batch/out"], 1e-6)


@pytest.mark.parametrize("spec", G.errors, ids=lambda s: str(s))
def test_error_parity_cuda(spec):
    op = torch.ones(spec["op_shape"], dtype=DT[spec["op_dtype"]], device=DEV)
    st = torch.ones(spec["state_shape"], dtype=DT[spec["state_dtype"]],
                    device=DEV)
    call = (lambda: ug.apply_all_qubits(op, st)) \
        if spec["fn"] == "apply_all_qubits" \
        else (lambda: ug.apply_operator(op, spec["qubits"], st))
    if "error" in spec:
        with pytest.raises(EXC[spec["error"]]):
            call()
    else:
        assert list(call().shape) == spec["ok"]


# ------------------------------------------------------------ oracle ------
def _rand(rng, shape, dtype):
    a = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return a.astype(np.complex64 if dtype == torch.complex64 else
                    np.complex128)


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_every_target_position_vs_oracle(oracle, dtype):
    """k = 1 on every qubit and k = 2 on low/low, low/high, high/high pairs
    (both orders), for 1..14 qubits and three batch structures."""
    rng = np.random.default_rng(11)
    for n in range(1, 15):
        pairs = [(q,) for q in range(n)]
        if n >= 2:
            cand = {(n - 1, n - 2), (n - 2, n - 1), (0, n - 1), (n - 1, 0),
                    (0, 1), (1, 0)}
            if n >= 3:
                cand |= {(n - 3, n - 1), (n - 1, n - 3), (n - 3, 0)}
            pairs += sorted(c for c in cand if c[0] != c[1])
        for qs in pairs:
            k = len(qs)
            for ob, sb in (((), (3,)), ((3,), (3,)), ((2,), ())):
                op = _rand(rng, ob + (2 ** k, 2 ** k), dtype)
                st = _rand(rng, sb + (2 ** n,), dtype)
                ref = oracle.apply_operator(op, qs, st)
                got = ug.apply_operator(cu(op), qs, cu(st))
                assert_close(got, ref, 4 * tol_of(dtype))


def test_unaligned_and_inplace_paths(oracle):
    rng = np.random.default_rng(5)
    for dtype in (torch.complex64, torch.complex128):
        for qs in ([0], [7], [8], [3, 8], [8, 7], [0, 1]):
            k = len(qs)
            op = _rand(rng, (2 ** k, 2 ** k), dtype)
            big = _rand(rng, (1 + 2 * 512,), dtype)
            base = cu(big)
            st = base[1:].view(2, 512)  # 8- or 16-byte aligned view
            ref = oracle.apply_operator(op, qs, big[1:].reshape(2, 512))
            assert_close(ug.apply_operator(cu(op), qs, st), ref,
                         4 * tol_of(dtype))
            s2 = cu(big[1:].reshape(2, 512)).contiguous()
            ug.apply_operator_(cu(op), qs, s2)
            assert_close(s2, ref, 4 * tol_of(dtype))


@pytest.mark.parametrize("k", [3, 4, 5])
def test_wide_operators_vs_oracle(oracle, k):
    rng = np.random.default_rng(k)
    n = 9
    for trial in range(4):
        qs = [int(q) for q in rng.permutation(n)[:k]]
        op = _rand(rng, (2, 2 ** k, 2 ** k), torch.complex128)
        st = _rand(rng, (2, 2 ** n), torch.complex128)
        assert_close(ug.apply_operator(cu(op), qs, cu(st)),
                     oracle.apply_operator(op, qs, st), 1e-12)


def test_all_qubits_extension_each(oracle):
    rng = np.random.default_rng(3)
    n = 9
    ops = _rand(rng, (4, n, 2, 2), torch.complex64)
    st = _rand(rng, (4, 2 ** n), torch.complex64)
    ref = oracle.apply_all_qubits_each(ops, st)
    assert_close(ug.apply_each_qubit(cu(ops), cu(st)), ref, 2e-5)


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5),
                                       (torch.complex128, 1e-12)])
def test_1000_gate_circuit_vs_complex128_oracle(oracle, dtype, tol):
    """The accuracy target: <= 1e-5 (c64) / 1e-12 (c128) max abs amplitude
    error after 1,000 random gates against the complex128 oracle."""
    n, batch = 14, 2
    gates = random_circuit(n, 1000, seed=42)
    psi0 = random_states(n, (batch,), dtype, seed=42)
    psi = psi0.to(DEV)
    for g in gates:
        m = torch.from_numpy(g.matrix()).to(device=DEV, dtype=dtype)
        psi = ug.apply_operator(m, g.qubits, psi)
    ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in gates],
                             psi0.numpy().astype(np.complex128))
    err = float(np.abs(psi.cpu().numpy() - ref).max())
    drift = float((S.norm_squared_fp64(psi) - 1).abs().max())
    print(f"{dtype}: max|err| {err:.3e}, norm drift {drift:.3e}")
    assert err <= tol
    assert drift <= (1e-5 if dtype == torch.complex64 else 1e-12)


def test_golden_circuits():
    for c in G.of_kind("circuit"):
        dtype = torch.complex64 if c["dtype"].endswith("complex64") else \
            torch.complex128
        psi = cu(G[c["name"] + "/state"])
        for g in random_circuit(c["n"], c["depth"], seed=c["seed"]):
            m = torch.from_numpy(g.matrix()).to(device=DEV, dtype=dtype)
            psi = ug.apply_operator(m, g.qubits, psi)
        ref = G[c["name"] + "/out"]
        assert_close(psi, ref, 2e-5 if dtype == torch.complex64 else 1e-12)
        np.testing.assert_allclose(ug.norm_squared(psi).cpu().numpy(),
                                   G[c["name"] + "/norms"], rtol=1e-5)


def test_large_reductions_vs_oracle(oracle):
    rng = np.random.default_rng(9)
    for shape in ((1, 2 ** 22), (3, 2 ** 17), (600, 256)):
        a = _rand(rng, shape, torch.complex64)
        b = _rand(rng, shape, torch.complex64)
        ra = S.norm_squared_fp64(cu(a)).cpu().numpy()
        np.testing.assert_allclose(ra, oracle.norm_squared(a), rtol=1e-12)
        ip = ug.inner_product(cu(a), cu(b)).cpu().numpy()
        np.testing.assert_allclose(ip, oracle.inner_product(a, b), rtol=1e-6)
        d = rng.normal(size=shape[-1:]).astype(np.float64)
        de = ug.diag_expectation_value(cu(d), cu(a)).cpu().numpy()
        np.testing.assert_allclose(de, oracle.diag_expectation_value(d, a),
                                   rtol=1e-9, atol=1e-9)
        # deterministic: the same bits twice
        r2 = S.norm_squared_fp64(cu(a)).cpu().numpy()
        assert np.array_equal(ra, r2)


def test_empty_batches():
    st = torch.zeros(0, 16, dtype=torch.complex64, device=DEV)
    op = torch.eye(2, dtype=torch.complex64, device=DEV)
    assert ug.apply_operator(op, [1], st).shape == (0, 16)
    assert ug.norm_squared(st).shape == (0,)
    assert ug.apply_phase(torch.zeros(16, device=DEV), st).shape == (0, 16)


def test_30_qubit_round_trip():
    """Full size (30 qubits, complex64, 8 GiB): 200 random gates then their
    inverses in reverse order must return |0...0> (size-independent
    property), with the norm kept to FP32 rounding."""
    n = 30
    free = torch.cuda.mem_get_info()[0]
    if free < 20 * 2 ** 30:
        pytest.skip("needs 20 GiB free device memory")
    gates = random_circuit(n, 200, seed=7)
    psi = zero_state(n, (), torch.complex64, device=DEV)
    mats = [torch.from_numpy(g.matrix()).to(device=DEV,
                                            dtype=torch.complex64)
            for g in gates]
    for g, m in zip(gates, mats):
        ug.apply_operator_(m, g.qubits, psi)
    for g, m in zip(reversed(gates), reversed(mats)):
        ug.apply_operator_(m.conj().T.contiguous(), g.qubits, psi)
    norm = float(S.norm_squared_fp64(psi))
    drift = abs(norm - 1)
    a0 = complex(psi[0].item())
    rest = norm - abs(a0) ** 2  # weight left outside |0...0>
    del psi
    torch.cuda.empty_cache()
    assert drift < 1e-4
    assert abs(a0 - 1) < 1e-4
    assert rest < 1e-8


def test_launch_counter_counts_kernels():
    before = _lib.launch_count()
    st = torch.ones(4, 64, dtype=torch.complex64, device=DEV)
    ug.apply_operator(ug.gates.hadamard(device=DEV), [2], st)
    ug.norm_squared(st)
    assert _lib.launch_count() - before == 2


@pytest.mark.parametrize("k", [3, 4, 5, 6])
@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-6),
                                       (torch.complex128, 1e-13)])
def test_wide_operators_group_kernel(oracle, k, dtype, tol):
    """3- to 6-qubit operators (one thread per group of 2^k amplitudes, or
    the wide-operator kernel through a temporary when in place): shared and
    per-state matrices, target 0 among the targets or not, against the
    complex128 oracle."""
    import qcware_unitair_gb300 as ug
    rng = np.random.default_rng(40 + k)
    n, B = 9, 3
    psi = (rng.standard_normal((B, 2 ** n)) +
           1j * rng.standard_normal((B, 2 ** n)))
    for qubits in ([int(q) for q in rng.choice(n, k, replace=False)],
                   [n - 1] + [int(q) for q in rng.choice(n - 1, k - 1,
                                                        replace=False)]):
        for batched in (False, True):
            shape = (B, 2 ** k, 2 ** k) if batched else (2 ** k, 2 ** k)
            op = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            st = torch.from_numpy(psi).to(DEV, dtype)
            got = ug.apply_operator(torch.from_numpy(op).to(DEV, dtype),
                                    qubits, st).cpu().numpy()
            ref = oracle.apply_operator(op, qubits, psi)
            assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
            ug.apply_operator_(torch.from_numpy(op).to(DEV, dtype), qubits,
                               st)
            assert np.abs(st.cpu().numpy() - ref).max() <= (
                tol * np.abs(ref).max())
