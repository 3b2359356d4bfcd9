"""apply_to_qubits, swap / permute_qubits / roll_qubits, multi_cz,
multi_controlled_z / x and measure against the reference's outputs
(golden vectors) and, for sampling, against |psi|^2."""
import numpy as np
import pytest
import torch

import qcware_unitair_gb300 as ug
from conftest import golden_data

pytestmark = pytest.mark.gpu
G = golden_data()
DEV = torch.device("cuda:0")


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def close(got, ref, tol):
    got = got.cpu().numpy()
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("case", G.of_kind("perm"), ids=lambda c: c["name"])
def test_permutations_exact(case):
    st = cu(G[case["name"] + "/state"])
    n = case["n"]
    g = lambda k: G[case["name"] + "/" + k]
    # pure permutations: bit-exact
    assert np.array_equal(ug.swap(st, (1, n - 1)).cpu().numpy(), g("swap"))
    assert np.array_equal(ug.swap(st, (0, -1)).cpu().numpy(), g("swap_neg"))
    assert np.array_equal(ug.permute_qubits(list(reversed(range(n))),
                                            st).cpu().numpy(), g("perm"))
    assert np.array_equal(ug.permute_qubits([2, 0, 1] + list(range(3, n)),
                                            st).cpu().numpy(), g("perm2"))
    assert np.array_equal(ug.roll_qubits(st, 1).cpu().numpy(), g("roll1"))
    assert np.array_equal(ug.roll_qubits(st, 3).cpu().numpy(), g("roll3"))
    assert np.array_equal(ug.roll_qubits(st, -2).cpu().numpy(), g("rollm"))
    assert ug.swap(st, (2, 2)) is st


@pytest.mark.parametrize("case", G.of_kind("to_qubits"),
                         ids=lambda c: c["name"])
def test_apply_to_qubits(case):
    st = cu(G[case["name"] + "/state"])
    ops = cu(G[case["name"] + "/ops"])
    ref = G[case["name"] + "/out"]
    tol = 1e-5 if ref.dtype == np.complex64 else 1e-12
    got = ug.apply_to_qubits(list(ops), case["qubits"], st)
    close(got, ref, 8 * tol)


def test_multi_controlled():
    st = cu(G["mcz_0/state"])
    pairs = torch.from_numpy(G["mcz_0/pairs"]).to(DEV)
    assert np.array_equal(ug.multi_cz(pairs, st).cpu().numpy(),
                          G["mcz_0/out"])
    assert np.array_equal(
        ug.multi_cz(torch.tensor([3, 1], device=DEV), st).cpu().numpy(),
        G["mcz_0/single"])
    assert np.array_equal(ug.multi_controlled_z([1, 4, 2], st).cpu().numpy(),
                          G["mcz_0/mcz"])
    # unitair builds it as H, C..CZ, H: equal up to that rounding
    close(ug.multi_controlled_x(st, [0, 5], 2), G["mcz_0/mcx"], 1e-6)
    with pytest.raises(ValueError):
        ug.multi_cz(torch.tensor([[0, 0]], device=DEV), st)
    with pytest.raises(ValueError):
        ug.multi_cz(torch.tensor([0, 1]), st)  # device mismatch


def test_measure_distribution():
    n = 10
    rng = np.random.default_rng(0)
    amps = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    amps[::7] = 0  # zero-probability outcomes must never be drawn
    amps /= np.linalg.norm(amps)
    st = cu(amps.astype(np.complex64))
    N = 400000
    idx = ug.measurement.sample(st, N, seed=123).cpu().numpy()
    assert idx.min() >= 0 and idx.max() < 2 ** n
    assert not np.any(np.isin(idx, np.arange(0, 2 ** n, 7)))
    freq = np.bincount(idx, minlength=2 ** n) / N
    p = np.abs(amps) ** 2
    # each bin within 6 sigma of its binomial mean
    sigma = np.sqrt(p * (1 - p) / N) + 1e-12
    assert np.all(np.abs(freq - p) <= 6 * sigma + 1e-9)
    again = ug.measurement.sample(st, N, seed=123).cpu().numpy()
    assert np.array_equal(idx, again)  # a function of the seed only
    h = ug.measure(st, 1000, seed=5)
    assert sum(h.histogram.values()) == 1000
    counts = list(h.histogram.values())
    assert counts == sorted(counts, reverse=True)
    assert all(len(k) == n for k in h.histogram)
    raw = ug.measure(st, 1000, raw_output=True, seed=5)
    assert sum(raw.values()) == 1000
    assert h["0" * n] == raw.get(0, 0)


def test_measure_large_state_chunks():
    n = 22
    st = torch.zeros(2 ** n, dtype=torch.complex64, device=DEV)
    st[5] = 0.6
    st[2 ** n - 3] = 0.8j
    idx = ug.measurement.sample(st, 100000, seed=1).cpu().numpy()
    assert set(np.unique(idx)) == {5, 2 ** n - 3}
    frac = np.mean(idx == 5)
    assert abs(frac - 0.36) < 0.01


def test_measure_sparse_blocks():
    """Mass in a few 256-amplitude chunks only (the first chunk, one in the
    middle and the last), so most blocks of the sampling table hold zero
    probability and the block search must skip them."""
    n = 20
    rng = np.random.default_rng(11)
    amps = np.zeros(2 ** n, dtype=np.complex128)
    for start in (0, 2 ** 19 + 3 * 256, 2 ** n - 256):
        amps[start:start + 256] = rng.normal(size=256) + \
            1j * rng.normal(size=256)
    amps[::5] = 0
    amps /= np.linalg.norm(amps)
    st = cu(amps.astype(np.complex64))
    N = 300000
    idx = ug.measurement.sample(st, N, seed=21).cpu().numpy()
    p = np.abs(amps) ** 2
    assert np.all(p[idx] > 0)
    support = np.flatnonzero(p)
    freq = np.bincount(idx, minlength=2 ** n)[support] / N
    ps = p[support]
    sigma = np.sqrt(ps * (1 - ps) / N) + 1e-12
    assert np.all(np.abs(freq - ps) <= 6 * sigma + 1e-9)


@pytest.mark.parametrize("n", [1, 3, 6, 8, 9, 12, 16])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_measure_distribution_sizes(n, dtype):
    """Chunks and groups of amplitudes (256 / 16 for complex64 states of
    whole chunks, 1024 / 32 otherwise), partial groups for tiny states,
    zero-probability groups, both precisions."""
    rng = np.random.default_rng(n)
    amps = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    if n >= 6:
        amps[32:64] = 0  # an empty group
    amps /= np.linalg.norm(amps)
    st = cu(amps.astype(dtype))
    N = 200000
    idx = ug.measurement.sample(st, N, seed=9).cpu().numpy()
    assert idx.min() >= 0 and idx.max() < 2 ** n
    p = np.abs(amps) ** 2
    assert np.all(p[idx] > 0)
    # binomial test on at most 1024 contiguous bins (enough samples per bin
    # for the normal approximation)
    nb = min(2 ** n, 1024)
    pb = p.reshape(nb, -1).sum(axis=1)
    freq = np.bincount(idx // (2 ** n // nb), minlength=nb) / N
    sigma = np.sqrt(pb * (1 - pb) / N) + 1e-12
    assert np.all(np.abs(freq - pb) <= 6 * sigma + 1e-9)


@pytest.mark.parametrize("n", [4, 9, 13, 15])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_random_permutations_tiled(n, dtype):
    """permute_qubits against numpy's transpose of the tensor layout for
    random permutations, batched, including ones that move the low bits."""
    rng = np.random.default_rng(n)
    B = 3
    x = (rng.standard_normal((B, 2 ** n)) +
         1j * rng.standard_normal((B, 2 ** n))).astype(dtype)
    st = cu(x)
    for _ in range(4):
        perm = [int(p) for p in rng.permutation(n)]
        ref = x.reshape((B,) + (2,) * n).transpose(
            [0] + [1 + p for p in perm]).reshape(B, -1)
        got = ug.permute_qubits(perm, st).cpu().numpy()
        assert np.array_equal(got, ref)


def test_measure_offset_view():
    """A state viewed at an 8-byte offset (not 16-byte aligned) samples
    like the same state copied to an aligned buffer."""
    n = 12
    rng = np.random.default_rng(4)
    amps = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    amps /= np.linalg.norm(amps)
    big = torch.zeros(2 ** n + 1, dtype=torch.complex64, device=DEV)
    big[1:] = cu(amps.astype(np.complex64))
    view = big[1:]
    assert view.data_ptr() % 16 == 8
    a = ug.measurement.sample(view, 5000, seed=2).cpu().numpy()
    b = ug.measurement.sample(view.clone(), 5000, seed=2).cpu().numpy()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_tensor_layout_variants(dtype):
    """The *_tensor functions equal the vector-layout functions (pinned to
    the reference by the golden vectors) on the same states, viewed in
    tensor layout, and the contiguous permutation equals the view's copy."""
    from qcware_unitair_gb300 import gates as Gt
    from qcware_unitair_gb300.states import to_tensor_layout
    n, B = 7, 3
    g = torch.Generator(device=DEV).manual_seed(3)
    psi = torch.randn(B, 2 ** n, dtype=dtype, device=DEV, generator=g)
    T = to_tensor_layout(psi)
    rx = Gt.exp_x(0.3, dtype=dtype).to(DEV)
    cn = Gt.cnot(dtype=dtype).to(DEV)
    u3 = torch.linalg.qr(torch.randn(8, 8, dtype=dtype, device=DEV,
                                     generator=g))[0]
    eq = (lambda a, b: torch.allclose(a, b, atol=1e-6 if dtype ==
                                      torch.complex64 else 1e-13, rtol=0))
    for op, q in ((rx, [4]), (cn, [5, 1]), (u3, [6, 0, 3])):
        got = ug.simulation.apply_operator_tensor(op, q, T, n)
        assert got.shape == T.shape
        assert eq(got, to_tensor_layout(ug.apply_operator(op, q, psi)))
    got = ug.simulation.act_first_qubits_tensor(cn, T, n)
    assert eq(got, to_tensor_layout(ug.apply_operator(cn, [0, 1], psi)))
    got = ug.simulation.apply_all_qubits_tensor(rx, T, n)
    assert eq(got, to_tensor_layout(ug.apply_all_qubits(rx, psi)))
    ops = [rx, Gt.exp_z(0.7, dtype=dtype).to(DEV), rx]
    got = ug.simulation.apply_to_qubits_tensor(ops, [2, 5, 2], T, n)
    assert eq(got, to_tensor_layout(ug.apply_to_qubits(ops, [2, 5, 2],
                                                       psi)))
    # the last tensor dim contracted with the operator
    got = ug.simulation.act_last_qubit_tensor(rx, T)
    ref = torch.einsum("ab,...b->...a", rx.to(torch.complex128),
                       T.to(torch.complex128))
    assert eq(got.to(torch.complex128), ref)
    perm = [3, 0, 6, 1, 5, 2, 4]
    got = ug.simulation.permute_qubits_tensor(perm, T, n,
                                              contiguous_output=True)
    assert got.is_contiguous()
    assert torch.equal(got,
                       ug.simulation.permute_qubits_tensor(perm, T, n)
                       .contiguous())

