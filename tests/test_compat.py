"""compat.install(): the engine replaces unitair's hot-path functions.

A stand-in ``unitair`` module tree (same module names and attributes as
unitair 0.3.0: src/unitair/__init__.py, simulation/__init__.py,
simulation/operations.py, simulation/measurement.py, states/__init__.py,
states/innerprod.py) is placed in sys.modules, so the test needs no
unitair install.
"""
import sys
import types

import numpy as np
import pytest
import torch

from qcware_unitair_gb300 import compat, measurement, simulation, states

_MODULES = {
    "unitair": ["inner_product", "norm_squared", "abs_squared",
                "diag_expectation_value"],
    "unitair.simulation": ["apply_operator", "apply_all_qubits",
                           "apply_phase", "act_first_qubits",
                           "act_last_qubit", "apply_to_qubits", "swap",
                           "multi_cz", "multi_controlled_z",
                           "multi_controlled_x", "measure"],
    "unitair.simulation.operations": [
        "apply_operator", "apply_all_qubits", "apply_phase",
        "act_first_qubits", "act_last_qubit", "apply_to_qubits", "swap",
        "permute_qubits", "roll_qubits", "multi_cz", "multi_controlled_z",
        "multi_controlled_x", "apply_operator_tensor",
        "act_first_qubits_tensor", "act_last_qubit_tensor",
        "apply_all_qubits_tensor", "apply_to_qubits_tensor", "swap_tensor",
        "roll_qubits_tensor", "permute_qubits_tensor"],
    "unitair.simulation.measurement": ["measure"],
    "unitair.states": ["inner_product", "norm_squared", "abs_squared",
                       "diag_expectation_value"],
    "unitair.states.innerprod": ["inner_product", "norm_squared",
                                 "abs_squared", "diag_expectation_value"],
}


def _sentinel(name):
    def f(*a, **k):
        return ("original", name)
    return f


@pytest.fixture
def fake_unitair(monkeypatch):
    for modname, names in _MODULES.items():
        mod = types.ModuleType(modname)
        for name in names:
            setattr(mod, name, _sentinel(name))
        monkeypatch.setitem(sys.modules, modname, mod)
    yield
    compat.uninstall()


def test_install_replaces_every_hot_path_name(fake_unitair):
    replaced = compat.install()
    expected = {f"{m}.{n}" for m, names in _MODULES.items() for n in names}
    assert set(replaced) == expected
    ops = sys.modules["unitair.simulation.operations"]
    assert ops.apply_operator is simulation.apply_operator
    assert ops.multi_controlled_x is simulation.multi_controlled_x
    assert ops.permute_qubits is simulation.permute_qubits
    assert sys.modules["unitair.simulation"].measure is measurement.measure
    assert sys.modules["unitair"].norm_squared is states.norm_squared


def test_uninstall_restores(fake_unitair):
    compat.install()
    compat.uninstall()
    for modname, names in _MODULES.items():
        for name in names:
            assert getattr(sys.modules[modname], name)() == ("original", name)


def test_mover_passes_cuda_free_calls_through():
    calls = []

    def fn(*a, **k):
        calls.append((a, k))
        return 7

    w = compat._mover(fn, "cuda")
    assert w(1, [2, 3], x=4) == 7
    assert calls == [((1, [2, 3]), {"x": 4})]


def test_mover_finds_nested_cpu_tensors():
    t = torch.zeros(2)
    assert compat._has_cpu_tensor([1, (t,)])
    assert not compat._has_cpu_tensor([1, (2,)])
    moved = compat._to([t, (t, 3)], "cpu")
    assert isinstance(moved, list) and isinstance(moved[1], tuple)


def test_engine_rejects_cpu_tensors_without_mover(fake_unitair):
    compat.install()
    ops = sys.modules["unitair.simulation.operations"]
    psi = torch.zeros(4, dtype=torch.complex64)
    h = torch.eye(2, dtype=torch.complex64)
    with pytest.raises(RuntimeError):
        ops.apply_operator(h, [0], psi)


@pytest.mark.gpu
def test_installed_engine_with_cpu_tensors_matches_oracle(fake_unitair):
    from oracle import oracle
    compat.install(move_cpu_tensors=True)
    ops = sys.modules["unitair.simulation.operations"]
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((3, 64)) + 1j * rng.standard_normal((3, 64))
    op = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    out = ops.apply_operator(torch.from_numpy(op).to(torch.complex128), [2],
                             torch.from_numpy(psi))
    assert out.device.type == "cpu"
    ref = oracle.apply_operator(op, [2], psi)
    assert np.abs(out.numpy() - ref).max() < 1e-12
    # list-of-tensors arguments move too
    ops2 = [torch.from_numpy(op).to(torch.complex128)] * 2
    out2 = ops.apply_to_qubits(ops2, [1, 4], torch.from_numpy(psi))
    ref2 = oracle.apply_operator(op, [4], oracle.apply_operator(op, [1], psi))
    assert np.abs(out2.numpy() - ref2).max() < 1e-12
    pairs = torch.tensor([[0, 1], [2, 5]])
    out3 = ops.multi_cz(pairs, torch.from_numpy(psi))
    assert out3.device.type == "cpu"
