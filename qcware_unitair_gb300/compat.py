"""Swap the GB300 engine into an installed ``unitair`` package.

    import unitair
    from qcware_unitair_gb300 import compat
    compat.install()          # unitair.simulation.apply_operator -> engine

After install(), unitair's module attributes for the hot path point at the
engine functions, including the module-level names that unitair's own
wrappers call (e.g. multi_controlled_x calls operations.apply_operator,
src/unitair/simulation/operations.py:793-805).  uninstall() restores them.

The engine computes on CUDA tensors only.  ``move_cpu_tensors=True``
installs adapters that copy CPU inputs to ``device``, run the kernels there
and copy the results back -- the computation still happens on the GPU; it
exists so that code written for CPU tensors (such as unitair's own tests)
can drive the engine unchanged.
"""
from __future__ import annotations

import functools
import importlib

import torch

from . import measurement, simulation, states

# unitair.simulation.operations functions replaced by the engine (same
# signatures, operations.py:15-805).
_OPERATIONS = {
    "apply_operator": simulation.apply_operator,
    "apply_all_qubits": simulation.apply_all_qubits,
    "apply_phase": simulation.apply_phase,
    "act_first_qubits": simulation.act_first_qubits,
    "act_last_qubit": simulation.act_last_qubit,
    "apply_to_qubits": simulation.apply_to_qubits,
    "swap": simulation.swap,
    "permute_qubits": simulation.permute_qubits,
    "roll_qubits": simulation.roll_qubits,
    "multi_cz": simulation.multi_cz,
    "multi_controlled_z": simulation.multi_controlled_z,
    "multi_controlled_x": simulation.multi_controlled_x,
    # tensor-layout variants (operations.py:151-654)
    "apply_operator_tensor": simulation.apply_operator_tensor,
    "act_first_qubits_tensor": simulation.act_first_qubits_tensor,
    "act_last_qubit_tensor": simulation.act_last_qubit_tensor,
    "apply_all_qubits_tensor": simulation.apply_all_qubits_tensor,
    "apply_to_qubits_tensor": simulation.apply_to_qubits_tensor,
    "swap_tensor": simulation.swap_tensor,
    "roll_qubits_tensor": simulation.roll_qubits_tensor,
    "permute_qubits_tensor": simulation.permute_qubits_tensor,
}
_SIM_EXPORTS = ("apply_operator", "apply_all_qubits", "apply_phase",
                "act_first_qubits", "act_last_qubit", "apply_to_qubits",
                "swap", "multi_cz", "multi_controlled_z",
                "multi_controlled_x")

_TARGETS = {
    "unitair.simulation.operations": dict(_OPERATIONS),
    "unitair.simulation": dict(
        {k: _OPERATIONS[k] for k in _SIM_EXPORTS},
        measure=measurement.measure),
    "unitair.simulation.measurement": {"measure": measurement.measure},
    "unitair.states.innerprod": {
        "inner_product": states.inner_product,
        "norm_squared": states.norm_squared,
        "abs_squared": states.abs_squared,
        "diag_expectation_value": states.diag_expectation_value,
    },
    "unitair.states": {
        "inner_product": states.inner_product,
        "norm_squared": states.norm_squared,
        "abs_squared": states.abs_squared,
        "diag_expectation_value": states.diag_expectation_value,
    },
    "unitair": {
        "inner_product": states.inner_product,
        "norm_squared": states.norm_squared,
        "abs_squared": states.abs_squared,
        "diag_expectation_value": states.diag_expectation_value,
    },
}

_saved: dict = {}


def _has_cpu_tensor(x) -> bool:
    if isinstance(x, torch.Tensor):
        return not x.is_cuda
    if isinstance(x, (list, tuple)):
        return any(_has_cpu_tensor(v) for v in x)
    return False


def _to(x, device):
    if isinstance(x, torch.Tensor):
        return x.to(device)
    if isinstance(x, (list, tuple)):
        return type(x)(_to(v, device) for v in x)
    return x


def _mover(fn, device):
    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        if not (_has_cpu_tensor(args) or _has_cpu_tensor(list(
                kwargs.values()))):
            return fn(*args, **kwargs)
        out = fn(*_to(args, device),
                 **{k: _to(v, device) for k, v in kwargs.items()})
        return _to(out, "cpu")
    return wrapper


def install(move_cpu_tensors: bool = False, device="cuda") -> list:
    """Patch unitair; return the list of replaced 'module.name' entries."""
    replaced = []
    for modname, funcs in _TARGETS.items():
        try:
            mod = importlib.import_module(modname)
        except ImportError:
            continue
        for name, fn in funcs.items():
            if not hasattr(mod, name):
                continue
            key = (modname, name)
            if key not in _saved:
                _saved[key] = getattr(mod, name)
            setattr(mod, name, _mover(fn, device) if move_cpu_tensors else fn)
            replaced.append(f"{modname}.{name}")
    return replaced


def uninstall() -> None:
    for (modname, name), fn in _saved.items():
        setattr(importlib.import_module(modname), name, fn)
    _saved.clear()
