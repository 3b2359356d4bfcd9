"""qcware_unitair_gb300 -- a GB300-native state-vector engine.

Drop-in for unitair's hot path: ``simulation.apply_operator``,
``apply_all_qubits``, ``apply_phase`` and the ``states`` reductions, on the
same torch tensors (vector layout, qubit 0 = most significant index bit,
unitair's batch broadcasting).  Every operation is a hand-written sm_103a
CUDA kernel reached through the C ABI in include/gbsv.h; CUDA tensors only.
"""
from . import gates, states, simulation, initializations, utils  # noqa: F401
from .states import (StateLayout, StateShapeError, count_qubits,  # noqa
                     hilbert_space_dim, diag_expectation_value,
                     inner_product, norm_squared, abs_squared)
from .simulation import (apply_operator, apply_operator_, apply_all_qubits,  # noqa
                         apply_each_qubit, apply_phase, act_first_qubits,
                         apply_to_qubits, act_last_qubit, swap,
                         permute_qubits, roll_qubits, multi_cz,
                         multi_controlled_z, multi_controlled_x)
from .measurement import measure, MeasurementHistogram  # noqa
from .fusion import Circuit, Program  # noqa
from .initializations import (unit_vector, uniform_superposition,  # noqa
                              rand_state)
from . import library  # noqa: F401  (torch.ops.gbsv.*)
from ._lib import (set_complex128_arithmetic,  # noqa: F401
                   complex128_arithmetic)

VECTOR_LAYOUT = StateLayout.VECTOR
TENSOR_LAYOUT = StateLayout.TENSOR

__version__ = "0.1.0"
