"""The torch.library registrations load without a GPU and name the
operations the engine exports to torch's dispatcher."""
import torch

import qcware_unitair_gb300  # noqa: F401


def test_ops_registered():
    for name in ("apply_operator", "apply_phase", "norm_squared",
                 "abs_squared", "inner_product"):
        op = getattr(torch.ops.gbsv, name)
        assert op.default._schema.name == f"gbsv::{name}"
    schema = str(torch.ops.gbsv.apply_operator.default._schema)
    assert "[] qubits" in schema and "Tensor state" in schema
