"""Renormalisation checkpoints (gbsv_renormalize, Program.run(renorm_every))
against the complex128 oracle: deep circuits keep their norm while every
amplitude stays within the complex64 tolerance (1e-5 max abs)."""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300 import _lib
from qcware_unitair_gb300 import states as S
from qcware_unitair_gb300.circuits import random_circuit, random_states
from qcware_unitair_gb300.fusion import Circuit

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


@pytest.mark.parametrize("dtype,rtol", [(torch.complex64, 2e-6),
                                        (torch.complex128, 1e-12)])
@pytest.mark.parametrize("rows,dim", [(3, 2 ** 10), (2, 2 ** 20),
                                      (5, 64)])
def test_renormalize_sets_target_norms(dtype, rtol, rows, dim):
    L = _lib.load()
    g = torch.Generator(device=DEV)
    g.manual_seed(rows + dim)
    psi = torch.randn(rows, dim, dtype=dtype, device=DEV, generator=g)
    before = psi.clone()
    target = torch.rand(rows, dtype=torch.float64, device=DEV,
                        generator=g) + 0.5
    norms = torch.full((rows,), float("nan"), dtype=torch.float64,
                       device=DEV)
    nbytes = int(L.gbsv_reduce_scratch_bytes(rows, dim))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=DEV)
    code = _lib.C64 if dtype == torch.complex64 else _lib.C128
    stream = torch.cuda.current_stream(DEV).cuda_stream
    rc = L.gbsv_renormalize(psi.data_ptr(), code, rows, dim,
                            target.data_ptr(), norms.data_ptr(),
                            scratch.data_ptr(), nbytes, stream)
    _lib.check(rc, "renormalize")
    host = before.cpu().numpy().astype(np.complex128)
    want_before = (np.abs(host) ** 2).sum(axis=1)
    np.testing.assert_allclose(norms.cpu().numpy(), want_before, rtol=1e-12)
    after = S.norm_squared_fp64(psi).cpu().numpy()
    np.testing.assert_allclose(after, target.cpu().numpy(), rtol=rtol)
    # a per-row positive scale: directions are unchanged
    ratio = psi.cpu().numpy().astype(np.complex128) / host
    scale = np.sqrt(target.cpu().numpy() / want_before)
    np.testing.assert_allclose(ratio, np.broadcast_to(scale[:, None],
                                                      ratio.shape),
                               rtol=10 * rtol, atol=0)


def test_10000_gate_circuit_with_checkpoints(oracle):
    """14 qubits, complex64, 10,000 random gates on the fused engine: with
    a checkpoint every 8 passes the norm stays at 1 and the amplitudes
    within 1e-5 of the complex128 oracle; the drift the checkpoints removed
    and the drift without them are reported."""
    n, depth = 14, 10000
    gates = random_circuit(n, depth, seed=21)
    circ = Circuit.from_gates(n, gates)
    prog = circ.compile(torch.complex64, DEV)
    psi0 = random_states(n, (2,), torch.complex64, seed=21)
    ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in gates],
                             psi0.numpy().astype(np.complex128))
    plain = prog.run(psi0.to(DEV))
    drift_plain = float((S.norm_squared_fp64(plain) - 1).abs().max())
    err_plain = float(np.abs(plain.cpu().numpy() - ref).max())
    ck = prog.run(psi0.to(DEV), renorm_every=8)
    removed = prog.renorm_drift()
    drift_ck = float((S.norm_squared_fp64(ck) - 1).abs().max())
    err_ck = float(np.abs(ck.cpu().numpy() - ref).max())
    print(f"passes={prog.num_passes} tensor_cores={prog.tensor_cores} "
          f"without checkpoints: drift {drift_plain:.2e} max|err| "
          f"{err_plain:.2e}; with: drift {drift_ck:.2e} max|err| "
          f"{err_ck:.2e}, largest drift removed {removed:.2e}")
    assert err_ck <= 1e-5
    # what is left is the drift of the passes after the last checkpoint
    assert drift_ck <= 5e-6
    assert removed > 0.0
