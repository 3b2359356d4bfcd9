"""Tensor-core stages (gbsv_run_stage_tc) on the GPU.

Checked against the complex128 oracle at the complex64 tolerance (1e-5 max
abs amplitude error, norm drift reported), against the CPU execution of the
same records (tests/test_tc_exec.py), in place against out of place, and
against the register-blocked stages on the same circuit.  Every run must
leave the kernel's bounded-wait status at 0.
"""
import ctypes

import numpy as np
import pytest
import torch

from qcware_unitair_gb300 import _lib
from qcware_unitair_gb300 import states as S
from qcware_unitair_gb300.circuits import random_circuit, random_states, \
    zero_state
from qcware_unitair_gb300.fusion import Circuit

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def tc_status(clear=True):
    st = ctypes.c_int(-1)
    _lib.check(_lib.load().gbsv_tc_status(ctypes.byref(st), int(clear)),
               "tc_status")
    return st.value


def oracle_run(oracle, circ, psi0):
    gates = [(g.matrix.detach().cpu().numpy(), g.qubits) for g in circ.gates]
    return oracle.run_circuit(gates, psi0.astype(np.complex128))


@pytest.mark.parametrize("n,depth,batch", [(12, 300, 2), (13, 400, 3),
                                           (14, 1000, 1), (16, 300, 2),
                                           (18, 200, 1)])
def test_tc_random_circuits_vs_oracle(oracle, n, depth, batch):
    tc_status()
    circ = Circuit.from_gates(n, random_circuit(n, depth, seed=n + depth))
    prog = circ.compile(torch.complex64, DEV, tensor_cores=True)
    assert prog.tensor_cores and prog.num_passes < len(circ)
    psi0 = random_states(n, (batch,), torch.complex64, seed=n)
    out = prog.run(psi0.to(DEV))
    ref = oracle_run(oracle, circ, psi0.numpy())
    err = float(np.abs(out.cpu().numpy().astype(np.complex128) - ref).max())
    drift = float((S.norm_squared_fp64(out) - 1).abs().max())
    print(f"n={n} gates={depth} stages={prog.num_stages} "
          f"max|err|={err:.2e} norm drift={drift:.2e}")
    assert err <= 1e-5
    assert drift <= 1e-5
    st = psi0.to(DEV).clone()
    prog.run(st, inplace=True)
    assert torch.equal(st, out)
    assert tc_status() == 0


def test_tc_matches_cpu_record_execution():
    from test_tc_exec import run_tc_records
    n = 14
    circ = Circuit.from_gates(n, random_circuit(n, 250, seed=3))
    prog = circ.compile(torch.complex64, DEV, tensor_cores=True)
    psi0 = random_states(n, (2,), torch.complex64, seed=3)
    out = prog.run(psi0.to(DEV)).cpu().numpy()
    want = run_tc_records(prog, psi0.numpy().astype(np.complex128))
    assert np.abs(out - want).max() < 2e-6
    assert tc_status() == 0


def test_tc_wide_and_diagonal_gates(oracle):
    n = 15
    rng = np.random.default_rng(11)
    circ = Circuit(n)
    for step in range(120):
        k = int(rng.integers(1, 6))
        qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
        if step % 4 == 0:
            qs = qs[:2]
            m = np.diag(np.exp(1j * rng.uniform(0, 6.3, size=2 ** len(qs))))
        else:
            a = rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(
                size=(2 ** k, 2 ** k))
            m, _ = np.linalg.qr(a)
        circ.append(torch.from_numpy(m), qs)
    prog = circ.compile(torch.complex64, DEV, tensor_cores=True)
    psi0 = random_states(n, (2,), torch.complex64, seed=4)
    out = prog.run(psi0.to(DEV))
    ref = oracle_run(oracle, circ, psi0.numpy())
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-5
    assert tc_status() == 0


def test_tc_matches_register_stages():
    n = 20
    circ = Circuit.from_gates(n, random_circuit(n, 500, seed=8))
    tc = circ.compile(torch.complex64, DEV, tensor_cores=True)
    reg = circ.compile(torch.complex64, DEV, tensor_cores=False)
    psi = random_states(n, (2,), torch.complex64, seed=2).to(DEV)
    a, b = tc.run(psi), reg.run(psi)
    assert float((a - b).abs().max()) < 1e-5
    assert tc_status() == 0


def test_tc_30q_round_trip():
    """Full size: 200 random gates then their inverses return |0...0>."""
    if torch.cuda.mem_get_info()[0] < 12 * 2 ** 30:
        pytest.skip("needs 12 GiB free")
    n = 30
    circ = Circuit.from_gates(n, random_circuit(n, 200, seed=1))
    fwd = circ.compile(torch.complex64, DEV, tensor_cores=True)
    inv = circ.inverse().compile(torch.complex64, DEV, tensor_cores=True)
    psi = zero_state(n, (), torch.complex64, DEV)
    fwd.run(psi, inplace=True)
    norm = float(S.norm_squared_fp64(psi))
    inv.run(psi, inplace=True)
    err0 = abs(complex(psi[0].item()) - 1)
    psi[0] = 0
    rest = float(psi.abs().max())
    del psi
    torch.cuda.empty_cache()
    assert abs(norm - 1) < 1e-5
    assert err0 < 1e-5 and rest < 1e-5
    assert tc_status() == 0
