"""Serving: every request's result is the same alone and in the mix (the
continuous-batching test), matches the plain per-gate path and the
complex128 oracle (<= 1e-5, complex64), admission keeps the HBM budget, and
later arrivals run while earlier requests are still on the GPU."""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300.serve import (Server, _init_states, make_trace,
                                        serve_plain, summarize)

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def small_trace(num=40, seed=3, rate=400.0):
    return make_trace(num, rate=rate, seed=seed, qubits=(4, 17),
                      depth=(10, 80), batch=(1, 8), grad_fraction=0.2)


def test_results_same_alone_and_in_mix(oracle):
    trace = small_trace()
    mixed = Server(DEV, keep_states=True).serve(trace)
    assert len(mixed) == len(trace)
    for req, res in zip(trace, mixed):
        alone = Server(DEV, keep_states=True).serve([req])[0]
        assert np.abs(res.final.cpu().numpy() -
                      alone.final.cpu().numpy()).max() <= 1e-5
        assert np.abs(res.norms - alone.norms).max() <= 1e-5
        assert np.abs(res.z0 - alone.z0).max() <= 1e-5
        assert np.abs(res.norms - 1).max() <= 1e-5
        if req.want_grad:
            assert res.grads is not None
            assert np.abs(res.grads - alone.grads).max() <= 1e-5 * max(
                1.0, np.abs(alone.grads).max())
    # a few against the oracle from the same initial states
    for req, res in list(zip(trace, mixed))[:6]:
        psi0 = _init_states(req, DEV).cpu().numpy().astype(np.complex128)
        ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in req.gates],
                                 psi0)
        assert np.abs(res.final.cpu().numpy() - ref).max() <= 1e-5


def test_plain_baseline_agrees():
    trace = small_trace(num=12, seed=5)
    a = Server(DEV).serve(trace)
    b = serve_plain(trace, DEV)
    for x, y in zip(a, b):
        assert np.abs(x.norms - y.norms).max() <= 1e-5
        assert np.abs(x.z0 - y.z0).max() <= 1e-5
        if x.grads is not None:
            assert np.abs(x.grads - y.grads).max() <= 1e-4 * max(
                1.0, np.abs(y.grads).max())


def test_admission_budget_and_overlap():
    trace = make_trace(30, rate=1000.0, seed=7, qubits=(14, 20),
                       depth=(20, 60), batch=(4, 16), grad_fraction=0.0)
    budget = 3 * max(r.footprint for r in trace)
    srv = Server(DEV, budget_bytes=budget)
    res = srv.serve(trace)
    assert srv.peak_used <= budget
    # continuous batching: some request was admitted while another one
    # admitted earlier had not finished yet
    spans = sorted((r.admitted, r.done) for r in res)
    overlap = any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))
    assert overlap
    s = summarize(res)
    assert s["requests"] == 30 and s["p99_s"] >= s["p50_s"]


def test_oversized_requests_split_by_state_blocks():
    """With a budget below their footprints, requests run as parts of whole
    8-state blocks; the joined outputs equal the unsplit requests'."""
    trace = make_trace(6, rate=1000.0, seed=5, qubits=(12, 15),
                       depth=(20, 60), batch=(17, 40), grad_fraction=0.5)
    budget = max(8 * r.bytes_per_state for r in trace)  # a block fits
    whole = Server(DEV, keep_states=True).serve(trace)
    srv = Server(DEV, budget_bytes=budget, keep_states=True)
    split = srv.serve(trace)
    assert srv.peak_used <= budget
    assert any(r.footprint > budget for r in trace)
    for req, a, b in zip(trace, whole, split):
        assert a.rid == b.rid == req.rid
        assert b.norms.shape == (req.num_states,)
        assert np.array_equal(a.final.cpu().numpy(), b.final.cpu().numpy())
        assert np.abs(a.norms - b.norms).max() <= 1e-12
        assert np.abs(a.z0 - b.z0).max() <= 1e-12
        if req.want_grad:
            assert np.abs(a.grads - b.grads).max() <= 1e-6 * max(
                1.0, np.abs(a.grads).max())


def test_same_size_requests_batched_in_rounds(oracle):
    """Requests above the one-tile size that arrive together with the same
    qubit count run their stages in shared launches (gbsv_run_stages_multi);
    each result matches the request served alone and the oracle."""
    trace = make_trace(12, rate=1e6, seed=8, qubits=(15, 16),
                       depth=(30, 200), batch=(1, 4), grad_fraction=0.0)
    server = Server(DEV, keep_states=True)
    calls = []
    orig = server._launch_large_batch

    def spy(reqs):
        calls.append(len(reqs))
        return orig(reqs)
    server._launch_large_batch = spy
    mixed = server.serve(trace)
    assert calls and max(calls) >= 2
    for req, res in zip(trace, mixed):
        alone = Server(DEV, keep_states=True).serve([req])[0]
        assert np.abs(res.final.cpu().numpy() -
                      alone.final.cpu().numpy()).max() <= 1e-5
        psi0 = _init_states(req, DEV).cpu().numpy().astype(np.complex128)
        ref = oracle.run_circuit([(g.matrix(), g.qubits) for g in req.gates],
                                 psi0)
        assert np.abs(res.final.cpu().numpy() - ref).max() <= 1e-5
