"""Serving host logic on CPU: the synthetic trace and its accounting."""
import numpy as np
import pytest

from qcware_unitair_gb300.serve import Request, make_trace


def test_trace_distribution():
    tr = make_trace(2000, rate=100.0, seed=1)
    arr = np.array([r.arrival for r in tr])
    assert np.all(np.diff(arr) > 0)
    assert abs(np.mean(np.diff(arr)) - 0.01) < 0.002  # Poisson at 100/s
    ns = [r.num_qubits for r in tr]
    assert min(ns) == 10 and max(ns) == 28
    ds = [len(r.gates) for r in tr]
    assert min(ds) >= 20 and max(ds) <= 500
    bs = [r.num_states for r in tr]
    assert min(bs) == 1 and max(bs) == 64
    g = np.mean([r.want_grad for r in tr])
    assert 0.17 < g < 0.23


def test_footprint():
    r = Request(0, 0.0, 28, 64, [], want_grad=False)
    assert r.state_bytes == 64 * 2 ** 28 * 8  # the largest request: 128 GiB
    assert r.footprint <= 160e9
    assert Request(1, 0.0, 10, 2, [], want_grad=True).footprint == \
        6 * 2 * 2 ** 10 * 8


def test_split_into_whole_state_blocks():
    """A request over the budget becomes parts of whole 8-state blocks that
    each fit and together cover its states in order; one that fits, or
    whose single block does not, stays whole."""
    from qcware_unitair_gb300.serve import STATE_BLOCK
    big = Request(3, 1.5, 28, 64, [], want_grad=True, seed=11)
    assert big.footprint > 160e9  # 768 GiB with gradients
    parts = big.split(160e9)
    assert len(parts) > 1
    assert [p.state_offset for p in parts] == sorted(
        p.state_offset for p in parts)
    k = 0
    for p in parts:
        assert p.state_offset == k and p.state_offset % STATE_BLOCK == 0
        assert p.footprint <= 160e9
        assert (p.rid, p.arrival, p.seed, p.want_grad) == (3, 1.5, 11, True)
        k += p.num_states
    assert k == 64
    small = Request(4, 0.0, 20, 5, [], want_grad=True)
    assert small.split(160e9) == [small]
    huge = Request(5, 0.0, 33, 8, [], want_grad=True)  # one block > budget
    assert huge.split(160e9) == [huge]


def test_merge_parts_joins_in_state_order():
    """The outputs of a split request's parts are joined by state offset,
    whatever order the parts finished in."""
    from qcware_unitair_gb300.serve import Result, _merge_parts
    def part(off, k, admitted, done, grads=True):
        return (off, Result(7, np.arange(off, off + k, dtype=float),
                            -np.arange(off, off + k, dtype=float),
                            np.full((k, 3), off, dtype=float) if grads
                            else None, 1.0, admitted, done))
    merged = _merge_parts([part(16, 4, 2.5, 3.0), part(0, 8, 1.5, 4.0),
                           part(8, 8, 2.0, 3.5)])
    assert merged.rid == 7
    assert merged.norms.tolist() == list(range(20))
    assert merged.z0.tolist() == [-float(i) for i in range(20)]
    assert merged.grads.shape == (20, 3)
    assert merged.grads[:, 0].tolist() == [0.0] * 8 + [8.0] * 8 + [16.0] * 4
    assert (merged.arrival, merged.admitted, merged.done) == (1.0, 1.5, 4.0)
    assert merged.final is None
    plain = _merge_parts([part(0, 8, 1.0, 2.0, False),
                          part(8, 2, 1.0, 2.0, False)])
    assert plain.grads is None and plain.norms.shape == (10,)


def test_split_properties():
    """Any request and budget: the parts cover the states once, in order,
    in whole 8-state blocks, and each fits the budget whenever one block
    does."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from qcware_unitair_gb300.serve import STATE_BLOCK

    @hyp.settings(max_examples=300, deadline=None)
    @hyp.given(n=st.integers(1, 30), states=st.integers(1, 200),
               grad=st.booleans(), budget=st.floats(1e3, 3e11))
    def check(n, states, grad, budget):
        req = Request(1, 0.5, n, states, [], want_grad=grad, seed=3)
        parts = req.split(budget)
        assert sum(p.num_states for p in parts) == states
        k = 0
        for p in parts:
            assert p.state_offset == k
            k += p.num_states
        if len(parts) > 1:
            assert all(p.state_offset % STATE_BLOCK == 0 for p in parts)
            assert all(p.footprint <= budget for p in parts)
        else:
            assert parts[0] is req
            assert (req.footprint <= budget or
                    STATE_BLOCK * req.bytes_per_state > budget)

    check()
