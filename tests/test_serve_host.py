"""Serving host logic on CPU: the synthetic trace and its accounting."""
import numpy as np

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
