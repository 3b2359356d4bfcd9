"""Property test of the broadcast descriptor that the reductions and
apply_phase kernels walk (host logic, no GPU): for random right-aligned
broadcast shapes, the per-row offsets the kernels compute from the
descriptor (rows in C order, last dim fastest, as row_offsets in
csrc/reduce.cu) equal the element offsets of numpy's broadcasting."""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300 import _lib
from qcware_unitair_gb300._core import bcast_desc, broadcast_strides

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")


def _row_offsets(d):
    """Offsets (a, b) of every row, in the kernels' row order."""
    shape = [d.shape[i] for i in range(d.ndim)]
    rows = int(np.prod(shape))
    out = []
    for r in range(rows):
        xa = xb = 0
        for i in range(d.ndim - 1, -1, -1):
            idx = r % shape[i]
            r //= shape[i]
            xa += idx * d.stride_a[i]
            xb += idx * d.stride_b[i]
        out.append((xa, xb))
    return out


@st.composite
def broadcast_pair(draw):
    nd = draw(st.integers(0, 4))
    out = [draw(st.integers(1, 4)) for _ in range(nd)]

    def operand():
        k = draw(st.integers(0, nd))
        # right-aligned trailing dims, each either the output's or 1
        return [o if draw(st.booleans()) else 1 for o in out[nd - k:]]
    return out, operand(), operand()


@hyp.settings(max_examples=200, deadline=None)
@hyp.given(broadcast_pair())
def test_descriptor_rows_match_numpy_broadcasting(pair):
    out, sa, sb = pair
    a = torch.zeros(sa) if sa else torch.zeros(())
    b = torch.zeros(sb) if sb else torch.zeros(())
    d = bcast_desc(out, broadcast_strides(a, out), broadcast_strides(b, out))
    assert 1 <= d.ndim <= _lib.MAX_DIMS
    got = _row_offsets(d)
    ia = np.broadcast_to(np.arange(a.numel()).reshape(sa), out).reshape(-1)
    ib = np.broadcast_to(np.arange(b.numel()).reshape(sb), out).reshape(-1)
    assert got == list(zip(ia.tolist(), ib.tolist()))
