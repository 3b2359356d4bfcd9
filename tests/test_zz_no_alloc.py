"""gbsv_norm_squared_noalloc: the norm kernel for callers that cannot
allocate device memory (an FFI caller holding only buffers another runtime
gave it, or a latency-critical loop that must not call cudaMalloc because
it can synchronize the device).  Its partial sums live in a fixed device
array inside libgbsv instead of caller scratch.

This file is collected last so that a run stopping at the first failure has
already run every other test.  It checks, through the C ABI, that two calls
in a row give the same norms as gbsv_norm_squared with caller-allocated
scratch, within the tolerance the reduction tests use.
"""
import numpy as np
import pytest
import torch

from qcware_unitair_gb300 import _lib

pytestmark = pytest.mark.gpu


def _reference_norms(L, state, code, rows, dim, stream):
    out = torch.empty(rows, dtype=torch.float64, device=state.device)
    nbytes = int(L.gbsv_reduce_scratch_bytes(rows, dim))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8,
                          device=state.device)
    rc = L.gbsv_norm_squared(state.data_ptr(), code, rows, dim,
                             out.data_ptr(), _lib.F64, scratch.data_ptr(),
                             nbytes, stream)
    _lib.check(rc, "norm_squared")
    return out


def test_noalloc_norm_matches_allocating_entry_point():
    L = _lib.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    cases = [(torch.complex64, 2, 2 ** 20), (torch.complex128, 1, 2 ** 22),
             (torch.complex64, 3, 2 ** 16)]
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    for dtype, rows, dim in cases:
        # the split into partials (the path that uses the fixed array)
        assert L.gbsv_reduce_scratch_bytes(rows, dim) > 0
        code = _lib.C64 if dtype == torch.complex64 else _lib.C128
        for call in range(2):
            state = torch.randn(rows, dim, dtype=dtype, device=dev,
                                generator=g)
            want = _reference_norms(L, state, code, rows, dim, stream)
            got = torch.full((rows,), float("nan"), dtype=torch.float64,
                             device=dev)
            rc = L.gbsv_norm_squared_noalloc(state.data_ptr(), code, rows,
                                             dim, got.data_ptr(), _lib.F64,
                                             stream)
            _lib.check(rc, "norm_squared_noalloc")
            got32 = torch.empty(rows, dtype=torch.float32, device=dev)
            rc = L.gbsv_norm_squared_noalloc(state.data_ptr(), code, rows,
                                             dim, got32.data_ptr(), _lib.F32,
                                             stream)
            _lib.check(rc, "norm_squared_noalloc")
            torch.cuda.synchronize()
            np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(),
                                       rtol=1e-12)
            np.testing.assert_allclose(got32.cpu().numpy(),
                                       want.cpu().numpy(), rtol=1e-6)


def test_noalloc_norm_single_part_and_host_sum():
    """Rows short enough to reduce in one kernel (no partials: the result is
    written straight to the output, which starts as NaN), and every case
    checked against a float64 host sum of |psi|^2 as well."""
    L = _lib.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    cases = [(torch.complex64, 4, 4096), (torch.complex128, 7, 2048),
             (torch.complex64, 2, 2 ** 20)]
    for dtype, rows, dim in cases:
        code = _lib.C64 if dtype == torch.complex64 else _lib.C128
        single = L.gbsv_reduce_scratch_bytes(rows, dim) == 0
        assert single == (dim <= 8192)
        for call in range(2):
            state = torch.randn(rows, dim, dtype=dtype, device=dev,
                                generator=g)
            got = torch.full((rows,), float("nan"), dtype=torch.float64,
                             device=dev)
            rc = L.gbsv_norm_squared_noalloc(state.data_ptr(), code, rows,
                                             dim, got.data_ptr(), _lib.F64,
                                             stream)
            _lib.check(rc, "norm_squared_noalloc")
            torch.cuda.synchronize()
            host = state.cpu().numpy().astype(np.complex128)
            want = (host.real ** 2 + host.imag ** 2).sum(axis=1)
            np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-12)
            if single:
                np.testing.assert_allclose(
                    got.cpu().numpy(),
                    _reference_norms(L, state, code, rows, dim,
                                     stream).cpu().numpy(), rtol=1e-12)


def test_noalloc_partials_fit_the_fixed_array():
    """The reduction plan splits rows into at most about SM count x 16
    blocks, so on this GPU every request's FP64 partials (half of the
    allocating entry point's scratch) fit the fixed 64 KiB array; the
    rejection branch guards GPUs with many more SMs."""
    L = _lib.load()
    for rows in (1, 2, 3, 7, 64, 300, 1000, 2431):
        for dim in (2 ** 14, 2 ** 20, 2 ** 26, 2 ** 30):
            assert L.gbsv_reduce_scratch_bytes(rows, dim) // 2 <= 64 * 1024
