"""The C-ABI library builds, loads without a GPU and exports exactly what
include/gbsv.h declares; argument errors come back as status codes without
touching the device."""
import ctypes
import re
from pathlib import Path

import pytest

from qcware_unitair_gb300 import _lib, build_lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "gbsv.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsv_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gbsv_apply_operator" in names
    assert "gbsv_norm_squared" in names
    assert len(names) >= 12


def test_library_exports_every_declared_symbol(lib_built):
    L = ctypes.CDLL(str(lib_built))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_status_codes_without_gpu(lib_built):
    L = _lib.load()
    assert L.gbsv_abi_version() == 1
    assert L.gbsv_status_string(0) == b"ok"
    q = _lib.qubit_array([0])
    # bad dtype, bad qubit, repeated qubit: rejected before any CUDA call
    assert L.gbsv_apply_operator(None, None, 7, 3, 1, 8, None, 0, q, 1,
                                 None) == _lib.GBSV_ERR_INVALID_ARG
    q5 = _lib.qubit_array([5])
    assert L.gbsv_apply_operator(1, 1, _lib.C64, 3, 1, 8, 1, 0, q5, 1,
                                 None) == _lib.GBSV_ERR_INVALID_ARG
    assert b"out of range" in L.gbsv_last_error()
    q11 = _lib.qubit_array([1, 1])
    assert L.gbsv_apply_operator(1, 1, _lib.C64, 3, 1, 8, 1, 0, q11, 2,
                                 None) == _lib.GBSV_ERR_INVALID_ARG
    assert b"repeated" in L.gbsv_last_error()
    # zero states: nothing to do, nothing launched
    before = L.gbsv_launch_count()
    assert L.gbsv_apply_operator(None, None, _lib.C64, 3, 0, 8, None, 0, q,
                                 1, None) == 0
    assert L.gbsv_launch_count() == before
    assert L.gbsv_norm_squared(None, _lib.C64, 1, 8, None, 9, None, 0,
                               None) == _lib.GBSV_ERR_INVALID_ARG


def test_scratch_sizing_is_consistent(lib_built):
    L = _lib.load()
    # small rows: one block per row, no scratch
    assert L.gbsv_reduce_scratch_bytes(64, 4096) == 0


def test_engine_refuses_cpu_tensors():
    """No CPU fallback: a CPU tensor is an error, not a slow path."""
    import torch
    import qcware_unitair_gb300 as ug
    with pytest.raises(RuntimeError, match="CUDA"):
        ug.apply_operator(torch.eye(2, dtype=torch.complex64), [0],
                          torch.ones(4, dtype=torch.complex64))
    with pytest.raises(RuntimeError, match="CUDA"):
        ug.norm_squared(torch.ones(4, dtype=torch.complex64))


def test_complex128_arithmetic_switch_without_gpu(lib_built):
    """gbsv_set_c128_arith / gbsv_get_c128_arith: both modes round-trip, an
    unknown mode is rejected and leaves the setting alone; no device call."""
    L = _lib.load()
    prev = L.gbsv_get_c128_arith()
    try:
        assert L.gbsv_set_c128_arith(1) == 0
        assert L.gbsv_get_c128_arith() == 1
        assert L.gbsv_set_c128_arith(0) == 0
        assert L.gbsv_get_c128_arith() == 0
        assert L.gbsv_set_c128_arith(7) == _lib.GBSV_ERR_INVALID_ARG
        assert b"unknown complex128 arithmetic mode" in L.gbsv_last_error()
        assert L.gbsv_get_c128_arith() == 0
        import qcware_unitair_gb300 as ug
        assert ug.set_complex128_arithmetic("fp64") == "pairs"
        assert ug.complex128_arithmetic() == "fp64"
        with pytest.raises(ValueError):
            ug.set_complex128_arithmetic("double")
    finally:
        L.gbsv_set_c128_arith(prev)


def test_inplace_rule_matches_the_library(lib_built):
    """_core.inplace_ok (which tells callers when to go through a
    temporary) agrees with gbsv_apply_operator: every in-place request it
    marks unsupported is refused with GBSV_ERR_UNSUPPORTED before any CUDA
    call (dummy pointers, never dereferenced).  Supported requests would
    launch kernels and are not called here; with a GPU present the test
    is skipped, so that a disagreement can never reach a launch."""
    import torch
    from qcware_unitair_gb300 import _core
    if torch.cuda.is_available():
        pytest.skip("dummy pointers: run without a GPU")
    L = _lib.load()
    p = 4096  # dummy device address
    for dtype, code in ((torch.complex64, _lib.C64),
                        (torch.complex128, _lib.C128)):
        for k in range(3, 13):
            for n in (k, k + 1, k + 3, k + 8):
                for per_state in (False, True):
                    if _core.inplace_ok(dtype, k, n, per_state):
                        continue
                    q = _lib.qubit_array(list(range(k)))
                    rc = L.gbsv_apply_operator(
                        p, p, code, n, 2, 2 ** n, p,
                        4 ** k if per_state else 0, q, k, None)
                    assert rc == _lib.GBSV_ERR_UNSUPPORTED, (dtype, k, n,
                                                             per_state)
                    assert b"in place" in L.gbsv_last_error()
    # complex64 wide operators: in place for shared operators at any size,
    # per-state ones once a state holds a whole tile of groups
    assert _core.inplace_ok(torch.complex64, 12, 12)
    assert not _core.inplace_ok(torch.complex64, 6, 12, True)
    assert _core.inplace_ok(torch.complex64, 6, 13, True)
    assert _core.inplace_ok(torch.complex64, 12, 13, True)
    assert not _core.inplace_ok(torch.complex128, 5, 20)
    # a strided batch in place is refused even for a shared operator
    q = _lib.qubit_array(list(range(7)))
    assert L.gbsv_apply_operator(p, p, _lib.C64, 9, 3, 2 ** 9 + 6, p, 0, q,
                                 7, None) == _lib.GBSV_ERR_UNSUPPORTED
