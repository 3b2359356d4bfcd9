"""torch.ops.gbsv.* give the same results as the engine's functions, trace
into one graph under torch.compile (the fake implementations supply the
shapes) and differentiate like the functions do."""
import pytest
import torch

import qcware_unitair_gb300 as ug
from qcware_unitair_gb300.circuits import random_states

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _ops(dtype=torch.complex64):
    g = torch.Generator().manual_seed(0)
    a = torch.randn(4, 4, dtype=dtype, generator=g)
    q, _ = torch.linalg.qr(a)
    psi = random_states(10, (3,), dtype, seed=1).to(DEV)
    return q.to(DEV), psi


def test_ops_match_functions():
    u, psi = _ops()
    got = torch.ops.gbsv.apply_operator(u, [2, 7], psi)
    assert torch.equal(got, ug.apply_operator(u, [2, 7], psi))
    angles = torch.rand(2 ** 10, device=DEV)
    assert torch.equal(torch.ops.gbsv.apply_phase(angles, psi),
                       ug.apply_phase(angles, psi))
    assert torch.equal(torch.ops.gbsv.norm_squared(psi),
                       ug.norm_squared(psi))
    assert torch.equal(torch.ops.gbsv.abs_squared(psi), ug.abs_squared(psi))
    assert torch.equal(torch.ops.gbsv.inner_product(psi, got),
                       ug.inner_product(psi, got))


def test_compile_traces_one_graph():
    u, psi = _ops()

    def f(u, psi):
        x = torch.ops.gbsv.apply_operator(u, [0, 3], psi)
        x = torch.ops.gbsv.apply_operator(u, [5, 1], x)
        return torch.ops.gbsv.norm_squared(x), x

    cf = torch.compile(f, backend="aot_eager", fullgraph=True)
    n1, x1 = cf(u, psi)
    n0, x0 = f(u, psi)
    assert torch.equal(x1, x0) and torch.equal(n1, n0)


def test_ops_differentiate_like_functions():
    u, psi = _ops()
    for use_op in (True, False):
        uu = u.clone().requires_grad_()
        pp = psi.clone().requires_grad_()
        fn = torch.ops.gbsv.apply_operator if use_op else ug.apply_operator
        out = fn(uu, [1, 4], pp)
        loss = (out.abs() ** 2 * torch.arange(out.shape[-1], device=DEV)
                ).sum()
        loss.backward()
        if use_op:
            g_op = (uu.grad.clone(), pp.grad.clone())
        else:
            g_fn = (uu.grad.clone(), pp.grad.clone())
    assert torch.allclose(g_op[0], g_fn[0], atol=1e-5)
    assert torch.allclose(g_op[1], g_fn[1], atol=1e-5)
