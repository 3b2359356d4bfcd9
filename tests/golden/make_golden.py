"""Generate golden vectors by running the reference (unitair 0.3.0) itself.

Run from the repository root in a container that has the reference source:

    python tests/golden/make_golden.py /path/to/qcware-unitair

It imports ``unitair`` from ``<reference>/src`` with torch on the CPU, feeds
it seeded inputs and writes
  tests/golden/golden.npz   inputs and the reference's outputs
  tests/golden/cases.json   case metadata, including the exception type the
                            reference raises for each rejected input
The engine's tests and the oracle's pin-tests read only these files; the
reference is not needed at test time.
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def main(ref_root: str) -> None:
    sys.path.insert(0, str(Path(ref_root) / "src"))
    sys.path.insert(0, str(REPO))
    import unitair  # noqa: F401
    from unitair import gates as G
    from unitair import states as S
    from unitair.simulation import (apply_all_qubits, apply_operator,
                                    apply_phase)
    from qcware_unitair_gb300.circuits import random_circuit

    torch.manual_seed(1234)
    rng = np.random.default_rng(1234)
    arrays: dict = {}
    cases: list = []

    def cplx(shape, dtype):
        a = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        return torch.from_numpy(a).to(dtype)

    def put(name, **kw):
        for k, v in kw.items():
            if isinstance(v, torch.Tensor):
                v = v.detach().numpy()
            arrays[f"{name}/{k}"] = np.asarray(v)

    # ---- known answers from the reference's README / tutorial ----------
    h0 = apply_operator(G.hadamard(), [0], unitair.unit_vector(0, 1))
    put("kat_h0", out=h0)
    cases.append({"name": "kat_h0", "kind": "kat"})
    bell = apply_operator(G.hadamard(), [0], unitair.unit_vector(0, 2))
    bell = apply_operator(G.cnot(), [0, 1], bell)
    put("kat_bell", out=bell)
    cases.append({"name": "kat_bell", "kind": "kat"})
    put("kat_expx", out=G.exp_x(0.5))
    cases.append({"name": "kat_expx", "kind": "kat"})
    t = torch.arange(0, math.pi, 0.01)
    put("kat_expx_batch", t=t,
        out=apply_operator(G.exp_x(t), [0], unitair.unit_vector(0, 1)))
    cases.append({"name": "kat_expx_batch", "kind": "kat"})

    # ---- apply_operator over batch structures, orders and dtypes ---------
    batch_specs = [
        ((), ()), ((), (3,)), ((3,), ()), ((2, 3), (2, 3)), ((3,), (2, 3)),
        ((1, 3), (2, 3)), ((2, 1), (2, 3)), ((4,), (4,)), ((1, 1, 3), (2, 3)),
    ]
    qubit_specs = {
        1: lambda n: [[0], [n - 1], [n // 2]],
        2: lambda n: [[0, n - 1], [n - 1, 0], [n - 2, n - 1], [n - 1, n - 2],
                      [1, 0]],
        3: lambda n: [[0, n - 1, 1], [n - 1, 0, n - 2]],
    }
    idx = 0
    for dtype in (torch.complex64, torch.complex128):
        for n in (1, 2, 3, 5, 8):
            for k in (1, 2, 3):
                if k > n:
                    continue
                for qs in qubit_specs[k](n):
                    if len(set(qs)) != k or min(qs) < 0:
                        continue
                    ob, sb = batch_specs[idx % len(batch_specs)]
                    idx += 1
                    op = cplx(ob + (2 ** k, 2 ** k), dtype)
                    st = cplx(sb + (2 ** n,), dtype)
                    out = apply_operator(op, qs, st)
                    name = f"apply_{idx}"
                    put(name, op=op, state=st, out=out)
                    cases.append({"name": name, "kind": "apply",
                                  "qubits": qs, "n": n, "k": k,
                                  "dtype": str(dtype)})
    # every batch structure at a mid size with a 1- and a 2-qubit gate
    for dtype in (torch.complex64, torch.complex128):
        for ob, sb in batch_specs:
            for qs in ([3], [4, 1]):
                idx += 1
                k = len(qs)
                op = cplx(ob + (2 ** k, 2 ** k), dtype)
                st = cplx(sb + (2 ** 6,), dtype)
                out = apply_operator(op, qs, st)
                name = f"apply_{idx}"
                put(name, op=op, state=st, out=out)
                cases.append({"name": name, "kind": "apply", "qubits": qs,
                              "n": 6, "k": k, "dtype": str(dtype)})
    # a 10-qubit state batch with every single target position
    for dtype in (torch.complex64, torch.complex128):
        st = cplx((2, 2 ** 10), dtype)
        shared = f"state10_{str(dtype)[-3:]}"
        put(shared, state=st)
        for q in range(10):
            idx += 1
            op = cplx((2, 2), dtype)
            name = f"apply_{idx}"
            put(name, op=op, out=apply_operator(op, [q], st))
            cases.append({"name": name, "kind": "apply", "qubits": [q],
                          "n": 10, "k": 1, "dtype": str(dtype),
                          "state_key": f"{shared}/state"})
    # k = 0 (scalar operator) and k = 4
    for qs, n in (([], 3), ([2, 0, 5, 3], 6)):
        idx += 1
        k = len(qs)
        op = cplx((2 ** k, 2 ** k), torch.complex64)
        st = cplx((2, 2 ** n), torch.complex64)
        name = f"apply_{idx}"
        put(name, op=op, state=st, out=apply_operator(op, qs, st))
        cases.append({"name": name, "kind": "apply", "qubits": qs, "n": n,
                      "k": k, "dtype": "torch.complex64"})

    # ---- apply_all_qubits --------------------------------------------------
    for j, (dtype, n, ob, sb) in enumerate([
            (torch.complex64, 1, (), ()), (torch.complex64, 4, (), (3,)),
            (torch.complex64, 7, (3,), (3,)), (torch.complex128, 5, (3,), ()),
            (torch.complex128, 6, (), (2, 2))]):
        op = cplx(ob + (2, 2), dtype)
        st = cplx(sb + (2 ** n,), dtype)
        name = f"allq_{j}"
        put(name, op=op, state=st, out=apply_all_qubits(op, st))
        cases.append({"name": name, "kind": "all_qubits", "n": n,
                      "dtype": str(dtype)})

    # ---- apply_phase -----------------------------------------------------
    for j, (adt, sdt, ashape, sshape) in enumerate([
            (torch.float32, torch.complex64, (32,), (32,)),
            (torch.float32, torch.complex64, (2, 3, 16), (2, 3, 16)),
            (torch.float32, torch.complex64, (16,), (4, 16)),
            (torch.float32, torch.complex64, (4, 1), (4, 16)),
            (torch.float32, torch.complex64, (), (4, 16)),
            (torch.float64, torch.complex64, (16,), (16,)),
            (torch.float32, torch.complex128, (3, 8), (3, 8)),
            (torch.float64, torch.complex128, (3, 8), (8,))]):
        ang = torch.from_numpy(rng.uniform(-7, 7, size=ashape)).to(adt)
        st = cplx(sshape, sdt)
        name = f"phase_{j}"
        put(name, angles=ang, state=st, out=apply_phase(ang, st))
        cases.append({"name": name, "kind": "phase"})

    # ---- reductions -------------------------------------------------------
    for j, (dtype, sa, sb) in enumerate([
            (torch.complex64, (5, 64), (5, 64)),
            (torch.complex128, (64,), (3, 64)),
            (torch.complex64, (2, 1, 32), (1, 3, 32))]):
        a, b = cplx(sa, dtype), cplx(sb, dtype)
        name = f"inner_{j}"
        put(name, a=a, b=b, out=S.inner_product(a, b))
        cases.append({"name": name, "kind": "inner"})
    for j, (dtype, shape) in enumerate([(torch.complex64, (3, 4, 128)),
                                        (torch.complex128, (256,)),
                                        (torch.complex64, (2, 2 ** 14))]):
        s = cplx(shape, dtype)
        name = f"norm_{j}"
        put(name, state=s, out=S.norm_squared(s))
        if s.numel() <= 4096:
            put(name, abs2=S.abs_squared(s))
        cases.append({"name": name, "kind": "norm"})
    for j, (ddt, sdt, dshape, sshape) in enumerate([
            (torch.float32, torch.complex64, (64,), (3, 64)),
            (torch.float64, torch.complex64, (3, 64), (3, 64)),
            (torch.float32, torch.complex128, (2, 1, 16), (3, 16))]):
        d = torch.from_numpy(rng.normal(size=dshape)).to(ddt)
        s = cplx(sshape, sdt)
        name = f"diag_{j}"
        put(name, diag=d, state=s, out=S.diag_expectation_value(d, s))
        cases.append({"name": name, "kind": "diag"})

    # ---- autograd through apply_operator ----------------------------------
    for j, (ob, sb, qs, n) in enumerate([((), (3,), [1], 4),
                                         ((3,), (3,), [2, 0], 4),
                                         ((3,), (), [0], 3),
                                         ((4,), (2, 4), [1, 3], 5)]):
        k = len(qs)
        op = cplx(ob + (2 ** k, 2 ** k), torch.complex128).requires_grad_()
        st = cplx(sb + (2 ** n,), torch.complex128).requires_grad_()
        out = apply_operator(op, qs, st)
        w = cplx(out.shape, torch.complex128)
        loss = (out * w).real.sum() + (out.conj() * out).real.sum()
        loss.backward()
        name = f"grad_{j}"
        put(name, op=op, state=st, w=w, out=out, gop=op.grad, gstate=st.grad)
        cases.append({"name": name, "kind": "grad", "qubits": qs, "n": n})

    # ---- permutations, apply_to_qubits, multi-controlled gates ----------
    from unitair.simulation.operations import (
        swap, permute_qubits, roll_qubits, apply_to_qubits, multi_cz,
        multi_controlled_z, multi_controlled_x)
    for j, (dtype, shape) in enumerate([(torch.complex64, (3, 2 ** 6)),
                                        (torch.complex128, (2 ** 5,))]):
        st = cplx(shape, dtype)
        n = 6 if len(shape) == 2 else 5
        name = f"perm_{j}"
        put(name, state=st,
            swap=swap(st, (1, n - 1)), swap_neg=swap(st, (0, -1)),
            perm=permute_qubits(list(reversed(range(n))), st),
            perm2=permute_qubits([2, 0, 1] + list(range(3, n)), st),
            roll1=roll_qubits(st, 1), roll3=roll_qubits(st, 3),
            rollm=roll_qubits(st, -2))
        cases.append({"name": name, "kind": "perm", "n": n})
    for j, (dtype, ob) in enumerate([(torch.complex64, ()),
                                     (torch.complex128, ())]):
        n = 5
        st = cplx((3, 2 ** n), dtype)
        qs = [0, 3, 0, 4, 1, 3]
        ops = [cplx(ob + (2, 2), dtype) for _ in qs]
        name = f"tq_{j}"
        put(name, state=st, ops=torch.stack(ops),
            out=apply_to_qubits(ops, qs, st))
        cases.append({"name": name, "kind": "to_qubits", "qubits": qs})
    st = cplx((2, 2 ** 6), torch.complex64)
    pairs = torch.tensor([[0, 1], [2, 5], [1, 4], [0, 1]])
    put("mcz_0", state=st, pairs=pairs, out=multi_cz(pairs, st),
        single=multi_cz(torch.tensor([3, 1]), st),
        mcz=multi_controlled_z([1, 4, 2], st),
        mcx=multi_controlled_x(st, [0, 5], 2))
    cases.append({"name": "mcz_0", "kind": "multi"})

    # ---- variational gradient through unitair + torch autograd -----------
    # ansatz: per layer, on every qubit RZ(phi) then RY(theta) (U = RY RZ),
    # then a CZ ring; loss = mean_b <sum_i Z_i + 0.5 sum_i X_i X_{i+1}>.
    # unitair's exp_* return complex64, so the rotation matrices are built
    # here in float64 (RY(t) = exp_y(t/2), RZ(t) = exp_z(t/2)).
    n, B, layers = 5, 2, 2
    params = torch.from_numpy(rng.normal(size=(B, layers, n, 2)))
    params.requires_grad_()
    psi = torch.zeros(B, 2 ** n, dtype=torch.complex128)
    psi[:, 0] = 1
    cz = torch.diag(torch.tensor([1, 1, 1, -1], dtype=torch.complex128))
    for l in range(layers):
        for q in range(n):
            ph = params[:, l, q, 1] / 2
            rz = torch.zeros(B, 2, 2, dtype=torch.complex128)
            rz[:, 0, 0] = torch.exp(-1j * ph)
            rz[:, 1, 1] = torch.exp(1j * ph)
            psi = apply_operator(rz, [q], psi)
            th = params[:, l, q, 0] / 2
            c, s_ = torch.cos(th), torch.sin(th)
            ry = torch.stack([torch.stack([c, -s_], -1),
                              torch.stack([s_, c], -1)], -2).to(
                                  torch.complex128)
            psi = apply_operator(ry, [q], psi)
        for q in range(n):
            psi = apply_operator(cz, [q, (q + 1) % n], psi)
    zdiag = torch.zeros(2 ** n, dtype=torch.float64)
    idx = torch.arange(2 ** n)
    for q in range(n):
        zdiag += 1 - 2 * ((idx >> (n - 1 - q)) & 1).to(torch.float64)
    energy = S.diag_expectation_value(zdiag, psi)
    xx = torch.tensor([[0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0],
                       [1, 0, 0, 0]], dtype=torch.complex128)
    for q in range(n - 1):
        energy = energy + 0.5 * S.inner_product(
            psi, apply_operator(xx, [q, q + 1], psi)).real
    energy.mean().backward()
    put("ansatz_grad", params=params.detach(), energy=energy.detach(),
        grad=params.grad)
    cases.append({"name": "ansatz_grad", "kind": "ansatz", "n": n,
                  "layers": layers})

    # ---- circuits (canonical generator) -----------------------------------
    for name, n, batch, depth, seed, dtype in (
            ("circ_c64", 12, 4, 200, 0, torch.complex64),
            ("circ_c128", 10, 2, 1000, 1, torch.complex128)):
        torch.manual_seed(seed)
        st0 = unitair.rand_state(n, batch_dims=(batch,), dtype=dtype)
        st = st0
        for g in random_circuit(n, depth, seed=seed):
            m = torch.from_numpy(g.matrix()).to(dtype)
            st = apply_operator(m, list(g.qubits), st)
        put(name, state=st0, out=st, norms=S.norm_squared(st))
        cases.append({"name": name, "kind": "circuit", "n": n,
                      "depth": depth, "seed": seed, "dtype": str(dtype)})

    # ---- rejected inputs: which exception the reference raises ----------
    errors = []
    specs = [
        ("apply_operator", (2, 2), (5,), [0], "c64", "c64"),
        ("apply_operator", (2, 2), (8,), [3], "c64", "c64"),
        ("apply_operator", (2, 2), (8,), [-1], "c64", "c64"),
        ("apply_operator", (4, 4), (8,), [0], "c64", "c64"),
        ("apply_operator", (3, 3), (8,), [0], "c64", "c64"),
        ("apply_operator", (2, 2), (8,), [0], "c128", "c64"),
        ("apply_operator", (3, 2, 2), (3, 5, 16), [1], "c64", "c64"),
        ("apply_operator", (3, 5, 2, 2), (1, 5, 16), [1], "c64", "c64"),
        ("apply_operator", (7, 2, 2), (1, 16), [1], "c64", "c64"),
        ("apply_operator", (4, 4), (8,), [1, 1], "c64", "c64"),
        ("apply_all_qubits", (4, 4), (8,), None, "c64", "c64"),
        ("apply_operator", (2, 2), (3, 8), [2], "c64", "c64"),
        ("apply_operator", (5, 2, 2), (3, 5, 16), [0], "c64", "c64"),
        ("apply_operator", (1, 3, 5, 2, 2), (3, 5, 16), [0], "c64", "c64"),
    ]
    dt = {"c64": torch.complex64, "c128": torch.complex128}
    for fn, oshape, sshape, qs, odt, sdt in specs:
        op = torch.ones(oshape, dtype=dt[odt])
        st = torch.ones(sshape, dtype=dt[sdt])
        try:
            if fn == "apply_operator":
                r = apply_operator(op, qs, st)
            else:
                r = apply_all_qubits(op, st)
            result = {"ok": list(r.shape)}
        except Exception as e:  # noqa: BLE001 - record the reference's type
            result = {"error": type(e).__name__}
        errors.append({"fn": fn, "op_shape": list(oshape),
                       "state_shape": list(sshape), "qubits": qs,
                       "op_dtype": odt, "state_dtype": sdt, **result})

    # ---- operators on 6-8 qubits (drawn last: earlier cases keep their
    # random inputs) -----------------------------------------------------
    wide_specs = [
        # (operator batch, state batch, n, qubits, dtype)
        ((), (2,), 8, [5, 0, 7, 2, 6, 3], torch.complex64),   # bit 0 targeted
        ((), (3,), 7, [6, 1, 4, 0, 3, 5], torch.complex128),
        ((), (3,), 7, [3, 6, 0, 5, 1, 4, 2], torch.complex64),  # n == k
        ((), (), 10, [0, 2, 4, 6, 8, 1, 3, 5], torch.complex64),
        ((3,), (), 9, [8, 1, 4, 6, 2, 0], torch.complex64),   # state broadcast
    ]
    for j, (ob, sb, n, qs, dtype) in enumerate(wide_specs):
        k = len(qs)
        op = cplx(ob + (2 ** k, 2 ** k), dtype) / 2 ** (k / 2)
        st = cplx(sb + (2 ** n,), dtype)
        name = f"apply_wide_{j}"
        put(name, op=op, state=st, out=apply_operator(op, qs, st))
        cases.append({"name": name, "kind": "apply", "qubits": qs, "n": n,
                      "k": k, "dtype": str(dtype)})
    # ---- 5-qubit operators (drawn after the wide cases) -----------------
    for j, (ob, sb, n, qs, dtype) in enumerate([
            ((2,), (2,), 7, [4, 6, 0, 2, 5], torch.complex64),
            ((), (3,), 6, [5, 3, 1, 0, 2], torch.complex128)]):
        k = len(qs)
        op = cplx(ob + (2 ** k, 2 ** k), dtype) / 2 ** (k / 2)
        st = cplx(sb + (2 ** n,), dtype)
        name = f"apply_k5_{j}"
        put(name, op=op, state=st, out=apply_operator(op, qs, st))
        cases.append({"name": name, "kind": "apply", "qubits": qs, "n": n,
                      "k": k, "dtype": str(dtype)})

    np.savez_compressed(HERE / "golden.npz", **arrays)
    meta = {"reference": "unitair 0.3.0 (setup.cfg:3)",
            "torch": torch.__version__, "cases": cases, "errors": errors}
    (HERE / "cases.json").write_text(json.dumps(meta, indent=1))
    print(f"{len(cases)} cases, {len(errors)} error specs, "
          f"{(HERE / 'golden.npz').stat().st_size} bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py "
                         "<path of the unitair source tree>")
    main(sys.argv[1])
