"""Small, fixed workloads for timing and profiling the kernels one at a time.

    python -m qcware_unitair_gb300.workloads stage 26          # random circuit
    python -m qcware_unitair_gb300.workloads gates 24 H 64     # one stage, 64 H
    python -m qcware_unitair_gb300.workloads adjoint 16        # 20q ansatz grad
    python -m qcware_unitair_gb300.workloads serve 300         # server only
    python -m qcware_unitair_gb300.workloads kinds 28          # c128 per gate

Each runs its workload twice (a warm-up, then a CUDA-event-timed run) and
prints one line; under a profiler, skip the first run's launches.

``stage``: the canonical random circuit (``circuits.random_circuit``, numpy
seed 0) on n qubits, 200 gates, complex64, compiled into fused stages and run
in place from |0...0>.

``gates``: one fused stage on n qubits holding 8 Hadamards on spread tile
bits plus k copies of one gate kind (H, X, RX, or RZout = RZ on a bit that is
never a register bit), for the per-gate cost of the stage kernel.

``adjoint``: forward + adjoint backward of the 20-qubit, 12-layer
hardware-efficient ansatz (RY, RZ per qubit, CZ ring) at the given batch,
loss mean(<sum Z> + 0.5 <sum XX>).

``serve``: the serving trace of the benchmark (Poisson 150 requests/s,
10-22 qubits, depth 20-500, 1-64 states, 20% adjoint gradients) replayed
once against the continuous-batching server after a 16-request warm-up,
with the host time of the server's launch paths.

``kinds``: one plain gate of each canonical kind (angle 0.7 for rotations)
applied in place to an n-qubit complex128 state, 10 launches after 2
warm-up launches each, ms per launch and GB/s over one read and one write
of the state.
"""
from __future__ import annotations

import sys

import torch


def _timed(fn):
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def stage(n: int = 26, gates: int = 200) -> float:
    from .circuits import random_circuit, zero_state
    from .fusion import Circuit
    dev = torch.device("cuda")
    prog = Circuit.from_gates(n, random_circuit(n, gates, seed=0)).compile(
        torch.complex64, dev)
    psi = zero_state(n, (), torch.complex64, dev)
    ms = _timed(lambda: prog.run(psi, inplace=True))
    print(f"stage n={n} gates={gates} passes={prog.num_passes} {ms:.3f} ms")
    return ms


def gates(n: int = 24, kind: str = "H", k: int = 64) -> float:
    from .circuits import gate_matrix
    from .fusion import Circuit
    dev = torch.device("cuda")

    def q(bit):
        return n - 1 - bit

    c = Circuit(n)
    for b in (6, 8, 10, 12, 14, 16, 18, 20):
        c.h(q(b))
    for i in range(k):
        if kind == "H":
            c.h(q(0))
        elif kind == "X":
            c.x(q(0))
        elif kind == "RX":
            c.append(gate_matrix("RX", 0.3 + i), [q(0)], "dense")
        elif kind == "RZout":
            c.append(gate_matrix("RZ", 0.3 + i), [q(5)], "diag")
        else:
            raise ValueError(f"unknown gate kind {kind}")
    prog = c.compile(torch.complex64, dev, tile_qubits=12)
    psi = torch.randn(2 ** n, dtype=torch.complex64, device=dev)
    ms = _timed(lambda: prog.run(psi, inplace=True))
    print(f"gates n={n} kind={kind} k={k} passes={prog.num_passes} "
          f"{ms:.3f} ms")
    return ms


def adjoint(batch: int = 16, n: int = 20, layers: int = 12) -> float:
    from .adjoint import PauliSum, expectation, hardware_efficient_ansatz
    dev = torch.device("cuda")
    pc = hardware_efficient_ansatz(n, layers)
    H = PauliSum(n)
    for i in range(n):
        H.z(i)
    for i in range(n - 1):
        H.xx(i, i + 1, coeff=0.5)
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    params = torch.randn(batch, pc.num_params, generator=g, device=dev)

    def step():
        p = params.clone().requires_grad_()
        expectation(pc, p, H).mean().backward()
        return p.grad

    ms = _timed(step)
    print(f"adjoint n={n} layers={layers} batch={batch} {ms:.3f} ms")
    return ms


def serve(num: int = 300) -> float:
    import collections
    import time
    from . import serve as S
    dev = torch.device("cuda")
    spent = collections.defaultdict(float)

    def timed(obj, name, key):
        f = getattr(obj, name)

        def w(*a, **k):
            t = time.perf_counter()
            try:
                return f(*a, **k)
            finally:
                spent[key] += time.perf_counter() - t
        setattr(obj, name, w)
        return f

    warm = S.make_trace(16, rate=1000.0, seed=99, qubits=(10, 22),
                        depth=(20, 100))
    S.Server(dev).serve(warm)
    saved = [(S.Server, "_launch_small",
              timed(S.Server, "_launch_small", "small launches")),
             (S.Server, "_launch_large",
              timed(S.Server, "_launch_large", "large launches")),
             (S, "_run_grad", timed(S, "_run_grad", "gradient requests"))]
    try:
        trace = S.make_trace(num, rate=150.0, seed=0, qubits=(10, 22))
        res = S.summarize(S.Server(dev).serve(trace))
    finally:
        for obj, name, f in saved:
            setattr(obj, name, f)
    print(f"serve {res}; host seconds: "
          + ", ".join(f"{k} {v:.3f}" for k, v in spent.items()))
    return res["circuits_per_s"]


def kinds(n: int = 28) -> None:
    import qcware_unitair_gb300 as ug
    from .circuits import gate_matrix
    dev = torch.device("cuda")
    psi = torch.randn(2 ** n, dtype=torch.complex128, device=dev)
    psi /= psi.abs().pow(2).sum().sqrt()
    cases = [("X", [5]), ("H", [5]), ("RY", [5]), ("RX", [5]), ("RZ", [5]),
             ("T", [5]), ("Z", [5]), ("Y", [5]), ("CNOT", [3, 20]),
             ("CZ", [3, 20]), ("SWAP", [3, 20]), ("X", [n - 1]),
             ("RX", [n - 1]), ("CNOT", [n - 2, n - 1])]
    for name, q in cases:
        theta = 0.7 if name.startswith("R") else None
        m = torch.from_numpy(gate_matrix(name, theta)).to(dev)
        for _ in range(2):
            ug.apply_operator_(m, q, psi)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            ug.apply_operator_(m, q, psi)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        print(f"kinds n={n} {name} {q}: {ms:.3f} ms "
              f"{2 * 16 * 2 ** n / ms / 1e6:.0f} GB/s")


if __name__ == "__main__":
    what, args = sys.argv[1], sys.argv[2:]
    if what == "stage":
        stage(*(int(a) for a in args))
    elif what == "gates":
        gates(int(args[0]) if args else 24, args[1] if len(args) > 1 else "H",
              int(args[2]) if len(args) > 2 else 64)
    elif what == "adjoint":
        adjoint(*(int(a) for a in args))
    elif what == "serve":
        serve(*(int(a) for a in args))
    elif what == "kinds":
        kinds(*(int(a) for a in args))
    else:
        raise SystemExit(f"unknown workload {what}")
