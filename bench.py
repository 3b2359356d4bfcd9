"""Benchmark: 30-qubit complex64 state, 1,000 random gates, one kernel per
gate -- algorithmic HBM GB/s and fraction of the measured copy peak.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = the whole 1,000-gate circuit (canonical generator, seed 0) from
|0...0> over the 8 GiB state.  Algorithmic bytes = 2 x 8 B x 2^30 per gate
(each amplitude read once and written once).  The state is 64x larger than
L2, so no flush is needed between steps.

value:   device-timed (CUDA events around the timed steps), state resident.
e2e:     the same metric through the public functional API
         (qcware_unitair_gb300.apply_operator) with the initial state copied
         from pinned host memory and the final state copied back inside
         the timed region.
roofline: dense gate kernel, per-launch CUDA-event durations.
cpu_baseline / --impl reference: the oracle's complex64 C port of the
         reference path (OpenMP, all host threads) on the first gates of
         the same circuit.
Multi-GPU: replicas only (each rank runs its own state), scaling "weak".
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "30q c64 HBM GB/s & %peak; served circuits/s, p50/p99 vs plain " \
         "per-gate path"
WORKLOAD = ("{n}-qubit complex64 state from |0...0>, {g} random "
            "gates from {{H,X,Y,Z,S,T,RX,RY,RZ,CNOT,CZ,SWAP}}, one kernel per "
            "gate")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--qubits", type=int, default=30)
    p.add_argument("--gates", type=int, default=1000)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the adjoint and serving measurements")
    p.add_argument("--workload", nargs="+", default=None,
                   help="run one small profiling workload (see the "
                        "workloads section) instead of the benchmark")
    return p.parse_args()


def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def sm_max_mhz():
    """Maximum SM clock of the GB300s (MEASURED_PEAKS.json; 2070 MHz
    nominal otherwise)."""
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        v = json.loads(f.read_text()).get("sm_max_mhz")
        if v:
            return float(v)
    return 2070.0


# DRAM bytes (read + write) of one dense_chunk_kernel launch on a 30-qubit
# complex64 state: ncu dram__bytes_read.sum + dram__bytes_write.sum of a
# 26-qubit capture, scaled by 16 (traffic is proportional to the state; a
# 30-qubit capture is beyond the capture-size rule).
DENSE_GATE_TRAFFIC_30Q = 16_238_000_000
DENSE_GATE_TRAFFIC_SOURCE = "ncu 26q x16"


# ----------------------------------------------------------- distributed --
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float, backend_device=None) -> float:
    """Max of a float across ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([value], dtype=torch.float64,
                     device=backend_device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while timing."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(f"/tmp/gbsv_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "note": "nvidia-smi unavailable"}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "note": "no samples"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------- CPU baseline --
def cpu_sample(n: int, gates, budget_s: float):
    """Time the oracle's complex64 port (all host threads) on the first gates
    of the circuit, in place on an n-qubit state, until budget_s passes."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    psi = np.zeros(2 ** n, dtype=np.complex64)
    psi[0] = 1
    done, t0 = 0, time.perf_counter()
    L = O.lib()
    import ctypes
    for g in gates:
        m = np.ascontiguousarray(g.matrix().astype(np.complex64))
        q = (ctypes.c_int * len(g.qubits))(*g.qubits)
        rc = L.oracle_apply_c64(psi.ctypes.data, psi.ctypes.data, 1, n, 0,
                                m.ctypes.data, 0, q, len(g.qubits))
        if rc:
            raise RuntimeError("oracle rejected a gate")
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    gbs = done * 2 * 8 * 2 ** n / dt / 1e9
    return {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"first {done} gates of the {n}-qubit circuit, "
                      f"in place, {dt:.1f} s",
            "s_per_gate": dt / done}


# ------------------------------------------------- variational gradient ---
def _tfim(n):
    from qcware_unitair_gb300.adjoint import PauliSum
    H = PauliSum(n)
    for q in range(n):
        H.z(q)
    for q in range(n - 1):
        H.xx(q, q + 1, 0.5)
    return H


def _autograd_plain_loss(pc, p, H, n):
    """The same loss through torch autograd over the per-gate path."""
    import torch
    import qcware_unitair_gb300 as ug
    B = p.shape[0]
    psi = torch.zeros(B, 2 ** n, dtype=torch.complex64, device=p.device)
    psi[:, 0] = 1
    fns = {"X": ug.gates.rx, "Y": ug.gates.ry, "Z": ug.gates.rz}
    fixed = {}
    for op in pc.ops:
        if op[0] == "rot":
            _, gen, q, pi, scale = op
            psi = ug.apply_operator(fns[gen](p[:, pi] * scale), [q], psi)
        else:
            key = id(op[1])
            if key not in fixed:
                fixed[key] = op[1].to(device=p.device, dtype=torch.complex64)
            psi = ug.apply_operator(fixed[key], list(op[2]), psi)
    idx = torch.arange(2 ** n, device=p.device)
    zdiag = sum(1 - 2 * ((idx >> (n - 1 - q)) & 1).float() for q in range(n))
    e = ug.diag_expectation_value(zdiag, psi)
    xx = torch.tensor([[0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0], [1, 0, 0, 0]],
                      dtype=torch.complex64, device=p.device)
    for q in range(n - 1):
        e = e + 0.5 * ug.inner_product(psi, ug.apply_operator(
            xx, [q, q + 1], psi)).real
    return e.mean()


def bench_adjoint(dev, n=20, layers=12, batch=256, small_batch=8):
    """Forward + adjoint backward of the 20-qubit hardware-efficient ansatz
    (batch 256, 12 layers, complex64, loss = mean <sum Z + 0.5 sum XX>), and
    the same gradient through torch autograd over the plain per-gate path
    at a batch whose saved states fit in memory."""
    import torch
    from qcware_unitair_gb300.adjoint import (expectation,
                                              hardware_efficient_ansatz)
    pc = hardware_efficient_ansatz(n, layers)
    H = _tfim(n)
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    params = torch.randn(batch, pc.num_params, generator=g, device=dev)

    def adj(pp):
        p = pp.clone().requires_grad_()
        expectation(pc, p, H).mean().backward()
        return p.grad

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    t_full = timed(lambda: adj(params), 2)
    small = params[:small_batch].contiguous()
    t_adj_small = timed(lambda: adj(small), 3)

    def ag():
        p = small.clone().requires_grad_()
        _autograd_plain_loss(pc, p, H, n).backward()
        return p.grad

    ga = ag()
    gb = adj(small)
    agree = float((ga - gb).abs().max() / gb.abs().max())
    t_ag_small = timed(ag, 2)
    torch.cuda.empty_cache()
    return {"workload": f"{n}-qubit hardware-efficient ansatz, {layers} "
                        f"layers of RY.RZ + CZ ring, complex64, loss mean "
                        "<sum Z_i + 0.5 sum X_i X_i+1>",
            "batch": batch, "params": batch * pc.num_params,
            "s_per_step_forward_backward": round(t_full, 4),
            "compare_batch": small_batch,
            "adjoint_s": round(t_adj_small, 4),
            "autograd_plain_s": round(t_ag_small, 4),
            "speedup_vs_autograd": round(t_ag_small / t_adj_small, 2),
            "grad_rel_diff_vs_autograd": agree}


# ------------------------------------------------------- small-state configs
def _cuda_time(fn, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_c0(dev):
    """12 qubits x 64 random states, complex64, 200 canonical gates: the
    plain per-gate path (apply_operator per gate) against the whole circuit
    as one fused launch (each state is one 4096-amplitude tile)."""
    import torch
    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300.circuits import random_circuit, random_states
    from qcware_unitair_gb300.fusion import Circuit
    n, B, G = 12, 64, 200
    gates = random_circuit(n, G, seed=0)
    psi0 = random_states(n, (B,), torch.complex64, seed=0).to(dev)
    mats = [torch.from_numpy(g.matrix()).to(dev, torch.complex64)
            for g in gates]

    def plain():
        st = psi0
        for g, m in zip(gates, mats):
            st = ug.apply_operator(m, g.qubits, st)
        return ug.norm_squared(st)

    prog = Circuit.from_gates(n, gates).compile(torch.complex64, dev)

    def fused():
        return ug.norm_squared(prog.run(psi0))

    a = plain()
    b = fused()
    return {"workload": "12 qubits x 64 states, complex64, 200 random gates, "
                        "final states and norms",
            "plain_ms": round(_cuda_time(plain, 5), 3),
            "fused_ms": round(_cuda_time(fused, 20), 4),
            "fused_launches": prog.num_passes + 1,
            "max_norm_diff": float((a - b).abs().max())}


def bench_c2(dev, layers=100):
    """4096 states x 16 qubits (batch (64, 64)), complex64: 100 layers of
    per-state RX, RY, RZ on every qubit (angles (64, 64, 16) ~ U[0, 2pi))
    and a CNOT ladder i -> i+1.  The fused layer program is captured once
    as a CUDA graph of all layers and replayed; the plain path launches one
    kernel per gate.  Plus the broadcast case: one 16-qubit state under
    4096 gate batches."""
    import math
    import torch
    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300.adjoint import (ParamCircuit, _forward_program,
                                              _rotation_values)
    from qcware_unitair_gb300.circuits import random_states
    n, B = 16, 4096
    pc = ParamCircuit(n, 3 * n)
    for q in range(n):
        pc.rx(q, 3 * q)
        pc.ry(q, 3 * q + 1)
        pc.rz(q, 3 * q + 2)
    for q in range(n - 1):
        pc.cnot(q, q + 1)
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    angles = torch.rand(layers, B, 3 * n, generator=g, device=dev,
                        dtype=torch.float32) * (2 * math.pi)
    psi0 = random_states(n, (B,), torch.complex64, seed=2).to(dev)
    prog, which, _ = _forward_program(pc, 0, len(pc.ops), B,
                                      torch.complex64, dev, True)
    idx = torch.cat([torch.arange(off, off + B * nv, device=dev)
                     for _, _, _, off, nv in which])
    vals = torch.stack([_rotation_values(which, angles[l], B,
                                         torch.complex64)
                        for l in range(layers)])
    psi = psi0.clone()

    def circuit():
        for l in range(layers):
            prog.pool.index_copy_(0, idx, vals[l])
            prog.run(psi, inplace=True)

    circuit()  # warm-up outside capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream(dev)
    stream.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            circuit()
    torch.cuda.current_stream(dev).wait_stream(stream)

    def replay():
        psi.copy_(psi0)
        graph.replay()

    graph_ms = _cuda_time(replay, 3)
    fused_out = psi.clone()
    # plain path: one kernel per gate, per-state 2x2 matrices
    rx = ug.gates.rx
    ry = ug.gates.ry
    rz = ug.gates.rz
    cnot = ug.gates.cnot(device=dev)

    def plain():
        st = psi0
        for l in range(layers):
            a = angles[l].view(B, n, 3)
            for q in range(n):
                st = ug.apply_operator(rx(a[:, q, 0]), [q], st)
                st = ug.apply_operator(ry(a[:, q, 1]), [q], st)
                st = ug.apply_operator(rz(a[:, q, 2]), [q], st)
            for q in range(n - 1):
                st = ug.apply_operator(cnot, [q, q + 1], st)
        return st

    plain_out = plain()
    diff = float((plain_out - fused_out).abs().max())
    plain_ms = _cuda_time(plain, 1)
    # broadcast: one state, 4096 operator batches
    one = psi0[0].contiguous()
    ops = rx(angles[0].view(B, n, 3)[:, 0, 0])
    bc_ms = _cuda_time(lambda: ug.apply_operator(ops, [0], one), 10)
    bc_bytes = 2 ** n * 8 * (1 + B)
    return {"workload": f"4096 x 16 qubits complex64, {layers} layers of "
                        "per-state RX, RY, RZ on every qubit + CNOT ladder",
            "graph_ms": round(graph_ms, 2), "plain_ms": round(plain_ms, 1),
            "speedup": round(plain_ms / graph_ms, 2),
            "passes_per_layer": prog.num_passes,
            "max_abs_diff_fused_vs_plain": diff,
            "broadcast_1x4096_ms": round(bc_ms, 4),
            "broadcast_GBs": round(bc_bytes / (bc_ms / 1e3) / 1e9, 1)}


# ----------------------------------------------- the path's other rows ----
def bench_path_rows(dev, n=30):
    """apply_phase, the state reductions, apply_all_qubits and a 3-qubit
    operator on a 30-qubit complex64 state (8 GiB).  Algorithmic bytes per
    amplitude: phase 20 (angle 4 + read 8 + write 8), norm 8, inner product
    16, |psi|^2 12 (read 8, write 4), diagonal expectation 12, a gate pass
    16."""
    import numpy as np
    import torch
    import qcware_unitair_gb300 as ug
    N = 2 ** n
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    psi = torch.randn(N, dtype=torch.complex64, device=dev, generator=g)
    psi /= torch.linalg.vector_norm(psi)
    psi2 = torch.roll(psi, 1)
    angles = torch.rand(N, device=dev, generator=g)
    diag = torch.rand(N, device=dev, generator=g)
    peak = peaks()[0]
    h = torch.tensor([[1, 1], [1, -1]], dtype=torch.complex64,
                     device=dev) / np.sqrt(2)
    rng = np.random.default_rng(1)
    u3 = np.linalg.qr(rng.standard_normal((8, 8)) +
                      1j * rng.standard_normal((8, 8)))[0]
    u3 = torch.from_numpy(u3).to(dev, torch.complex64)
    cases = [
        ("apply_phase(float32 angles)", lambda: ug.apply_phase(angles, psi),
         20, 1),
        ("norm_squared", lambda: ug.norm_squared(psi), 8, 1),
        ("inner_product", lambda: ug.inner_product(psi, psi2), 16, 1),
        ("abs_squared", lambda: ug.abs_squared(psi), 12, 1),
        ("diag_expectation_value",
         lambda: ug.diag_expectation_value(diag, psi), 12, 1),
        ("apply_all_qubits(H)", lambda: ug.apply_all_qubits(h, psi), 16, n),
        ("apply_operator(3 qubits)",
         lambda: ug.apply_operator(u3, [3, 14, n - 3], psi), 16, 1),
    ]
    out = {}
    for name, fn, bpa, passes in cases:
        ms = _cuda_time(fn, 3)
        gbs = bpa * N * passes / (ms / 1e3) / 1e9
        out[name] = {"ms": round(ms, 3), "passes": passes,
                     "GB_s": round(gbs, 1),
                     "frac_of_peak": round(gbs / peak, 3)}
        torch.cuda.empty_cache()
    return {"workload": f"{n}-qubit complex64 state ({8 * 2 ** n / 2 ** 30:g} GiB), functional API",
            "peak_GBs": peak, "ops": out}


# ------------------------------------------------- next-row operations ----
def bench_next_rows(dev, n=30):
    """The operations around the gate path on a 30-qubit complex64 state
    (8 GiB, far above L2): qubit permutations (swap, permute, roll), the
    phase-flip pass of multi_cz, multi-controlled X, apply_to_qubits with
    one random single-qubit operator per qubit (fused), and sampling 2^20
    outcomes.  Algorithmic bytes: a functional copy-like pass reads and
    writes the state (16 B / amplitude); sampling reads it once (8 B)."""
    import numpy as np
    import torch
    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300.measurement import sample
    N = 2 ** n
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    psi = torch.randn(N, dtype=torch.complex64, device=dev, generator=g)
    psi /= torch.linalg.vector_norm(psi)
    peak = peaks()[0]
    rng = np.random.default_rng(3)
    ops1 = torch.from_numpy(np.stack([
        np.linalg.qr(rng.standard_normal((2, 2)) +
                     1j * rng.standard_normal((2, 2)))[0]
        for _ in range(n)])).to(dev, torch.complex64)
    pairs = torch.tensor([[i, (i + 7) % n] for i in range(0, n, 3)],
                         device=dev)
    perm = list(reversed(range(n)))
    cases = [
        (f"swap(0, {n - 1})", lambda: ug.swap(psi, (0, n - 1)), 16),
        ("permute_qubits(reversed)", lambda: ug.permute_qubits(perm, psi), 16),
        ("roll_qubits(1)", lambda: ug.roll_qubits(psi, 1), 16),
        ("multi_cz(10 pairs)", lambda: ug.multi_cz(pairs, psi), 16),
        ("multi_controlled_x([0,1,2], 5)",
         lambda: ug.multi_controlled_x(psi, [0, 1, 2], 5), 16),
        ("apply_to_qubits(30 x 1q)",
         lambda: ug.apply_to_qubits(list(ops1), list(range(n)), psi), None),
        ("sample(2^20)", lambda: sample(psi, 1 << 20, seed=1), 8),
    ]
    out = {}
    for name, fn, bpa in cases:
        ms = _cuda_time(fn, 3)
        row = {"ms": round(ms, 3)}
        if bpa is not None:
            gbs = bpa * N / (ms / 1e3) / 1e9
            row.update({"GB_s": round(gbs, 1), "frac_of_peak": round(gbs / peak, 3)})
        else:
            prog_passes = None
            try:
                from qcware_unitair_gb300.fusion import Circuit
                c = Circuit(n)
                for q in range(n):
                    c.append(ops1[q].cpu(), [q], "dense")
                prog_passes = c.compile(torch.complex64, dev).num_passes
            except Exception:  # informative only
                pass
            row.update({"passes": prog_passes,
                        "GB_s_per_pass": round(16 * N * (prog_passes or 1) /
                                               (ms / 1e3) / 1e9, 1)})
        out[name] = row
        torch.cuda.empty_cache()
    return {"workload": f"{n}-qubit complex64 state ({8 * 2 ** n / 2 ** 30:g} GiB), functional API",
            "peak_GBs": peak, "ops": out}


# ------------------------------------------ operators on 6-12 qubits ------
def bench_wide_ops(dev, n=30):
    """Dense 6- and 8-qubit operators (random unitaries) on a 30-qubit
    complex64 state (8 GiB), in place through apply_operator_ and (k = 6)
    through the functional apply_operator.  Targets on the high qubits
    (0..k-1: the state's most significant bits) and on the low ones
    (n-k..n-1: bit 0 among the targets).  Each output amplitude is a
    2^k-term complex dot product: 8 * 2^k FP32 flops per amplitude, so the
    bound is the FP32 pipe (SMs x 128 lanes x 2 flops x clock), not HBM;
    both fractions are reported."""
    import numpy as np
    import torch
    import qcware_unitair_gb300 as ug
    N = 2 ** n
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    psi = torch.randn(N, dtype=torch.complex64, device=dev, generator=g)
    psi /= torch.linalg.vector_norm(psi)
    peak = peaks()[0]
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = sm_max_mhz()
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_mhz / 1e6  # TF/s
    rng = np.random.default_rng(4)
    ops = {}
    for k in (6, 8):
        a = rng.standard_normal((2 ** k, 2 ** k)) + \
            1j * rng.standard_normal((2 ** k, 2 ** k))
        q, r = np.linalg.qr(a)
        ops[k] = torch.from_numpy(q * (np.diag(r) / np.abs(np.diag(r)))).to(
            dev, torch.complex64)
    cases = []
    for k in (6, 8):
        for where, qs in (("high", list(range(k))),
                          ("low", list(range(n - k, n)))):
            cases.append((f"apply_operator_({k} qubits, {where})", k,
                          lambda k=k, qs=qs: ug.apply_operator_(ops[k], qs,
                                                                psi)))
    cases.append(("apply_operator(6 qubits, high)", 6,
                  lambda: ug.apply_operator(ops[6], list(range(6)), psi)))
    out = {}
    for name, k, fn in cases:
        ms = _cuda_time(fn, 3)
        gbs = 16 * N / (ms / 1e3) / 1e9
        tfl = 8 * N * 2 ** k / (ms / 1e3) / 1e12
        out[name] = {"ms": round(ms, 3), "GB_s": round(gbs, 1),
                     "frac_of_copy_peak": round(gbs / peak, 3),
                     "fp32_TFLOPs": round(tfl, 1),
                     "frac_of_fp32_peak": round(tfl / fp32_peak, 3)}
        torch.cuda.empty_cache()
    nrm = float(ug.norm_squared(psi))
    return {"workload": f"{n}-qubit complex64 state ({8 * N / 2 ** 30:g} GiB), "
                        "random unitaries; in place repeats the operator",
            "peak_GBs": peak, "fp32_peak_TFLOPs": round(fp32_peak, 1),
            "fp32_peak_basis": "SMs x 128 FP32 lanes x 2 x max SM clock",
            "norm_after": round(nrm, 6), "ops": out}


# ------------------------------------------------- C1 in complex128 -------
def bench_c1_c128(dev, n=28, num_gates=1000, seed=0):
    """The canonical random circuit (1000 gates, numpy seed 0) on a 28-qubit
    complex128 state (4 GiB, far above L2) from |0...0>: one kernel per gate
    in place, and as fused stages.  Algorithmic bytes per gate: one read and
    one write of the state (2 * 2^n * 16 B); a stage counts as one pass.
    Also the largest amplitude difference between the two paths and the
    norm drift of the fused result."""
    import torch
    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300.circuits import random_circuit
    from qcware_unitair_gb300.fusion import Circuit
    gates = random_circuit(n, num_gates, seed=seed)
    mats = [torch.from_numpy(g.matrix()).to(dev) for g in gates]
    N = 2 ** n
    psi = torch.zeros(N, dtype=torch.complex128, device=dev)

    def plain():
        psi.zero_()
        psi[0] = 1
        for g, m in zip(gates, mats):
            ug.apply_operator_(m, g.qubits, psi)

    prog = Circuit.from_gates(n, gates).compile(torch.complex128, dev)

    def fused():
        psi.zero_()
        psi[0] = 1
        prog.run(psi, inplace=True)

    plain_ms = _cuda_time(plain, 1)
    ref = psi.clone()
    fused_ms = _cuda_time(fused, 2)
    diff = float((psi - ref).abs().max())
    drift = abs(float(torch.linalg.vector_norm(psi)) ** 2 - 1.0)
    del ref
    gate_bytes = 2 * N * 16
    return {"workload": f"{n} qubits complex128 (4 GiB), {num_gates} random "
                        "gates from |0...0>, in place",
            "plain_ms": round(plain_ms, 1),
            "plain_GBs_per_gate": round(gate_bytes * num_gates /
                                        (plain_ms / 1e3) / 1e9, 1),
            "fused_ms": round(fused_ms, 1), "passes": prog.num_passes,
            "fused_hbm_GBs": round(gate_bytes * prog.num_passes /
                                   (fused_ms / 1e3) / 1e9, 1),
            "speedup": round(plain_ms / fused_ms, 2),
            "max_abs_diff_fused_vs_plain": diff,
            "fused_norm_drift": drift}


# ---------------------------------------------------------------- serving --
def bench_serving(dev, num=300, rate=150.0, qubits=(10, 22)):
    """The serving trace (Poisson arrivals; qubits, depth 20-500 and 1-64
    states uniform; 20% ask for adjoint gradients of <Z_0>; HBM admission
    budget 160 GB) replayed against the continuous-batching server and the
    plain per-gate FIFO path.  The qubit range is capped so that both arms
    finish in seconds (a 28-qubit, 64-state request alone takes minutes on
    the plain path)."""
    from qcware_unitair_gb300.serve import (Server, make_trace, serve_plain,
                                            summarize)
    warm = make_trace(16, rate=1000.0, seed=99, qubits=qubits,
                      depth=(20, 100))
    Server(dev).serve(warm)
    serve_plain(warm, dev)
    trace = make_trace(num, rate=rate, seed=0, qubits=qubits)
    server = summarize(Server(dev).serve(trace))
    plain = summarize(serve_plain(trace, dev))
    return {"workload": f"{num} requests, Poisson {rate}/s, qubits "
                        f"U{{{qubits[0]}..{qubits[1]}}}, depth U{{20..500}}, "
                        "states U{1..64}, 20% adjoint gradients of <Z_0>, "
                        "complex64, 160 GB admission budget",
            "server": server, "plain_per_gate": plain,
            "throughput_ratio": round(server["circuits_per_s"] /
                                      plain["circuits_per_s"], 2),
            "p99_ratio": round(plain["p99_s"] / server["p99_s"], 2)}


def bench_serving_full_range(dev, num=60, rate=20.0, plain_cap_s=60.0):
    """The serving trace over the full qubit range U{10..28} (up to
    64 x 2^28 amplitudes per request), both arms on the same trace.  The
    plain per-gate path cannot finish it in a bounded bench: it starts no
    request after ``plain_cap_s`` seconds, and its unfinished requests
    count with latency (cap - arrival), a lower bound."""
    import numpy as np
    from qcware_unitair_gb300.serve import (Server, make_trace, serve_plain,
                                            summarize)
    import torch
    trace = make_trace(num, rate=rate, seed=3, qubits=(10, 28))
    server = summarize(Server(dev).serve(trace))
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    done = serve_plain(trace, dev, wall_cap_s=plain_cap_s)
    wall = time.perf_counter() - t0
    finished = {r.rid for r in done}
    lat = [r.latency for r in done] + [max(0.0, wall - q.arrival)
                                       for q in trace if q.rid not in finished]
    plain = {"requests": num, "finished": len(done),
             "circuits_per_s": round(len(done) / wall, 3),
             "p50_s": round(float(np.percentile(lat, 50)), 4),
             "p99_s": round(float(np.percentile(lat, 99)), 4),
             "latencies_are_lower_bounds": len(done) < num,
             "wall_s": round(wall, 2), "wall_cap_s": plain_cap_s}
    return {"workload": f"{num} requests, Poisson {rate:g}/s, qubits "
                        "U{10..28}, depth U{20..500}, states U{1..64}, 20% "
                        "adjoint gradients of <Z_0>, complex64, 160 GB "
                        "admission budget",
            "qubits": [10, 28], "server": server, "plain_per_gate": plain,
            "throughput_ratio": round(server["circuits_per_s"] /
                                      max(plain["circuits_per_s"], 1e-9), 2),
            "p99_ratio": round(plain["p99_s"] / server["p99_s"], 2)}


def bench_serving_sweep(dev, rates=(300.0, 600.0), num=300,
                        wide=(100, 100.0)):
    """The server alone at higher offered rates (same trace shape, qubits
    U{10..22}), and a trace over the full qubit range U{10..28} (up to
    64 x 2^28 amplitudes, 128 GiB, per request) at a lower rate."""
    from qcware_unitair_gb300.serve import Server, make_trace, summarize
    out = {}
    for r in rates:
        trace = make_trace(num, rate=r, seed=1, qubits=(10, 22))
        out[f"rate_{r:g}"] = summarize(Server(dev).serve(trace))
    wn, wr = wide
    trace = make_trace(wn, rate=wr, seed=2, qubits=(10, 28))
    out[f"qubits_10_28_rate_{wr:g}"] = summarize(Server(dev).serve(trace))
    out["workload"] = (f"server only; {num} requests per rate, qubits "
                       f"U{{10..22}}; {wn} requests at {wr:g}/s with qubits "
                       "U{10..28}; depth U{20..500}, states U{1..64}, 20% "
                       "adjoint gradients")
    return out


def _gpu_local_cpus(dev):
    """CPUs on the GPU's NUMA node (sysfs local_cpulist of its PCI
    function), or None when unknown."""
    import torch
    try:
        p = torch.cuda.get_device_properties(dev)
        bdf = (f"{getattr(p, 'pci_domain_id', 0):04x}:"
               f"{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0")
        txt = Path(f"/sys/bus/pci/devices/{bdf}/local_cpulist").read_text()
        cpus = parse_cpulist(txt) & os.sched_getaffinity(0)
        return cpus or None
    except (OSError, ValueError, AttributeError, RuntimeError):
        return None


def parse_cpulist(txt: str) -> set:
    """CPU numbers of a sysfs cpulist such as "0-3,8,10-11"."""
    cpus = set()
    for part in txt.strip().split(","):
        if not part:
            continue
        lo, _, hi = part.partition("-")
        cpus.update(range(int(lo), int(hi or lo) + 1))
    return cpus


# ------------------------------------------------------------ workloads --
# Small fixed workloads for timing and profiling one kernel at a time
# (python bench.py --workload NAME [ARGS]); each runs twice (a warm-up, then
# a CUDA-event-timed run) and prints one line, so under a profiler skip the
# first run's launches.
#   stage N [GATES]      canonical random circuit (numpy seed 0), complex64,
#                        fused (tensor-core stages), in place from |0...0>
#   stage_reg N [GATES]  the same on the register-blocked stages
#   gates N KIND K       one register stage: 8 Hadamards on spread tile bits
#                        plus K copies of KIND (H, X, RX, RZout = RZ on a bit
#                        that is never a register bit)
#   adjoint B            20-qubit, 12-layer ansatz forward + adjoint backward
#   serve NUM            the serving trace (150/s, 10-22 qubits) on the server
#                        after a 16-request warm-up, with host time per path
#   kinds N              one plain complex128 gate of each kind, 10 launches
#   wide N K [low]       one dense K-qubit unitary (numpy seed K) in place on
#                        an N-qubit complex64 state, targets 0..K-1 (or
#                        N-K..N-1 with "low")
def _wl_timed(fn):
    import torch
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def wl_stage(n: int = 26, gates: int = 200, tensor_cores=None,
             dtype: str = "c64") -> float:
    """A random circuit through fused stages (complex64, or complex128 in
    the process's arithmetic mode)."""
    import torch
    from qcware_unitair_gb300.circuits import random_circuit, zero_state
    from qcware_unitair_gb300.fusion import Circuit
    dev = torch.device("cuda")
    dt = torch.complex64 if dtype == "c64" else torch.complex128
    prog = Circuit.from_gates(n, random_circuit(n, gates, seed=0)).compile(
        dt, dev, tensor_cores=tensor_cores)
    psi = zero_state(n, (), dt, dev)
    ms = _wl_timed(lambda: prog.run(psi, inplace=True))
    print(f"stage n={n} gates={gates} dtype={dtype} "
          f"tensor_cores={prog.tensor_cores} passes={prog.num_passes} "
          f"{ms:.3f} ms")
    return ms


def wl_gates(n: int = 24, kind: str = "H", k: int = 64) -> float:
    import torch
    from qcware_unitair_gb300.circuits import gate_matrix
    from qcware_unitair_gb300.fusion import Circuit
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
    prog = c.compile(torch.complex64, dev, tile_qubits=12,
                     tensor_cores=False)
    psi = torch.randn(2 ** n, dtype=torch.complex64, device=dev)
    ms = _wl_timed(lambda: prog.run(psi, inplace=True))
    print(f"gates n={n} kind={kind} k={k} passes={prog.num_passes} "
          f"{ms:.3f} ms")
    return ms


def wl_adjoint(batch: int = 16, n: int = 20, layers: int = 12) -> float:
    import torch
    from qcware_unitair_gb300.adjoint import PauliSum, expectation, hardware_efficient_ansatz
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

    ms = _wl_timed(step)
    print(f"adjoint n={n} layers={layers} batch={batch} {ms:.3f} ms")
    return ms


def wl_serve(num: int = 300) -> float:
    import torch
    import collections
    import time
    from qcware_unitair_gb300 import serve as S
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


def wl_kinds(n: int = 28, mode: str = "pairs") -> None:
    """Each complex128 gate kind on an n-qubit state, in the given
    arithmetic mode ("pairs" or "fp64"); 10 timed launches after 2."""
    import numpy as np
    import torch
    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300.circuits import gate_matrix
    ug.set_complex128_arithmetic(mode)
    dev = torch.device("cuda")
    psi = torch.randn(2 ** n, dtype=torch.complex128, device=dev)
    psi /= psi.abs().pow(2).sum().sqrt()
    rng = np.random.default_rng(0)

    def unitary(k):
        q, _ = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) +
                            1j * rng.normal(size=(2 ** k, 2 ** k)))
        return q

    cry = np.eye(4, dtype=np.complex128)
    cry[2:, 2:] = gate_matrix("RY", 0.7)
    cases = [("X", [5]), ("H", [5]), ("RY", [5]), ("RX", [5]), ("RZ", [5]),
             ("T", [5]), ("Z", [5]), ("Y", [5]), ("S", [5]), ("U2", [5]),
             ("CNOT", [3, 20]), ("CZ", [3, 20]), ("SWAP", [3, 20]),
             ("CRY", [3, 20]), ("U4", [3, 20]), ("X", [n - 1]),
             ("RX", [n - 1]), ("CNOT", [n - 2, n - 1]),
             ("U8", [3, 11, 20]), ("U16", [2, 9, 15, 22])]
    for name, q in cases:
        if name == "U2":
            mat = unitary(1)
        elif name == "U4":
            mat = unitary(2)
        elif name == "U8":
            mat = unitary(3)
        elif name == "U16":
            mat = unitary(4)
        elif name == "CRY":
            mat = cry
        else:
            mat = gate_matrix(name, 0.7 if name.startswith("R") else None)
        m = torch.from_numpy(mat).to(dev)
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
        print(f"kinds n={n} {mode} {name} {q}: {ms:.3f} ms "
              f"{2 * 16 * 2 ** n / ms / 1e6:.0f} GB/s")


def wl_phase128(n: int = 28) -> None:
    """apply_phase on an n-qubit complex128 state with float64 angles, in
    both complex128 arithmetic modes."""
    import torch
    import qcware_unitair_gb300 as ug
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    psi = torch.randn(2 ** n, dtype=torch.complex128, device=dev, generator=g)
    ang = torch.rand(2 ** n, dtype=torch.float64, device=dev,
                     generator=g) * 6.3
    for mode in ("pairs", "fp64"):
        ug.set_complex128_arithmetic(mode)
        ms = _wl_timed(lambda: ug.apply_phase(ang, psi))
        gbs = 2 ** n * (16 + 16 + 8) / ms / 1e6
        print(f"phase128 n={n} {mode}: {ms:.3f} ms {gbs:.0f} GB/s")
    ug.set_complex128_arithmetic("pairs")


def wl_wide(n: int = 26, k: int = 6, where: str = "high") -> None:
    """One dense k-qubit unitary applied in place to an n-qubit complex64
    state (the wide-operator tile kernel)."""
    import numpy as np
    import torch
    import qcware_unitair_gb300 as ug
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    psi = torch.randn(2 ** n, dtype=torch.complex64, device=dev, generator=g)
    rng = np.random.default_rng(k)
    q, r = np.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) +
                        1j * rng.standard_normal((2 ** k, 2 ** k)))
    op = torch.from_numpy(q * (np.diag(r) / np.abs(np.diag(r)))).to(
        dev, torch.complex64)
    qs = list(range(n - k, n)) if where == "low" else list(range(k))
    ms = _wl_timed(lambda: ug.apply_operator_(op, qs, psi))
    print(f"wide n={n} k={k} {where}: {ms:.3f} ms "
          f"{8 * 2 ** n * 2 ** k / ms / 1e9:.1f} FP32 TFLOP/s")


def run_workload(argv):
    import torch  # noqa: F401  (CUDA initialised before the workload)
    what, args = argv[0], argv[1:]
    if what == "stage":
        wl_stage(*(int(a) for a in args))
    elif what == "stage_reg":
        wl_stage(*(int(a) for a in args), tensor_cores=False)
    elif what == "stage128":  # n gates [fp64]
        import qcware_unitair_gb300 as ug
        if len(args) > 2:
            ug.set_complex128_arithmetic(args[2])
        wl_stage(*(int(a) for a in args[:2]), dtype="c128")
    elif what == "gates":
        wl_gates(int(args[0]) if args else 24,
                 args[1] if len(args) > 1 else "H",
                 int(args[2]) if len(args) > 2 else 64)
    elif what == "adjoint":
        wl_adjoint(*(int(a) for a in args))
    elif what == "serve":
        wl_serve(*(int(a) for a in args))
    elif what == "phase128":
        wl_phase128(int(args[0]) if args else 28)
    elif what == "kinds":
        wl_kinds(int(args[0]) if args else 28,
                 args[1] if len(args) > 1 else "pairs")
    elif what == "wide":
        wl_wide(int(args[0]) if args else 26,
                int(args[1]) if len(args) > 1 else 6,
                args[2] if len(args) > 2 else "high")
    else:
        raise SystemExit(f"unknown workload {what}")


# -------------------------------------------------------------- GPU arm ---
def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch

    import qcware_unitair_gb300 as ug
    from qcware_unitair_gb300 import _lib
    from qcware_unitair_gb300.circuits import random_circuit

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    n, G = args.qubits, args.gates
    gates = random_circuit(n, G, seed=args.seed)
    N = 2 ** n
    bytes_per_gate = 2 * 8 * N
    mats_host = [torch.from_numpy(g.matrix()).to(torch.complex64)
                 for g in gates]
    mats = [m.to(dev) for m in mats_host]
    # ---- e2e through the public functional API, host buffers -----------
    # Measured first, on device memory no earlier phase has fragmented:
    # after the device-timed phases the 8 GiB copies ran 2-10x slower
    # (the same copy alone: 41 ms at 211 GB/s).
    # pinned buffers are placed from the GPU's local CPUs: pages pinned on
    # a far NUMA node cut host-to-device bandwidth several-fold
    cpus = _gpu_local_cpus(dev)
    old_aff = os.sched_getaffinity(0)
    try:
        if cpus:
            os.sched_setaffinity(0, cpus)
    except OSError:
        pass
    try:
        host_in = torch.zeros(N, dtype=torch.complex64, pin_memory=True)
        host_in[0] = 1
        host_out = torch.zeros(N, dtype=torch.complex64, pin_memory=True)
        # the step's gate matrices as one pinned tensor per size (one copy
        # each instead of a thousand small ones)
        sizes = sorted({m.shape[-1] for m in mats_host})
        stacked = {d: torch.stack([m for m in mats_host if m.shape[-1] == d])
                   .pin_memory() for d in sizes}
        slot = []
        seen = {d: 0 for d in sizes}
        for m in mats_host:
            d = m.shape[-1]
            slot.append((d, seen[d]))
            seen[d] += 1
    finally:
        try:
            os.sched_setaffinity(0, old_aff)
        except OSError:
            pass

    def e2e_step(ev=None):
        if ev is not None:
            ev[0].record()
        state = host_in.to(dev, non_blocking=True)
        dmats = {d: t.to(dev, non_blocking=True) for d, t in stacked.items()}
        ops = [dmats[d][i] for d, i in slot]
        if ev is not None:
            ev[1].record()
        for g, m in zip(gates, ops):
            state = ug.apply_operator(m, g.qubits, state)
        if ev is not None:
            ev[2].record()
        host_out.copy_(state, non_blocking=True)
        if ev is not None:
            ev[3].record()
        return state

    e2e_step()
    torch.cuda.synchronize()
    # the box's own pinned host-to-device rate for this buffer (untimed):
    # it varies from box to box (23-211 GB/s seen for 8 GiB) and bounds
    # the e2e number
    probe = torch.empty(N, dtype=torch.complex64, device=dev)
    c0, c1 = torch.cuda.Event(enable_timing=True), \
        torch.cuda.Event(enable_timing=True)
    c0.record()
    probe.copy_(host_in, non_blocking=True)
    c1.record()
    torch.cuda.synchronize()
    h2d_probe_gbs = N * 8 / (c0.elapsed_time(c1) / 1e3) / 1e9
    del probe
    barrier()
    e2e_steps = max(1, min(args.steps, 2))
    gc.collect()
    gc.disable()  # no collector pauses inside the timed host loop
    e2e_ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)]
              for _ in range(e2e_steps)]
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(e2e_ev[k])
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
    gc.enable()
    # where an e2e step's time goes (CUDA events on the launching stream)
    e2e_parts = {
        name: round(statistics.mean(ev[i].elapsed_time(ev[i + 1])
                                    for ev in e2e_ev), 2)
        for i, name in enumerate(("h2d_ms", "gates_ms", "d2h_ms"))}
    e2e_parts["wall_ms"] = round(1e3 * e2e_s / e2e_steps, 2)
    e2e_parts["h2d_copy_alone_GBs"] = round(h2d_probe_gbs, 1)
    e2e_value = bytes_per_gate * G * e2e_steps * ws / e2e_s / 1e9
    h2d = N * 8 + sum(m.numel() * 8 for m in mats_host)
    d2h = N * 8
    # final state sanity: unit norm
    drift = abs(float(np.sum(np.abs(host_out.numpy().astype(np.complex128))
                             ** 2)) - 1.0)

    psi = torch.zeros(N, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def reset():
        psi.zero_()
        psi[0] = 1

    def step():
        for g, m in zip(gates, mats):
            ug.apply_operator_(m, g.qubits, psi)

    reset()
    for _ in range(args.warmup):
        step()
    # Timed: exactly K applications of the circuit, back to back, starting
    # from |0...0> (reset before the region); nothing else is launched.
    reset()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    gc.collect()
    gc.disable()  # no collector pauses inside the timed host loop
    with ClockSampler(local) as clocks:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            step()
        t1.record(stream)
        torch.cuda.synchronize()
    barrier()
    gc.enable()
    launches = _lib.launch_count() - l0
    ms = t0.elapsed_time(t1)
    ms = max_over_ranks(ms, dev)
    total_bytes = bytes_per_gate * G * args.steps * ws
    value = total_bytes / (ms / 1e3) / 1e9

    # per-launch durations of the dense gate kernel (roofline), in one more
    # untimed application of the circuit with events around every launch
    per_launch_ms = []
    reset()
    for g, m in zip(gates, mats):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ug.apply_operator_(m, g.qubits, psi)
        e1.record(stream)
        per_launch_ms.append((e0, e1))
    torch.cuda.synchronize()
    per_launch_ms = [a.elapsed_time(b) for a, b in per_launch_ms]
    gate_ms = statistics.mean(per_launch_ms)

    # ---- fused paths on the same circuit ------------------------------
    from qcware_unitair_gb300.fusion import Circuit
    circ = Circuit.from_gates(n, gates)

    def fused_run(prog):
        """K timed applications (after W warm-ups) from |0...0>; mean ms per
        circuit, per-stage launch durations of one more run, the norm."""
        reset()
        for _ in range(args.warmup):
            prog.run(psi, inplace=True)
        reset()
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        lc = _lib.launch_count()
        e0.record(stream)
        for _ in range(args.steps):
            prog.run(psi, inplace=True)
        e1.record(stream)
        torch.cuda.synchronize()
        nl = (_lib.launch_count() - lc) // max(1, args.steps)
        f_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)
        norm = float(torch.linalg.vector_norm(psi.to(torch.complex128)))
        # per-stage durations (one more run, events around each launch)
        reset()
        evs = []
        for op in prog.ops:
            a = torch.cuda.Event(enable_timing=True)
            z = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            prog.run_op(op, psi)
            z.record(stream)
            evs.append((op[0], a, z))
        torch.cuda.synchronize()
        stage_ms = [a.elapsed_time(z) for k, a, z in evs if k != "plain"]
        return f_ms, nl, norm, stage_ms

    prog = circ.compile(torch.complex64, dev)
    fused_ms, fused_launches, fused_norm, tc_stage_ms = fused_run(prog)
    stage_ms = fused_ms / prog.num_passes
    # the same circuit with a renormalisation checkpoint every 16 passes
    reset()
    ra = torch.cuda.Event(enable_timing=True)
    rb = torch.cuda.Event(enable_timing=True)
    ra.record(stream)
    prog.run(psi, inplace=True, renorm_every=16)
    rb.record(stream)
    torch.cuda.synchronize()
    renorm = {"every_passes": 16, "ms_per_step": round(ra.elapsed_time(rb), 3),
              "drift_removed": prog.renorm_drift(),
              "final_norm_drift": abs(float(torch.linalg.vector_norm(
                  psi.to(torch.complex128))) ** 2 - 1.0)}
    prog_reg = circ.compile(torch.complex64, dev, tensor_cores=False)
    reg_ms, _, reg_norm, _ = fused_run(prog_reg)
    del prog_reg

    peak, peak_kind = peaks()
    achieved = bytes_per_gate / (gate_ms / 1e3) / 1e9
    result = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic: canonical random circuit (numpy seed "
                f"{args.seed}) applied to |0...0>",
        "config": {"workload": WORKLOAD.format(n=n, g=G), "qubits": n, "gates": G,
                   "state_bytes": N * 8,
                   "l2": "inputs larger than L2 (8 GiB state vs 129 MB L2); "
                         "no flush",
                   "parallelism": f"replicas x{ws}"},
        "pct_of_peak": round(100 * value / peak, 1),
        "amp_updates_per_s": N * G * args.steps * ws / (ms / 1e3),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind,
                     "kernel": "dense_chunk_kernel (1- and 2-qubit gates)",
                     "traffic": DENSE_GATE_TRAFFIC_30Q,
                     "traffic_source": DENSE_GATE_TRAFFIC_SOURCE,
                     "algorithmic_bytes_per_launch": bytes_per_gate,
                     "launch_ms_mean": round(gate_ms, 4),
                     "launch_ms_p50": round(statistics.median(per_launch_ms),
                                            4),
                     "launch_ms_max": round(max(per_launch_ms), 4)},
        "e2e_step_parts": e2e_parts,
        "e2e": {"value": round(e2e_value, 1), "unit": "GB/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": "qcware_unitair_gb300.apply_operator (functional)",
                "step_parts": e2e_parts,
                "final_norm_drift": drift},
        "fused": {
            "engine": "tensor-core stages (tcgen05, 32x32 blocks)"
                      if prog.tensor_cores else "register stages",
            "ms_per_step": round(fused_ms, 3), "passes": prog.num_passes,
            "gates_per_pass": round(G / prog.num_passes, 2),
            "pass_reduction": round(G / prog.num_passes, 2),
            "blocks": sum(o[4] for o in prog.ops if o[0] == "tc"),
            "speedup_vs_plain": round((ms / args.steps) / fused_ms, 3),
            "tile_qubits": prog.m,
            "hbm_GBs": round(bytes_per_gate * prog.num_passes /
                             (fused_ms / 1e3) / 1e9, 1),
            "hbm_frac": round(bytes_per_gate * prog.num_passes /
                              (fused_ms / 1e3) / 1e9 / peaks()[0], 4),
            "gate_equivalent_GBs": round(bytes_per_gate * G /
                                         (fused_ms / 1e3) / 1e9, 1),
            "stage_ms_mean": round(stage_ms, 4),
            "stage_launch_ms_mean": round(statistics.mean(tc_stage_ms), 4)
                                    if tc_stage_ms else None,
            "launches_per_step": fused_launches,
            "final_norm": fused_norm,
            "final_norm_drift": abs(fused_norm ** 2 - 1.0),
            "with_renorm_checkpoints": renorm,
            "register_stages_ms": round(reg_ms, 3),
            "speedup_vs_register_stages": round(reg_ms / fused_ms, 3),
            "register_stages_final_norm": reg_norm},
        "roofline_fused": {
            "bound": "hbm", "kernel": "tc_stage_kernel" if prog.tensor_cores
            else "fused_reg_kernel",
            "achieved": round(bytes_per_gate / (statistics.mean(tc_stage_ms)
                                                / 1e3) / 1e9, 1)
                        if tc_stage_ms else None,
            "peak": peak, "unit": "GB/s",
            "frac": round(bytes_per_gate / (statistics.mean(tc_stage_ms)
                                            / 1e3) / 1e9 / peak, 4)
                    if tc_stage_ms else None,
            "algorithmic_bytes_per_launch": bytes_per_gate},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if not args.no_extras:
        result["c0_12q_x64"] = bench_c0(dev)
        result["c2_16q_x4096"] = bench_c2(dev)
        result["path_rows_30q"] = bench_path_rows(dev)
        result["next_rows_30q"] = bench_next_rows(dev)
        try:
            result["wide_ops_30q"] = bench_wide_ops(dev)
        except Exception as e:  # an extra never loses the line
            result["wide_ops_30q"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        result["adjoint"] = bench_adjoint(dev)
        result["serving"] = bench_serving(dev)
        for key, fn in (("serving_10_28", bench_serving_full_range),
                        ("serving_sweep", bench_serving_sweep),
                        ("c1_28q_c128", bench_c1_c128)):
            torch.cuda.empty_cache()
            try:
                result[key] = fn(dev)
            except Exception as e:  # an extra never loses the line
                result[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_sample(n, gates, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def unitair_sample(num_qubits: int, seed: int, budget_s: float = 10.0):
    """unitair's own torch CPU path (apply_operator, operations.py:45-148),
    installed under baseline/_ref, on every host thread: the canonical
    circuit's first gates on a num_qubits complex64 state from |0...0>
    until budget_s passes, as algorithmic GB/s (2 x 8 B x 2^n per gate)."""
    ref = REPO / "baseline" / "_ref"
    if not (ref / "unitair").is_dir():
        return {"unavailable": "baseline/_ref has no unitair install"}
    sys.path.insert(0, str(ref))
    try:
        import torch
        import unitair.simulation as usim
    except ImportError as e:
        return {"unavailable": f"unitair import failed: {e}"}
    from qcware_unitair_gb300.circuits import random_circuit
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    gates = random_circuit(num_qubits, 1000, seed=seed)
    psi = torch.zeros(2 ** num_qubits, dtype=torch.complex64)
    psi[0] = 1
    mats = [torch.from_numpy(g.matrix()).to(torch.complex64) for g in gates]
    psi = usim.apply_operator(mats[0], list(gates[0].qubits), psi)  # warm
    done, t0 = 0, time.perf_counter()
    for g, m in zip(gates, mats):
        psi = usim.apply_operator(m, list(g.qubits), psi)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": round(done * 2 * 8 * 2 ** num_qubits / dt / 1e9, 3),
            "unit": "GB/s", "qubits": num_qubits, "threads": threads,
            "gates_timed": done, "s_per_gate": round(dt / done, 4),
            "api": "unitair.simulation.apply_operator (torch CPU)",
            "sample": f"first {done} gates of the {num_qubits}-qubit "
                      f"canonical circuit, {dt:.1f} s"}


def run_reference(args, ws, rank):
    """Reference arm: the oracle's C port of the reference path (complex64
    arithmetic, OpenMP over all host threads); each step is a bounded sample
    of the same circuit.  Under torchrun only rank 0 runs."""
    if rank != 0:
        return
    from qcware_unitair_gb300.circuits import random_circuit
    n, G = args.qubits, args.gates
    gates = random_circuit(n, G, seed=args.seed)
    budget = max(2.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_sample(n, gates, budget)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sample(n, gates, budget))
    elapsed = time.perf_counter() - t0
    v = statistics.mean(x["value"] for x in vals)
    result = {
        "metric": METRIC, "value": round(v, 3), "unit": "GB/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * elapsed / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "impl": "reference",
        "data": "synthetic: canonical random circuit (numpy seed "
                f"{args.seed}) applied to |0...0>",
        "config": {"workload": WORKLOAD.format(n=n, g=G), "qubits": n, "gates": G,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(v, 3), "unit": "GB/s",
                         "cores": vals[0]["cores"], "kind": "port",
                         "sample": vals[0]["sample"]},
        "e2e": {"value": round(v, 3), "unit": "GB/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        # unitair itself, beside the port (a 30-qubit state is out of its
        # reach in a bounded run: about three 8 GiB copies per gate)
        "unitair": unitair_sample(24, args.seed),
    }
    print(json.dumps(result), flush=True)


def main():
    args = parse()
    if args.workload:
        run_workload(args.workload)
        return
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
