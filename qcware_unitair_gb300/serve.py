"""Continuous-batching circuit server.

Requests (a circuit of the canonical gate set on n qubits, a batch of
seeded random initial states, optionally adjoint gradients of <Z_0>) arrive
over time.  One host loop runs four things while earlier work is still on
the GPU:

  admission   FIFO by arrival; a request is admitted when its HBM footprint
              fits the byte budget (160 GB by default).  If the head of the
              queue does not fit, later requests may pass it only until it
              has waited ``reserve_after`` seconds; from then on admission
              waits for memory, so large requests are not starved.  A
              request larger than the whole budget (up to 64 x 2^28
              amplitudes with gradients) is split at arrival into parts of
              whole 8-state blocks that fit; their outputs are joined in
              state order when the last part finishes.
  packing     admitted requests whose states fit one tile (n <= 13 for
              complex64) are packed, whatever their circuits, into ONE
              multi-program launch per qubit count (gbsv_run_programs: one
              CTA per state, each running its own gate list).
  batching    larger requests admitted together with the same qubit count
              run as fused programs whose stages go out in rounds: round
              r launches stage r of every one of them in ONE launch
              (gbsv_run_stages_multi), so small states fill the GPU.
  streams     the rest (gradient requests, a lone request of its size) run
              as fused programs on a pool of CUDA streams, so several
              requests' kernels overlap on the device.
  completion  CUDA events are polled; finished requests return norms and
              <Z_0> (FP64 reductions) and free their memory for the next
              admissions.

``serve_plain`` is the baseline: the same trace, FIFO, one request at a
time, one kernel per gate on one stream.  Both return one ``Result`` per
request with arrival, admission and completion times.
"""
from __future__ import annotations

import collections
import ctypes
import dataclasses
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _core, _lib, simulation, states
from .circuits import Gate, gate_matrix, random_circuit, ROTATIONS
from .fusion import (FG_DTYPE, Program, gate_list_desc, native_plan)


# States are drawn in blocks of STATE_BLOCK, block b from its own generator
# seeded by (request seed, b), so any run of whole blocks of a request can be
# generated on its own: a request too large for the HBM budget is served as
# parts of whole blocks that reproduce the unsplit request's states.
STATE_BLOCK = 8


@dataclass
class Request:
    rid: int
    arrival: float
    num_qubits: int
    num_states: int
    gates: List[Gate]
    want_grad: bool = False
    seed: int = 0
    state_offset: int = 0  # first state of this part (a multiple of 8)

    @property
    def state_bytes(self) -> int:
        return self.num_states * (8 << self.num_qubits)

    @property
    def bytes_per_state(self) -> int:
        # gradients: the request's states, the forward copy, psi and lambda
        # of the sweep, and room for the sweep's temporaries
        return (8 << self.num_qubits) * (6 if self.want_grad else 1)

    @property
    def footprint(self) -> int:
        return self.num_states * self.bytes_per_state

    def split(self, budget: float) -> List["Request"]:
        """Parts of whole state blocks whose footprints fit ``budget`` (the
        request itself when it fits, or when one block does not)."""
        per_block = STATE_BLOCK * self.bytes_per_state
        if self.footprint <= budget or per_block > budget:
            return [self]
        step = int(budget // per_block) * STATE_BLOCK
        return [dataclasses.replace(self, num_states=min(step,
                                                         self.num_states - k),
                                    state_offset=self.state_offset + k)
                for k in range(0, self.num_states, step)]


@dataclass
class Result:
    rid: int
    norms: np.ndarray
    z0: np.ndarray
    grads: Optional[np.ndarray]
    arrival: float
    admitted: float
    done: float
    final: Optional[torch.Tensor] = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def make_trace(num_requests: int = 20000, rate: float = 50.0, seed: int = 0,
               qubits=(10, 28), depth=(20, 500), batch=(1, 64),
               grad_fraction: float = 0.2) -> List[Request]:
    """Poisson arrivals at ``rate`` per second; qubits, depth and states
    uniform in the given inclusive ranges; gates from the canonical set."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(num_requests):
        t += float(rng.exponential(1.0 / rate))
        n = int(rng.integers(qubits[0], qubits[1] + 1))
        d = int(rng.integers(depth[0], depth[1] + 1))
        b = int(rng.integers(batch[0], batch[1] + 1))
        g = bool(rng.random() < grad_fraction)
        out.append(Request(i, t, n, b, random_circuit(n, d, seed=seed * 1000003
                                                      + i), g, seed + i))
    return out


def summarize(results: Sequence[Result]) -> dict:
    lat = np.array([r.latency for r in results])
    t0 = min(r.arrival for r in results)
    t1 = max(r.done for r in results)
    return {"requests": len(results),
            "circuits_per_s": round(len(results) / (t1 - t0), 3),
            "p50_s": round(float(np.percentile(lat, 50)), 4),
            "p99_s": round(float(np.percentile(lat, 99)), 4),
            "mean_s": round(float(lat.mean()), 4),
            "makespan_s": round(t1 - t0, 3)}


# ---------------------------------------------------------------- helpers --
def _init_states(req: Request, device, dtype=torch.complex64):
    """The request's states [state_offset, state_offset + num_states):
    standard-normal amplitudes, normalised per state, block by block."""
    N = 2 ** req.num_qubits
    psi = torch.empty(req.num_states, N, dtype=dtype, device=device)
    g = torch.Generator(device=device)
    first = req.state_offset
    end = first + req.num_states
    for b in range(first // STATE_BLOCK, (end - 1) // STATE_BLOCK + 1):
        lo, hi = b * STATE_BLOCK, min((b + 1) * STATE_BLOCK, end)
        g.manual_seed((int(req.seed) * 0x9E3779B1 + b) & ((1 << 62) - 1))
        blk = torch.randn(hi - lo, N, dtype=dtype, device=device,
                          generator=g)
        a = max(lo, first)
        psi[a - first:hi - first] = blk[a - lo:]
    psi /= states.norm_squared(psi).sqrt().unsqueeze(-1)
    return psi


def _outputs(psi: torch.Tensor, n: int):
    """FP64 norms and <Z_0> (qubit 0 is the top index bit: <Z_0> is the
    weight of the first half minus that of the second)."""
    B = psi.shape[0]
    halves = states.norm_squared_fp64(psi.view(B * 2, 2 ** (n - 1)))
    halves = halves.view(B, 2)
    return halves.sum(-1), halves[:, 0] - halves[:, 1]


_FIXED_GATES: Dict[str, tuple] = {}


def _fixed_gate(name: str):
    """One matrix tensor per canonical fixed gate (planners reuse the same
    object's adjoint) and its structure: CZ / Z / S / T diagonal, CNOT
    controlled, the rest dense."""
    ent = _FIXED_GATES.get(name)
    if ent is None:
        from .fusion import _NAMED_KIND, DENSE
        ent = _FIXED_GATES[name] = (
            torch.as_tensor(gate_matrix(name).astype(np.complex128)),
            _NAMED_KIND.get(name, DENSE))
    return ent


def _grad_circuit(req: Request):
    """ParamCircuit with one parameter per rotation (angles shared by the
    request's states) and <Z_0> as the observable."""
    from .adjoint import ParamCircuit, PauliSum
    rots = [g for g in req.gates if g.name in ROTATIONS]
    pc = ParamCircuit(req.num_qubits, max(1, len(rots)))
    angles = []
    for g in req.gates:
        if g.name in ROTATIONS:
            {"RX": pc.rx, "RY": pc.ry, "RZ": pc.rz}[g.name](
                g.qubits[0], len(angles))
            angles.append(g.theta)
        else:
            mat, kind = _fixed_gate(g.name)
            pc.ops.append(("fixed", mat, tuple(int(q) for q in g.qubits),
                           kind))
    return pc, PauliSum(req.num_qubits).z(0), angles


def _run_grad(req: Request, psi0: torch.Tensor, fuse: bool = True):
    """d<Z_0>/d(angle) per state: forward from the gate list (native
    planner), then the adjoint backward sweep -- fused backward stages, or
    one kernel per rotation / fixed gate with ``fuse=False`` (the plain
    path)."""
    from .adjoint import _backward_fused, _backward_sweep
    pc, H, angles = _grad_circuit(req)
    dev = psi0.device
    params = torch.tensor(angles or [0.0], dtype=torch.float64)
    params = params.pin_memory().to(dev, non_blocking=True).expand(
        req.num_states, -1).contiguous()
    psi = psi0.clone()
    Program.from_gate_list(req.gates, req.num_qubits, torch.complex64, dev,
                           fuse=fuse).run(psi, inplace=True)
    sweep = _backward_fused if fuse else _backward_sweep
    return sweep(pc, params, H, psi, [], torch.complex64)


def _merge_parts(done_parts) -> Result:
    """One Result from the Results of a split request's parts: outputs
    concatenated in state order, admitted at the first part's admission,
    done when the last part is."""
    rs = [r for _, r in sorted(done_parts, key=lambda x: x[0])]
    grads = (np.concatenate([r.grads for r in rs])
             if rs[0].grads is not None else None)
    final = (torch.cat([r.final for r in rs])
             if all(r.final is not None for r in rs) else None)
    return Result(rs[0].rid, np.concatenate([r.norms for r in rs]),
                  np.concatenate([r.z0 for r in rs]), grads, rs[0].arrival,
                  min(r.admitted for r in rs), max(r.done for r in rs), final)


# ----------------------------------------------------------------- server --
class Server:
    def __init__(self, device="cuda", budget_bytes: float = 160e9,
                 num_streams: int = 4, reserve_after: float = 0.5,
                 keep_states: bool = False):
        self.device = torch.device(device)
        self.budget = float(budget_bytes)
        self.streams = [torch.cuda.Stream(self.device)
                        for _ in range(num_streams)]
        self.reserve_after = reserve_after
        self.keep_states = keep_states
        L = _lib.load()
        self.small_max = int(L.gbsv_fused_max_tile_qubits(_lib.C64))
        self._next_stream = 0
        self.peak_used = 0.0  # largest admitted footprint seen (bytes)

    def _stream(self):
        s = self.streams[self._next_stream % len(self.streams)]
        self._next_stream += 1
        return s

    # -- launches ---------------------------------------------------------
    def _launch_small(self, reqs):
        """Requests with one qubit count -> one packed launch."""
        n = reqs[0].num_qubits
        stream = self._stream()
        with torch.cuda.stream(stream):
            items = [(req, _init_states(req, self.device)) for req in reqs]
        recs, pool_parts, first, count, ptrs = [], [], [], [], []
        pool_len = 0
        nrec = 0
        for req, psi in items:
            # one whole-state stage per request, planned natively
            desc, mats = gate_list_desc(req.gates)
            nat = native_plan(None, n, n, n, 0, True, torch.complex64,
                              desc, mats)
            r = nat["records"].copy()
            r["mat"] += pool_len
            recs.append(r)
            pool_parts.append(nat["pool"])
            pool_len += len(nat["pool"])
            f0 = nrec
            nrec += len(r)
            N = 2 ** n
            base = psi.data_ptr()
            for j in range(req.num_states):
                ptrs.append(base + j * N * 8)
                first.append(f0)
                count.append(nrec - f0)
        dev = self.device
        with torch.cuda.stream(stream):
            allr = np.concatenate(recs) if recs else np.zeros(1, FG_DTYPE)
            gates = torch.from_numpy(allr.view(np.uint8).copy())
            pool = torch.from_numpy(np.concatenate(pool_parts)) \
                if pool_len else torch.zeros(1, dtype=torch.complex64)
            gates = gates.pin_memory().to(dev, non_blocking=True)
            pool = pool.pin_memory().to(dev, non_blocking=True)
            meta = torch.tensor(ptrs, dtype=torch.int64).pin_memory().to(
                dev, non_blocking=True)
            fi = torch.tensor(first, dtype=torch.int32).pin_memory().to(
                dev, non_blocking=True)
            co = torch.tensor(count, dtype=torch.int32).pin_memory().to(
                dev, non_blocking=True)
            rc = _lib.load().gbsv_run_programs(
                _lib.C64, n, len(ptrs), meta.data_ptr(), fi.data_ptr(),
                co.data_ptr(), gates.data_ptr(), pool.data_ptr(),
                stream.cuda_stream)
            _lib.check(rc, "run_programs")
            outs = [(req, psi, _outputs(psi, n)) for req, psi in items]
            ev = torch.cuda.Event()
            ev.record(stream)
        keep = (gates, pool, meta, fi, co)
        return [(ev, req, psi, o, None, keep) for req, psi, o in outs]

    def _launch_large(self, req):
        stream = self._stream()
        with torch.cuda.stream(stream):
            psi = _init_states(req, self.device)
            grads = None
            if req.want_grad:  # reads psi (its own forward runs on a copy)
                grads = _run_grad(req, psi)
            prog = Program.from_gate_list(req.gates, req.num_qubits,
                                          torch.complex64, self.device)
            prog.run(psi, inplace=True)
            o = _outputs(psi, req.num_qubits)
            ev = torch.cuda.Event()
            ev.record(stream)
        return (ev, req, psi, o, grads, prog)

    def _launch_large_batch(self, reqs):
        """Requests with one qubit count (no gradients): their programs'
        stages in rounds, one multi-program launch per round."""
        n = reqs[0].num_qubits
        stream = self._stream()
        N = 2 ** n
        L = _lib.load()
        with torch.cuda.stream(stream):
            items = []
            for req in reqs:
                psi = _init_states(req, self.device)
                prog = Program.from_gate_list(req.gates, n, torch.complex64,
                                              self.device)
                items.append((req, psi, prog))
        solo = [it for it in items
                if any(op[0] != "layouts" for op in it[2].ops)
                or it[2].m != items[0][2].m]
        batch = [it for it in items if it not in solo]
        out = []
        with torch.cuda.stream(stream):
            rounds = max((len(p.ops) for _, _, p in batch), default=0)
            for r in range(rounds):
                live = [it for it in batch if len(it[2].ops) > r]
                descs = (_lib.MultiStage * len(live))()
                for d, (req, psi, prog) in zip(descs, live):
                    _, c, positions, first, count = prog.ops[r]
                    d.state_in = d.state_out = psi.data_ptr()
                    d.gates = prog.gate_records.data_ptr()
                    d.layouts = prog.layout_records.data_ptr() + first * 32
                    d.pool = prog.pool.data_ptr()
                    d.num_states = req.num_states
                    d.in_stride = N
                    d.num_layouts = count
                    d.contiguous_qubits = c
                    for j in range(prog.m):
                        d.tile_positions[j] = positions[j]
                rc = L.gbsv_run_stages_multi(_lib.C64, n, live[0][2].m,
                                             ctypes.cast(descs,
                                                         ctypes.c_void_p),
                                             len(live), stream.cuda_stream)
                _lib.check(rc, "run_stages_multi")
                for req, psi, prog in live:
                    if len(prog.ops) == r + 1:  # this request is done
                        o = _outputs(psi, n)
                        ev = torch.cuda.Event()
                        ev.record(stream)
                        out.append((ev, req, psi, o, None, prog))
            for req, psi, prog in solo:
                prog.run(psi, inplace=True)
                o = _outputs(psi, n)
                ev = torch.cuda.Event()
                ev.record(stream)
                out.append((ev, req, psi, o, None, prog))
        return out

    # -- the loop ---------------------------------------------------------
    def serve(self, trace: Sequence[Request]) -> List[Result]:
        """Replay the trace against the wall clock; one Result per
        request, ordered by request id."""
        pending = collections.deque(sorted(trace, key=lambda r: r.arrival))
        waiting: collections.deque = collections.deque()
        inflight = []
        results: Dict[int, Result] = {}
        parts: Dict[int, list] = {}  # rid -> [parts left, finished parts]
        admitted_at = {}
        used = 0.0
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        while pending or waiting or inflight:
            now = clock()
            while pending and pending[0].arrival <= now:
                req = pending.popleft()
                split = req.split(self.budget)
                if len(split) > 1:
                    parts[req.rid] = [len(split), []]
                waiting.extend(split)
            # admission
            small, large = [], []
            blocked = False
            for req in list(waiting):
                fits = used + req.footprint <= self.budget or (
                    used == 0 and not inflight)
                if fits and not blocked:
                    waiting.remove(req)
                    used += req.footprint
                    self.peak_used = max(self.peak_used, used)
                    admitted_at[req.rid, req.state_offset] = now
                    if req.num_qubits <= self.small_max and not req.want_grad:
                        small.append(req)
                    else:
                        large.append(req)
                elif not fits and now - req.arrival > self.reserve_after:
                    blocked = True  # hold memory for this request
            by_n = collections.defaultdict(list)
            for req in small:
                by_n[req.num_qubits].append(req)
            for reqs in by_n.values():
                inflight.extend(self._launch_small(reqs))
            big_n = collections.defaultdict(list)
            for req in large:
                if req.want_grad:
                    inflight.append(self._launch_large(req))
                else:
                    big_n[req.num_qubits].append(req)
            for reqs in big_n.values():
                if len(reqs) == 1:
                    inflight.append(self._launch_large(reqs[0]))
                else:
                    inflight.extend(self._launch_large_batch(reqs))
            # completion
            still = []
            for item in inflight:
                ev, req, psi, (norms, z0), grads, _keep = item
                if ev.query():
                    done = clock()
                    res = Result(
                        req.rid, norms.cpu().numpy(), z0.cpu().numpy(),
                        grads.cpu().numpy() if grads is not None else None,
                        req.arrival, admitted_at[req.rid, req.state_offset],
                        done, psi if self.keep_states else None)
                    if req.rid in parts:
                        entry = parts[req.rid]
                        entry[0] -= 1
                        entry[1].append((req.state_offset, res))
                        if entry[0] == 0:
                            results[req.rid] = _merge_parts(entry[1])
                            del parts[req.rid]
                    else:
                        results[req.rid] = res
                    used -= req.footprint
                else:
                    still.append(item)
            inflight = still
            if inflight and not waiting:
                time.sleep(0.0002)
            elif not inflight and not waiting and pending:
                time.sleep(max(0.0, min(0.01, pending[0].arrival - clock())))
        return [results[r.rid] for r in sorted(trace, key=lambda r: r.rid)]


def serve_plain(trace: Sequence[Request], device="cuda",
                keep_states: bool = False,
                wall_cap_s: Optional[float] = None,
                budget_bytes: float = 160e9) -> List[Result]:
    """Baseline: FIFO, one request at a time, one kernel per gate.  A
    request larger than the HBM budget runs as the server's parts of whole
    state blocks, one after another.  With ``wall_cap_s`` no request starts
    after that many seconds; only the finished requests are returned."""
    dev = torch.device(device)
    out = []
    t0 = time.perf_counter()
    for whole in sorted(trace, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if wall_cap_s is not None and now > wall_cap_s:
            break
        if now < whole.arrival:
            time.sleep(whole.arrival - now)
        pieces = []
        for req in whole.split(budget_bytes):
            pieces.append((req.state_offset,
                           _plain_one(req, dev, t0, keep_states)))
        out.append(pieces[0][1] if len(pieces) == 1 else
                   _merge_parts(pieces))
    return sorted(out, key=lambda r: r.rid)


def _plain_one(req: Request, dev, t0: float, keep_states: bool) -> Result:
    """One request (or part) on the plain per-gate path."""
    admitted = time.perf_counter() - t0
    psi = _init_states(req, dev)
    grads = None
    if req.want_grad:
        grads = _run_grad(req, psi, fuse=False)
    # all of the request's gate matrices in one transfer, then one
    # kernel per gate
    mats = [torch.from_numpy(g.matrix()) for g in req.gates]
    by_size = {}
    for d in (2, 4):
        sel = [m for m in mats if m.shape[-1] == d]
        if sel:
            by_size[d] = iter(torch.stack(sel).to(torch.complex64)
                              .pin_memory().to(dev, non_blocking=True))
    for g, m in zip(req.gates, mats):
        simulation.apply_operator_(next(by_size[m.shape[-1]]), g.qubits,
                                   psi)
    norms, z0 = _outputs(psi, req.num_qubits)
    res = Result(req.rid, norms.cpu().numpy(), z0.cpu().numpy(),
                 grads.cpu().numpy() if grads is not None else None,
                 req.arrival, admitted, time.perf_counter() - t0,
                 psi if keep_states else None)
    del psi
    return res
