"""Adjoint differentiation of expectation values of parameterised circuits.

    pc = ParamCircuit(n, num_params)
    pc.ry(q, p); pc.rz(q, p); pc.cz(a, b); pc.end_layer()
    H = PauliSum(n).z(0).xx(0, 1, coeff=0.5)
    values = expectation(pc, params, H)            # (B,) float64, autograd
    values.mean().backward()                       # adjoint sweep, no tape

Rotations follow unitair's convention (src/unitair/gates/gates.py:6-91):
RX(theta) = exp_x(theta / 2) = exp(-i theta/2 X), likewise RY, RZ; the angle
of a rotation is ``scale * params[b, p]`` per batch entry b.

The forward pass runs the circuit as a fused program (one HBM pass per
stage) and keeps the state at checkpoints every ~sqrt(depth) layers.  The
backward pass starts from lambda = H psi_L (gbsv_pauli_sum_apply) and walks
the gates in reverse with gbsv_adjoint_rotation_step (gradient Im<l|P|psi>
accumulated in FP64, then U^dag applied to psi and lambda in the same pass);
fixed gates are uncomputed on both states in one launch.  At each
checkpoint the uncomputed psi is replaced by the stored forward state, so
rounding drift never accumulates over more than one segment.
This replaces torch autograd through unitair's apply_operator, which keeps
every intermediate state (one per gate) alive for the backward pass.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

import ctypes

from . import _core, _lib, states

ctypes_int32 = ctypes.c_int32
from .circuits import gate_matrix
from .fusion import CTRL, DENSE, DIAG, Circuit

GEN = {"X": 0, "Y": 1, "Z": 2}


class PauliSum:
    """H = sum_k c_k P_k with real c_k and Pauli strings P_k."""

    def __init__(self, num_qubits: int):
        self.num_qubits = num_qubits
        self.terms: List[tuple] = []  # (coeff, {qubit: 'X'|'Y'|'Z'})

    def add(self, coeff: float, paulis: Dict[int, str]) -> "PauliSum":
        for q, p in paulis.items():
            if p not in "XYZ" or not 0 <= q < self.num_qubits:
                raise ValueError(f"bad Pauli {p} on qubit {q}")
        self.terms.append((float(coeff), dict(paulis)))
        return self

    def z(self, q, coeff=1.0):
        return self.add(coeff, {q: "Z"})

    def xx(self, a, b, coeff=1.0):
        return self.add(coeff, {a: "X", b: "X"})

    def term_array(self) -> np.ndarray:
        """Records matching gbsv_pauli_term_t (xmask, zmask, re, im)."""
        n = self.num_qubits
        dt = np.dtype([("x", "<u8"), ("z", "<u8"), ("re", "<f8"),
                       ("im", "<f8")])
        out = np.zeros(len(self.terms), dtype=dt)
        for k, (c, ps) in enumerate(self.terms):
            xm = zm = 0
            ny = 0
            for q, p in ps.items():
                bit = 1 << (n - 1 - q)
                if p in "XY":
                    xm |= bit
                if p in "ZY":
                    zm |= bit
                ny += p == "Y"
            phase = 1j ** ny
            out[k] = (xm, zm, c * phase.real, c * phase.imag)
        return out

    def dense(self) -> np.ndarray:
        """2^n x 2^n matrix (small n; for tests)."""
        n = self.num_qubits
        P = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]),
             "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}
        H = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
        for c, ps in self.terms:
            m = np.array([[1.0]])
            for q in range(n):
                m = np.kron(m, P[ps.get(q, "I")])
            H += c * m
        return H


def hardware_efficient_ansatz(num_qubits: int, layers: int):
    """Each layer applies U = RY(theta) RZ(phi) to every qubit (RZ acts
    first), then a ring of CZ(q, q+1 mod n).  Parameter (layer, qubit, k)
    has index (layer * n + qubit) * 2 + k, k = 0 for theta and 1 for phi,
    i.e. a (B, layers, n, 2) tensor reshaped to (B, layers * n * 2)."""
    n = num_qubits
    pc = ParamCircuit(n, layers * n * 2)
    for l in range(layers):
        for q in range(n):
            base = (l * n + q) * 2
            pc.rz(q, base + 1)
            pc.ry(q, base + 0)
        for q in range(n):
            if n > 1 and (q + 1 < n or n > 2):
                pc.cz(q, (q + 1) % n)
        pc.end_layer()
    return pc


class ParamCircuit:
    """Rotations driven by a (B, num_params) parameter tensor plus fixed
    gates; ``end_layer`` marks layer boundaries for checkpointing."""

    def __init__(self, num_qubits: int, num_params: int):
        self.num_qubits = num_qubits
        self.num_params = num_params
        self.ops: list = []
        self.layer_ends: List[int] = []

    def _rot(self, gen, q, p, scale):
        if not 0 <= p < self.num_params:
            raise ValueError(f"parameter index {p} out of range")
        if not 0 <= q < self.num_qubits:
            raise ValueError(f"qubit {q} out of range")
        self.ops.append(("rot", gen, int(q), int(p), float(scale)))
        return self

    def rx(self, q, p, scale=1.0): return self._rot("X", q, p, scale)
    def ry(self, q, p, scale=1.0): return self._rot("Y", q, p, scale)
    def rz(self, q, p, scale=1.0): return self._rot("Z", q, p, scale)

    def gate(self, matrix, qubits, kind: Optional[str] = None):
        m = torch.as_tensor(np.asarray(matrix, dtype=np.complex128))
        self.ops.append(("fixed", m, tuple(int(q) for q in qubits), kind))
        return self

    def h(self, q): return self.gate(gate_matrix("H"), [q], DENSE)
    def cz(self, a, b): return self.gate(gate_matrix("CZ"), [a, b], DIAG)
    def cnot(self, c, t): return self.gate(gate_matrix("CNOT"), [c, t], CTRL)

    def end_layer(self):
        self.layer_ends.append(len(self.ops))
        return self

    # -- segments for checkpoints ---------------------------------------
    def segments(self, every: Optional[int] = None) -> List[tuple]:
        """Op ranges [a, b) between checkpoints, every ~sqrt(depth)
        layers (or ~sqrt(ops) without layer marks)."""
        ends = [e for e in self.layer_ends if 0 < e <= len(self.ops)]
        if ends and ends[-1] != len(self.ops):
            ends.append(len(self.ops))
        if not ends:
            k = every or max(1, int(math.ceil(math.sqrt(len(self.ops)))))
            ends = list(range(k, len(self.ops), k)) + [len(self.ops)]
        else:
            k = every or max(1, int(math.ceil(math.sqrt(len(ends)))))
            ends = ends[k - 1::k] if len(ends) > k else []
            if not ends or ends[-1] != len(self.ops):
                ends.append(len(self.ops))
        out, a = [], 0
        for e in ends:
            if e > a:
                out.append((a, e))
            a = e
        return out or [(0, 0)]

    # -- building blocks ---------------------------------------------------
    def _segment_circuit(self, a, b, params, dtype) -> Circuit:
        """Ops [a, b) as a Circuit with per-state rotation matrices."""
        c = Circuit(self.num_qubits)
        B = params.shape[0]
        for op in self.ops[a:b]:
            if op[0] == "fixed":
                _, m, qs, kind = op
                c.append(m, qs, kind)
                continue
            _, gen, q, p, scale = op
            th = params[:, p].detach().to(torch.float64) * (0.5 * scale)
            cs, sn = torch.cos(th), torch.sin(th)
            z = torch.zeros_like(cs)
            if gen == "X":
                m = torch.stack([torch.complex(cs, z), torch.complex(z, -sn),
                                 torch.complex(z, -sn), torch.complex(cs, z)],
                                -1)
                kind = DENSE
            elif gen == "Y":
                m = torch.stack([torch.complex(cs, z), torch.complex(-sn, z),
                                 torch.complex(sn, z), torch.complex(cs, z)],
                                -1)
                kind = DENSE
            else:
                m = torch.stack([torch.complex(cs, -sn), torch.complex(z, z),
                                 torch.complex(z, z), torch.complex(cs, sn)],
                                -1)
                kind = DIAG
            c.append(m.reshape(B, 2, 2).to(dtype), [q], kind)
        return c


# placeholder rotation matrices fix each rotation's record kind when a
# forward program is planned once per circuit structure: a generic complex
# 2x2 for X (dense), a real one for Y (real 2x2), a diagonal for Z
_PLACEHOLDER = {
    "X": torch.tensor([[0.6 + 0.2j, 0.1 - 0.3j], [0.4 + 0.1j, 0.7 - 0.2j]],
                      dtype=torch.complex128),
    "Y": torch.tensor([[0.8, -0.6], [0.6, 0.8]], dtype=torch.complex128),
    "Z": torch.tensor([[0.6 - 0.8j, 0], [0, 0.6 + 0.8j]],
                      dtype=torch.complex128),
}


def _forward_program(pc: ParamCircuit, a: int, b: int, B: int, dtype, dev,
                     fuse: bool):
    """(Program, scatter index, rotation index) for ops [a, b) with B
    states, planned once per structure.  Each call only writes the rotation
    values into the program's pool."""
    key = (a, b, B, dtype, str(dev), fuse)
    cache = pc.__dict__.setdefault("_fwd_cache", {})
    if key in cache:
        return cache[key]
    c = Circuit(pc.num_qubits)
    rots = []
    for op in pc.ops[a:b]:
        if op[0] == "fixed":
            _, m, qs, kind = op
            c.append(m, qs, kind)
            continue
        _, gen, q, p, scale = op
        ph = _PLACEHOLDER[gen].expand(B, 2, 2).clone()
        c.append(ph, [q], DIAG if gen == "Z" else DENSE)
        rots.append((c.gates[-1], op))
    prog = c.compile(dtype, dev, fuse=fuse, native=False)
    idx, which = [], []
    for g, op in rots:
        if fuse:
            off, nv = prog.gate_pool[id(g)]
        else:
            off, nv = None, 4
        which.append((op[1], op[3], op[4], off, nv))
    cache[key] = (prog, which, rots)
    return cache[key]


def _rotation_values(which, params, B, dtype):
    """All rotations' pool entries, flattened in ``which`` order (rotation,
    state, entry), from a handful of vectorised tensor ops."""
    dev = params.device
    cached = _rotation_values._meta.get(id(which))
    if cached is None or cached[0] is not which:
        gen = torch.tensor(["XYZ".index(w[0]) for w in which], device=dev)
        pidx = torch.tensor([w[1] for w in which], device=dev)
        half = torch.tensor([0.5 * w[2] for w in which], dtype=torch.float64,
                            device=dev)
        nv = torch.tensor([w[4] for w in which], device=dev)
        keep = (torch.arange(4, device=dev)[None, None, :] <
                nv[:, None, None]).expand(len(which), B, 4)
        cached = (which, gen, pidx, half, nv, keep)
        _rotation_values._meta[id(which)] = cached
    _, gen, pidx, half, nv, keep = cached
    th = params[:, pidx].to(torch.float64) * half          # (B, R)
    c, s = torch.cos(th).T, torch.sin(th).T                 # (R, B)
    z = torch.zeros_like(c)
    isx, isy = (gen == 0)[:, None], (gen == 1)[:, None]
    isz4 = ((gen == 2) & (nv == 4))[:, None]
    # entry k of each rotation, real and imaginary parts (R, B)
    re0, im0 = c, torch.where(isx | isy, z, -s)
    re1 = torch.where(isy, -s, torch.where(isx | isz4, z, c))
    im1 = torch.where(isx, -s, torch.where(isy | isz4, z, s))
    re2, im2 = torch.where(isy, s, z), torch.where(isx, -s, z)
    re3, im3 = c, torch.where(isz4, s, z)
    re = torch.stack([re0, re1, re2, re3], -1)
    im = torch.stack([im0, im1, im2, im3], -1)
    return torch.complex(re, im).to(dtype)[keep]


_rotation_values._meta = {}


def _initial_state(n, B, dtype, device, psi0):
    if psi0 is None:
        s = torch.zeros(B, 2 ** n, dtype=dtype, device=device)
        s[:, 0] = 1
        return s
    s = psi0.to(device=device, dtype=dtype)
    if s.dim() == 1:
        s = s.expand(B, -1)
    return s.reshape(B, 2 ** n).contiguous()


def _forward(pc: ParamCircuit, params, dtype, psi0, checkpoints: bool,
             fuse: bool = True):
    """Run the circuit; return (psi_L, [psi at each segment start])."""
    n, B = pc.num_qubits, params.shape[0]
    dev = params.device
    psi = _initial_state(n, B, dtype, dev, psi0)
    saved = []
    p = params.detach()
    for a, b in pc.segments():
        if checkpoints:
            saved.append(psi.clone())
        if b <= a:
            continue
        if not fuse:
            prog = pc._segment_circuit(a, b, params, dtype).compile(
                dtype, dev, fuse=False)
            prog.run(psi, inplace=True)
            continue
        prog, which, _ = _forward_program(pc, a, b, B, dtype, dev, fuse)
        if which:
            # one scatter of every rotation's values into the cached pool
            idx = prog.__dict__.get("_rot_index")
            if idx is None:
                parts = [torch.arange(off, off + B * nv, device=dev)
                         for _, _, _, off, nv in which]
                idx = prog._rot_index = torch.cat(parts)
            prog.pool.index_copy_(0, idx, _rotation_values(which, p, B,
                                                           dtype))
        prog.run(psi, inplace=True)
    return psi, saved


def _pauli_apply(H: PauliSum, psi: torch.Tensor, out: torch.Tensor):
    terms = torch.from_numpy(H.term_array().view(np.uint8).copy()).to(
        psi.device)
    n = H.num_qubits
    rc = _lib.load().gbsv_pauli_sum_apply(
        psi.data_ptr(), out.data_ptr(), _core.complex_code(psi.dtype), n,
        psi.numel() >> n, terms.data_ptr(), len(H.terms),
        _core.stream_of(psi.device))
    _lib.check(rc, "pauli_sum_apply")
    return out


def pauli_expectation(H: PauliSum, psi: torch.Tensor) -> torch.Tensor:
    """<psi|H|psi> per state (float64, FP64 accumulation)."""
    lam = torch.empty_like(psi)
    _pauli_apply(H, psi.contiguous(), lam)
    return _real_inner(psi, lam)


def _real_inner(a, b):
    """Re <a|b> per row with the FP64 accumulator returned unrounded."""
    ip = states._inner_product_kernel(a, b, out_dtype=torch.complex128)
    return ip.real


def _backward_sweep(pc, params, H, psi_L, saved, dtype):
    n, B = pc.num_qubits, params.shape[0]
    dev = params.device
    N = 2 ** n
    buf = torch.empty(2, B, N, dtype=dtype, device=dev)
    psi, lam = buf[0], buf[1]
    psi.copy_(psi_L)
    _pauli_apply(H, psi, lam)
    grads = torch.zeros(B, pc.num_params, dtype=torch.float64, device=dev)
    p = params.detach().contiguous()
    if p.dtype not in (torch.float32, torch.float64):
        p = p.to(torch.float64)
    L = _lib.load()
    code = _core.complex_code(dtype)
    acode = _core.real_code(p.dtype)
    esz = p.element_size()
    stream = _core.stream_of(dev)
    nbytes = int(L.gbsv_adjoint_scratch_bytes(B, n))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    both = buf.view(2 * B, N)
    # every fixed gate's adjoint, moved to the device in one transfer
    fixed = [op for op in pc.ops if op[0] == "fixed"]
    dag = {}
    if fixed:
        flat = [op[1].conj().T.contiguous().reshape(-1) for op in fixed]
        host = torch.cat(flat).to(dtype)
        if dev.type == "cuda":
            host = host.pin_memory()
        devbuf = host.to(dev, non_blocking=True)
        off = 0
        for op, f in zip(fixed, flat):
            d = op[1].shape[-1]
            dag[id(op)] = devbuf[off:off + f.numel()].view(d, d)
            off += f.numel()
    segs = pc.segments() if saved else [(0, len(pc.ops))]
    for si in range(len(segs) - 1, -1, -1):
        a, b = segs[si]
        for op in reversed(pc.ops[a:b]):
            if op[0] == "rot":
                _, gen, q, pi, scale = op
                rc = L.gbsv_adjoint_rotation_step(
                    psi.data_ptr(), lam.data_ptr(), code, n, B, q, GEN[gen],
                    p.data_ptr() + pi * esz, acode, pc.num_params, scale,
                    grads.data_ptr() + pi * 8, pc.num_params, scale,
                    scratch.data_ptr(), nbytes, stream)
                _lib.check(rc, "adjoint_rotation_step")
            else:
                _, m, qs, _kind = op
                md = dag[id(op)]
                wide = not _core.inplace_ok(dtype, len(qs), n)
                dst = torch.empty_like(both) if wide else both
                rc = L.gbsv_apply_operator(
                    both.data_ptr(), dst.data_ptr(), code, n, 2 * B, N,
                    md.data_ptr(), 0, _lib.qubit_array(qs), len(qs), stream)
                _lib.check(rc, "apply_operator")
                if wide:
                    both.copy_(dst)
        if saved:
            psi.copy_(saved[si])  # re-anchor at the forward checkpoint
    return grads


def evaluate(pc: ParamCircuit, params: torch.Tensor, H: PauliSum,
             psi0: Optional[torch.Tensor] = None,
             dtype=torch.complex64) -> torch.Tensor:
    """Forward only: <psi|H|psi> per batch entry (float64), no gradient."""
    _core.require_cuda(params)
    psi_L, _ = _forward(pc, params, dtype, psi0, False)
    return pauli_expectation(H, psi_L)


ADJOP_DTYPE = np.dtype([("kind", "<i4"), ("gen", "<i4"), ("bit", "<i4"),
                        ("slot", "<i4"), ("pidx", "<i4"), ("pad", "<i4"),
                        ("scale", "<f8")])


def _adjop_dtype():
    from .fusion import FG_DTYPE
    return np.dtype(ADJOP_DTYPE.descr + [("g", FG_DTYPE)])


def _plan_backward(pc: ParamCircuit, a: int, b: int, dtype, dev, m: int):
    """Fused backward stages for ops [a, b) walked in reverse: a list of
    ("stage", launch args) / ("rot", op) / ("fixed", op) entries.  Depends
    only on the circuit's structure, so it is cached per circuit."""
    from .fusion import CircuitGate, FG_DTYPE, _record, _to_device, plan
    n = pc.num_qubits
    ops = list(reversed(pc.ops[a:b]))
    stand = []
    dummy = torch.zeros(2, 2, dtype=torch.complex128)
    for op in ops:
        if op[0] == "rot":
            stand.append(CircuitGate(dummy, (op[2],),
                                     DIAG if op[1] == "Z" else DENSE))
        else:
            _, mat, qs, kind = op
            stand.append(CircuitGate(mat.conj().transpose(-1, -2), qs,
                                     kind or DENSE))
    index = {id(g): op for g, op in zip(stand, ops)}
    c_min = min(4 if dtype == torch.complex64 else 3, m)
    out = []
    AD = _adjop_dtype()
    for kind, item in plan(stand, n, m, c_min):
        if kind == "plain":
            op = index[id(item)]
            out.append(("rot" if op[0] == "rot" else "fixed", op))
            continue
        tile = item.tile
        c = 0
        while c in tile:
            c += 1
        c = min(c, m)
        order = list(range(c)) + sorted(p for p in tile if p >= c)
        local = {p: i for i, p in enumerate(order)}
        G = len(item.gates)
        recs = np.zeros(G, dtype=AD)  # filled by column: no per-record
        kinds = np.zeros(G, np.int32)  # structured-array promotion
        gens = np.zeros(G, np.int32)
        bits = np.zeros(G, np.int32)
        slots = np.zeros(G, np.int32)
        pidxs = np.zeros(G, np.int32)
        scales = np.zeros(G, np.float64)
        pool, slot_p, slot_s = [], [], []
        pool_len = 0
        for i, g in enumerate(item.gates):
            op = index[id(g)]
            if op[0] == "rot":
                _, gen, q, pi, scale = op
                pos = n - 1 - q
                gens[i] = GEN[gen]
                bits[i] = local[pos] if pos in local else -1 - pos
                slots[i], pidxs[i], scales[i] = len(slot_p), pi, scale
                slot_p.append(pi)
                slot_s.append(scale)
            else:
                rec, vals = _record(g, n, local, None)
                v = vals.reshape(-1).to(dtype)
                rec["mat"], rec["mat_bstride"] = pool_len, 0
                pool.append(v)
                pool_len += v.numel()
                kinds[i] = 1
                recs["g"][i] = rec
        recs["kind"], recs["gen"], recs["bit"] = kinds, gens, bits
        recs["slot"], recs["pidx"], recs["scale"] = slots, pidxs, scales
        args = {
            "c": c, "positions": (ctypes_int32 * m)(*order),
            "ops": _to_device(recs.view(np.uint8), dev),
            "num_ops": G,
            "pool": (torch.cat(pool) if pool else torch.zeros(1, dtype=dtype)
                     ).to(dev),
            "num_slots": len(slot_p),
            "slot_param": torch.tensor(slot_p or [0], dtype=torch.int32,
                                       device=dev),
            "slot_scale": torch.tensor(slot_s or [0.0], dtype=torch.float64,
                                       device=dev)}
        out.append(("stage", args))
    return out


def _plan_backward_native(pc: ParamCircuit, a: int, b: int, dtype, dev,
                          m: int):
    """_plan_backward with the stages planned by gbsv_plan (C++) and the
    adjoint records assembled by column: the same stages, records and
    values (one pool for all stages instead of one per stage)."""
    from .fusion import (DESC_DTYPE, _KIND_CODE, _to_device, native_plan)
    n = pc.num_qubits
    ops = list(reversed(pc.ops[a:b]))
    G = len(ops)
    desc = np.zeros(max(1, G), dtype=DESC_DTYPE)
    parts = [np.eye(2, dtype=np.complex128).reshape(-1)]  # rotations' stand-in
    off = 4
    kinds, nqs, q0s, q1s, offs = [], [], [], [], []
    is_rot = np.zeros(G, dtype=bool)
    gens = np.zeros(G, np.int32)
    pidxs = np.zeros(G, np.int32)
    scales = np.zeros(G, np.float64)
    dag = {}  # adjoints of repeated fixed matrices (the same object)
    for i, op in enumerate(ops):
        if op[0] == "rot":
            _, gen, q, pi, scale = op
            kinds.append(_KIND_CODE[DIAG if gen == "Z" else DENSE])
            nqs.append(1)
            q0s.append(q)
            q1s.append(0)
            offs.append(0)
            is_rot[i] = True
            gens[i], pidxs[i], scales[i] = GEN[gen], pi, scale
        else:
            _, mat, qs, kind = op
            md = dag.get(id(mat))
            if md is None:
                md = np.ascontiguousarray(
                    np.conj(mat.detach().cpu().numpy()).T,
                    dtype=np.complex128).reshape(-1)
                dag[id(mat)] = md
            kinds.append(_KIND_CODE[kind or DENSE])
            nqs.append(len(qs))
            q0s.append(qs[0])
            q1s.append(qs[1] if len(qs) > 1 else 0)
            offs.append(off)
            parts.append(md)
            off += md.size
    if G:
        desc["kind"][:G], desc["nq"][:G] = kinds, nqs
        desc["q0"][:G], desc["q1"][:G], desc["mat"][:G] = q0s, q1s, offs
        desc["num_batch"][:G] = 1
    mats = np.ascontiguousarray(np.concatenate(parts))
    c_min = min(4 if dtype == torch.complex64 else 3, m)
    nat = native_plan(None, n, m, c_min, 0, True, dtype, desc[:G], mats)
    recs = nat["records"]
    pool = torch.from_numpy(nat["pool"]).to(dev) if len(nat["pool"]) else \
        torch.zeros(1, dtype=dtype, device=dev)
    AD = _adjop_dtype()
    out = []
    nxt = 0  # next gate index not yet placed
    for op in nat["ops"]:
        t, first, count = int(op["type"]), int(op["first"]), int(op["count"])
        if t == 0:
            assert first == nxt
            src = ops[first]
            out.append(("rot" if src[0] == "rot" else "fixed", src))
            nxt = first + 1
            continue
        idx = np.arange(nxt, nxt + count)
        nxt += count
        r = recs[first:first + count]
        rot = is_rot[idx]
        ad = np.zeros(count, dtype=AD)
        ad["kind"] = np.where(rot, 0, 1)
        ad["gen"] = gens[idx]
        ad["bit"] = np.where(rot, r["b0"], 0)
        ad["slot"] = np.where(rot, np.cumsum(rot) - 1, 0)
        ad["pidx"] = np.where(rot, pidxs[idx], 0)
        ad["scale"] = np.where(rot, scales[idx], 0.0)
        ad["g"][~rot] = r[~rot]
        out.append(("stage", {
            "c": int(op["contiguous"]),
            "positions": (ctypes_int32 * m)(
                *[int(x) for x in op["positions"][:m]]),
            "ops": _to_device(ad.view(np.uint8), dev),
            "num_ops": count,
            "pool": pool,
            "num_slots": int(rot.sum()),
            "slot_param": torch.tensor(pidxs[idx][rot].tolist() or [0],
                                       dtype=torch.int32, device=dev),
            "slot_scale": torch.tensor(scales[idx][rot].tolist() or [0.0],
                                       dtype=torch.float64, device=dev)}))
    assert nxt == G
    return out


def _backward_fused(pc, params, H, psi_L, saved, dtype):
    """The adjoint sweep with fused backward stages (see the kernel
    gbsv_adjoint_stage): one read and write of psi and lambda per stage."""
    n, B = pc.num_qubits, params.shape[0]
    dev = params.device
    N = 2 ** n
    m = min(12 if dtype == torch.complex64 else 11, n)
    buf = torch.empty(2, B, N, dtype=dtype, device=dev)
    psi, lam = buf[0], buf[1]
    psi.copy_(psi_L)
    _pauli_apply(H, psi, lam)
    grads = torch.zeros(B, pc.num_params, dtype=torch.float64, device=dev)
    p = params.detach().contiguous()
    if p.dtype not in (torch.float32, torch.float64):
        p = p.to(torch.float64)
    L = _lib.load()
    code = _core.complex_code(dtype)
    pcode = _core.real_code(p.dtype)
    stream = _core.stream_of(dev)
    segs = pc.segments() if saved else [(0, len(pc.ops))]
    cache = pc.__dict__.setdefault("_adj_cache", {})
    tiles = B << (n - m)
    scratch = None
    both = buf.view(2 * B, N)
    for si in range(len(segs) - 1, -1, -1):
        a, b = segs[si]
        key = (a, b, dtype, str(dev), m)
        if key not in cache:
            host = all(op[0] == "rot" or not op[1].is_cuda
                       for op in pc.ops[a:b])
            cache[key] = (_plan_backward_native if host else _plan_backward)(
                pc, a, b, dtype, dev, m)
        for entry in cache[key]:
            if entry[0] == "stage":
                st = entry[1]
                need = st["num_slots"] * (tiles + 2 * B) * 8
                if need and (scratch is None or scratch.numel() < need):
                    scratch = torch.empty(need, dtype=torch.uint8, device=dev)
                rc = L.gbsv_adjoint_stage(
                    psi.data_ptr(), lam.data_ptr(), code, n, B, m, st["c"],
                    st["positions"], st["ops"].data_ptr(), st["num_ops"],
                    st["pool"].data_ptr(), p.data_ptr(), pcode,
                    pc.num_params, st["num_slots"],
                    st["slot_param"].data_ptr(), st["slot_scale"].data_ptr(),
                    grads.data_ptr(),
                    scratch.data_ptr() if need else None, need, stream)
                _lib.check(rc, "adjoint_stage")
            elif entry[0] == "rot":
                _, gen, q, pi, scale = entry[1]
                nbytes = int(L.gbsv_adjoint_scratch_bytes(B, n))
                sc = torch.empty(max(nbytes, 16), dtype=torch.uint8,
                                 device=dev)
                rc = L.gbsv_adjoint_rotation_step(
                    psi.data_ptr(), lam.data_ptr(), code, n, B, q, GEN[gen],
                    p.data_ptr() + pi * p.element_size(), pcode,
                    pc.num_params, scale, grads.data_ptr() + pi * 8,
                    pc.num_params, scale, sc.data_ptr(), nbytes, stream)
                _lib.check(rc, "adjoint_rotation_step")
            else:
                _, m_, qs, _k = entry[1]
                md = m_.conj().T.contiguous().to(device=dev, dtype=dtype)
                wide = not _core.inplace_ok(dtype, len(qs), n)
                dst = torch.empty_like(both) if wide else both
                rc = L.gbsv_apply_operator(
                    both.data_ptr(), dst.data_ptr(), code, n, 2 * B, N,
                    md.data_ptr(), 0, _lib.qubit_array(qs), len(qs), stream)
                _lib.check(rc, "apply_operator")
                if wide:
                    both.copy_(dst)
        if saved:
            psi.copy_(saved[si])
    return grads


def expectation_and_grad(pc: ParamCircuit, params: torch.Tensor,
                         H: PauliSum, psi0: Optional[torch.Tensor] = None,
                         dtype=torch.complex64, checkpoints: bool = True,
                         fuse: bool = True):
    """(values (B,), grads (B, num_params)), both float64.  ``fuse=False``
    runs the forward pass one kernel per gate."""
    _core.require_cuda(params)
    psi_L, saved = _forward(pc, params, dtype, psi0, checkpoints, fuse)
    values = pauli_expectation(H, psi_L)
    sweep = _backward_fused if fuse else _backward_sweep
    grads = sweep(pc, params, H, psi_L, saved, dtype)
    return values, grads


class _Expectation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, pc, H, psi0, dtype, checkpoints):
        psi_L, saved = _forward(pc, params, dtype, psi0, checkpoints)
        ctx.pc, ctx.H, ctx.dtype = pc, H, dtype
        ctx.psi_L, ctx.saved = psi_L, saved
        ctx.save_for_backward(params)
        return pauli_expectation(H, psi_L)

    @staticmethod
    def backward(ctx, g):
        (params,) = ctx.saved_tensors
        grads = _backward_fused(ctx.pc, params, ctx.H, ctx.psi_L,
                                ctx.saved, ctx.dtype)
        ctx.psi_L = ctx.saved = None
        out = (g.to(torch.float64).unsqueeze(-1) * grads).to(params.dtype)
        return out, None, None, None, None, None


def expectation(pc: ParamCircuit, params: torch.Tensor, H: PauliSum,
                psi0: Optional[torch.Tensor] = None, dtype=torch.complex64,
                checkpoints: bool = True) -> torch.Tensor:
    """<psi(params)|H|psi(params)> per batch entry (float64), differentiable
    with respect to ``params`` by the adjoint method."""
    _core.require_cuda(params)
    if params.dim() != 2 or params.shape[1] != pc.num_params:
        raise ValueError(f"params must be (B, {pc.num_params}), got "
                         f"{tuple(params.shape)}")
    return _Expectation.apply(params, pc, H, psi0, dtype, checkpoints)
