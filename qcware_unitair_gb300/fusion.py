"""Circuits, the fusion planner, and compiled programs.

A ``Circuit`` is an ordered list of gates (matrix + qubits).  ``compile``
turns it into a ``Program``: a sequence of fused stages (one HBM pass each,
``gbsv_run_stage``) and, for gates a stage cannot hold, single-gate launches
(``gbsv_apply_operator``).  ``fuse=False`` gives the plain path: one kernel
per gate, exactly what a loop of ``apply_operator`` calls launches.

Planner (greedy, in circuit order).  A stage owns m tile bits: the lowest
``c_min`` amplitude-index bits always (so tiles are made of >= 128-byte
contiguous runs) plus the bits its gates need.  A gate needs
  * dense 1-/2-qubit gate: its target bits;
  * controlled-U (a 4x4 of the form diag(I, U), control = first qubit): the
    target bit only -- a control outside the tile becomes a per-tile
    condition;
  * diagonal gate on 1-2 qubits: nothing -- outside the tile it is a factor
    per tile, inside a per-amplitude scale.
A gate joins the current stage if the union of needed bits still fits in m;
otherwise the stage closes and a new one starts.  Closed stages are topped up
to m bits with the lowest free positions (longer contiguous runs).
Wider gates (k >= 3 dense) run as single-gate launches between stages.

This generalises the host-side fusion unitair does in apply_to_qubits
(src/unitair/simulation/operations.py:416-503, gates/matrix_algebra.py:6-51,
which only multiplies repeated single-qubit gates on one qubit).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _core, _lib
from .circuits import Gate as NamedGate, gate_matrix

FG_DENSE1, FG_DENSE2, FG_DIAG = 0, 1, 2
FG_DTYPE = np.dtype([("kind", "<i4"), ("nq", "<i4"), ("b0", "<i4"),
                     ("b1", "<i4"), ("cmask", "<u8"), ("cval", "<u8"),
                     ("mat", "<i8"), ("mat_bstride", "<i8")])
assert FG_DTYPE.itemsize == 48

DENSE, DIAG, CTRL = "dense", "diag", "ctrl"


@dataclass
class CircuitGate:
    """A gate: ``matrix`` is (d, d) or (B, d, d) (torch tensor, any device)
    and ``kind`` says which structure the planner may exploit."""
    matrix: torch.Tensor
    qubits: Tuple[int, ...]
    kind: str = DENSE


def classify(matrix: torch.Tensor) -> str:
    """Structure of a host matrix: diagonal, controlled-U (4x4 diag(I, U))
    or dense.  Exact zeros only (gate builders produce them)."""
    m = matrix.detach()
    if m.is_cuda:
        return DENSE  # no device->host sync just to classify
    d = m.shape[-1]
    eye = torch.eye(d, dtype=torch.bool)
    off = m.masked_select(~eye.expand(m.shape)) if m.numel() else m
    if not bool((off != 0).any()):
        return DIAG
    if d == 4:
        tl = m[..., :2, :2]
        if (bool((m[..., :2, 2:] == 0).all()) and
                bool((m[..., 2:, :2] == 0).all()) and
                bool((tl == torch.eye(2, dtype=m.dtype)).all())):
            return CTRL
    return DENSE


class Circuit:
    """Ordered gates on ``num_qubits`` qubits (qubit 0 = most significant
    bit of the amplitude index, first listed qubit = matrix MSB)."""

    def __init__(self, num_qubits: int):
        self.num_qubits = int(num_qubits)
        self.gates: List[CircuitGate] = []

    def __len__(self):
        return len(self.gates)

    def append(self, matrix, qubits: Sequence[int],
               kind: Optional[str] = None) -> "Circuit":
        if not isinstance(matrix, torch.Tensor):
            matrix = torch.as_tensor(np.asarray(matrix))
        qubits = tuple(int(q) for q in qubits)
        if len(set(qubits)) != len(qubits) or any(
                q < 0 or q >= self.num_qubits for q in qubits):
            raise ValueError(f"bad qubits {qubits} for {self.num_qubits} "
                             "qubits")
        d = 2 ** len(qubits)
        if matrix.shape[-2:] != (d, d) or matrix.dim() > 3:
            raise ValueError(f"matrix {tuple(matrix.shape)} does not fit "
                             f"{len(qubits)} qubit(s); expected (d, d) or "
                             "(B, d, d)")
        self.gates.append(CircuitGate(matrix, qubits,
                                      kind or classify(matrix)))
        return self

    # named gates of the canonical set
    def _named(self, name, qubits, theta=None, kind=DENSE):
        return self.append(torch.from_numpy(gate_matrix(name, theta)), qubits,
                           kind)

    def h(self, q): return self._named("H", [q])
    def x(self, q): return self._named("X", [q])
    def y(self, q): return self._named("Y", [q])
    def z(self, q): return self._named("Z", [q], kind=DIAG)
    def s(self, q): return self._named("S", [q], kind=DIAG)
    def t(self, q): return self._named("T", [q], kind=DIAG)
    def cnot(self, c, t): return self._named("CNOT", [c, t], kind=CTRL)
    def cz(self, a, b): return self._named("CZ", [a, b], kind=DIAG)
    def swap(self, a, b): return self._named("SWAP", [a, b])

    def rx(self, q, theta): return self._rot("RX", q, theta)
    def ry(self, q, theta): return self._rot("RY", q, theta)
    def rz(self, q, theta): return self._rot("RZ", q, theta)

    def _rot(self, name, q, theta):
        """Rotation by a float or a tensor of per-state angles (B,)."""
        if isinstance(theta, torch.Tensor) and theta.dim() > 0:
            from . import gates as G
            fn = {"RX": G.rx, "RY": G.ry, "RZ": G.rz}[name]
            m = fn(theta.detach().to(torch.float64).cpu(),
                   dtype=torch.complex128)
            return self.append(m, [q], DIAG if name == "RZ" else DENSE)
        return self._named(name, [q], float(theta),
                           DIAG if name == "RZ" else DENSE)

    @classmethod
    def from_gates(cls, num_qubits: int, gates: Sequence[NamedGate]):
        c = cls(num_qubits)
        kinds = {"Z": DIAG, "S": DIAG, "T": DIAG, "RZ": DIAG, "CZ": DIAG,
                 "CNOT": CTRL}
        for g in gates:
            c._named(g.name, list(g.qubits), g.theta, kinds.get(g.name, DENSE))
        return c

    def inverse(self) -> "Circuit":
        c = Circuit(self.num_qubits)
        for g in reversed(self.gates):
            c.append(g.matrix.conj().transpose(-1, -2), g.qubits, g.kind)
        return c

    def compile(self, dtype=torch.complex64, device="cuda", fuse=True,
                tile_qubits: Optional[int] = None,
                min_contiguous: Optional[int] = None,
                layouts: bool = True, native: bool = True,
                tensor_cores: Optional[bool] = None) -> "Program":
        return Program(self, dtype, torch.device(device), fuse, tile_qubits,
                       min_contiguous, layouts, native, tensor_cores)

    def run(self, state: torch.Tensor, fuse: bool = True,
            inplace: bool = False) -> torch.Tensor:
        prog = self.compile(state.dtype, state.device, fuse)
        return prog.run(state, inplace=inplace)


# ------------------------------------------------------------ planning ----
@dataclass
class _Stage:
    tile: set
    gates: List[CircuitGate] = field(default_factory=list)


def _needs(g: CircuitGate, n: int):
    pos = [n - 1 - q for q in g.qubits]
    k = len(pos)
    if g.kind == DIAG and k <= 2:
        return set()
    if g.kind == CTRL and k == 2:
        return {pos[1]}
    if k <= 2:
        return set(pos)
    return None  # not stage-able


def plan(gates: Sequence[CircuitGate], n: int, m: int, c_min: int):
    """Greedy stage plan: list of ('stage', _Stage) / ('plain', gate)."""
    ops = []
    cur: Optional[_Stage] = None
    low = set(range(min(c_min, m)))
    for g in gates:
        need = _needs(g, n)
        if need is not None and len(low | need) > m:
            need = None  # cannot fit even a fresh tile: run it on its own
        if need is None:
            if cur is not None:
                ops.append(("stage", cur))
                cur = None
            ops.append(("plain", g))
            continue
        if cur is None:
            cur = _Stage(set(low))
        if len(cur.tile | need) <= m:
            cur.tile |= need
            cur.gates.append(g)
        else:
            ops.append(("stage", cur))
            cur = _Stage(set(low) | need, [g])
    if cur is not None:
        ops.append(("stage", cur))
    for kind, st in ops:
        if kind == "stage":
            p = 0
            while len(st.tile) < m:
                if p not in st.tile:
                    st.tile.add(p)
                p += 1
    return ops


LAYOUT_DTYPE = np.dtype([("rb", "<i4", (5,)), ("first_gate", "<i4"),
                         ("num_gates", "<i4"), ("pad", "<i4")])
assert LAYOUT_DTYPE.itemsize == 32
FG_CDENSE1, FG_REAL1, FG_ANTI1, FG_CANTI1, FG_PERM2, FG_RDIAG = 3, 4, 5, 6, 7, 8


def _host(m: torch.Tensor) -> Optional[torch.Tensor]:
    """The matrix on the host, or None when looking would need a sync."""
    return None if m.is_cuda else m.detach()


def _is_real(m) -> bool:
    h = _host(m)
    if h is None:
        return False
    return (not h.is_complex()) or bool((h.imag == 0).all())


def _is_anti(m) -> bool:
    h = _host(m)
    return h is not None and bool((h[..., 0, 0] == 0).all()) and bool(
        (h[..., 1, 1] == 0).all())


def _is_unit_swap(m) -> bool:
    h = _host(m)
    return h is not None and bool((h[..., 0, 1] == 1).all()) and bool(
        (h[..., 1, 0] == 1).all())


def _perm_code(m) -> Optional[int]:
    """4x4 0/1 permutation shared by every batch entry -> packed sources."""
    h = _host(m)
    if h is None:
        return None
    h = h.reshape(-1, 4, 4)
    if not bool(((h == 0) | (h == 1)).all()):
        return None
    code = 0
    for r in range(4):
        cols = [c for c in range(4) if bool((h[:, r, c] == 1).all())]
        if len(cols) != 1 or bool((h[:, r, :] != 0).sum(-1).ne(1).any()):
            return None
        code |= cols[0] << (2 * r)
    return code


def _dense1_kind(u) -> Tuple[int, int]:
    """(kind, nq flag) for a 2x2 applied on a register bit."""
    if _is_anti(u):
        return FG_ANTI1, int(_is_unit_swap(u))
    if _is_real(u):
        return FG_REAL1, 0
    return FG_DENSE1, 0


def _to_device(arr: Optional[np.ndarray], dev) -> torch.Tensor:
    """One pinned, non-blocking host-to-device copy (no host stall behind
    work already queued on the stream)."""
    if arr is None:
        return torch.zeros(64, dtype=torch.uint8, device=dev)
    t = torch.from_numpy(np.ascontiguousarray(arr).reshape(-1).copy())
    if dev.type == "cuda":
        t = t.pin_memory()
    return t.to(dev, non_blocking=True)


def _record(g: CircuitGate, n: int, local: dict, kreg: Optional[dict],
            rb: int = 0):
    """Gate record and its pool values.  ``local`` maps positions to tile
    bits; ``kreg`` (register-blocked stages) maps tile bits to register
    bits, None for the shared-memory stage kernel."""
    pos = [n - 1 - q for q in g.qubits]
    mat = g.matrix
    rec = np.zeros((), dtype=FG_DTYPE)
    reg = (lambda b: kreg[b]) if kreg is not None else (lambda b: b)
    if kreg is not None:
        return _layout_record(g, pos, mat, rec, local, kreg, rb)
    if g.kind == DIAG:
        vals = torch.diagonal(mat, dim1=-2, dim2=-1)
        bs = [local[p] if p in local else -1 - p for p in pos]
        rec["kind"], rec["nq"] = FG_DIAG, len(pos)
        rec["b0"] = bs[0]
        rec["b1"] = bs[1] if len(bs) > 1 else 0
    elif g.kind == CTRL and pos[0] not in local:
        vals = mat[..., 2:, 2:].reshape(mat.shape[:-2] + (4,))
        rec["kind"], rec["b0"] = FG_DENSE1, reg(local[pos[1]])
        rec["cmask"] = rec["cval"] = np.uint64(1 << pos[0])
    elif (g.kind == CTRL and kreg is not None
          and local[pos[0]] not in kreg):
        # control on a thread bit: a per-thread condition
        vals = mat[..., 2:, 2:].reshape(mat.shape[:-2] + (4,))
        rec["kind"] = FG_CDENSE1
        rec["b0"], rec["b1"] = reg(local[pos[1]]), local[pos[0]]
    elif len(pos) == 1:
        vals = mat.reshape(mat.shape[:-2] + (4,))
        rec["kind"], rec["b0"] = FG_DENSE1, reg(local[pos[0]])
    else:
        vals = mat.reshape(mat.shape[:-2] + (16,))
        rec["kind"] = FG_DENSE2
        rec["b0"], rec["b1"] = reg(local[pos[0]]), reg(local[pos[1]])
    return rec, vals


def _layout_record(g, pos, mat, rec, local, kreg, rb):
    """Record for a register-blocked stage, specialised by structure."""
    if g.kind == DIAG:
        vals = torch.diagonal(mat, dim1=-2, dim2=-1)
        enc = []
        for p in pos:
            if p not in local:
                enc.append(-1 - p)
            elif local[p] in kreg:
                enc.append(kreg[local[p]])
            else:
                enc.append(rb + local[p])
        rec["kind"], rec["nq"] = FG_RDIAG, len(pos)
        rec["b0"] = enc[0]
        rec["b1"] = enc[1] if len(enc) > 1 else 0
        return rec, vals
    if g.kind == CTRL:
        u = mat[..., 2:, 2:]
        vals4 = u.reshape(mat.shape[:-2] + (4,))
        c, t = local.get(pos[0]), local[pos[1]]
        if c is None:  # control outside the tile: a per-tile condition
            kind, flag = _dense1_kind(u)
            rec["kind"], rec["nq"], rec["b0"] = kind, flag, kreg[t]
            rec["cmask"] = rec["cval"] = np.uint64(1 << pos[0])
            return rec, vals4
        if c not in kreg:  # control on a thread bit
            if _is_anti(u):
                rec["kind"], rec["nq"] = FG_CANTI1, int(_is_unit_swap(u))
            else:
                rec["kind"] = FG_CDENSE1
            rec["b0"], rec["b1"] = kreg[t], c
            return rec, vals4
    if len(pos) == 1:
        kind, flag = _dense1_kind(mat)
        rec["kind"], rec["nq"], rec["b0"] = kind, flag, kreg[local[pos[0]]]
        return rec, mat.reshape(mat.shape[:-2] + (4,))
    code = _perm_code(mat)
    rec["b0"], rec["b1"] = kreg[local[pos[0]]], kreg[local[pos[1]]]
    if code is not None:
        rec["kind"], rec["nq"] = FG_PERM2, code
    else:
        rec["kind"] = FG_DENSE2
    return rec, mat.reshape(mat.shape[:-2] + (16,))


def _plan_layouts(gates, n, local, m, rb):
    """Group a stage's gates into register layouts (rb tile bits each)."""
    out = []
    need_all: set = set()
    cur: list = []
    for g in gates:
        pos = [n - 1 - q for q in g.qubits]
        if g.kind == DIAG:
            need = set()
        elif g.kind == CTRL and pos[0] not in local:
            need = {local[pos[1]]}
        elif g.kind == CTRL:
            need = {local[pos[1]]}
        else:
            need = {local[p] for p in pos}
        if len(need_all | need) <= rb:
            need_all |= need
            cur.append(g)
        else:
            out.append((need_all, cur))
            need_all, cur = set(need), [g]
    out.append((need_all, cur))
    layouts = []
    for need, lg in out:
        bits = sorted(need)
        b = m - 1  # top up with high tile bits: low bits stay thread bits
        while len(bits) < rb:
            if b not in need:
                bits.append(b)
            b -= 1
        layouts.append((bits, lg))
    return layouts


DESC_DTYPE = np.dtype([("kind", "<i4"), ("nq", "<i4"), ("q0", "<i4"),
                       ("q1", "<i4"), ("mat", "<i8"), ("mat_bstride", "<i8"),
                       ("num_batch", "<i8")])
PLANOP_DTYPE = np.dtype([("type", "<i4"), ("contiguous", "<i4"),
                         ("first", "<i4"), ("count", "<i4"),
                         ("positions", "<i4", (16,))])
_KIND_CODE = {DENSE: 0, DIAG: 1, CTRL: 2}


_NAMED_KIND = {"Z": DIAG, "S": DIAG, "T": DIAG, "RZ": DIAG, "CZ": DIAG,
               "CNOT": CTRL}
_FIXED = {}


def gate_list_desc(gates: Sequence[NamedGate]):
    """Descriptor and complex128 matrix arrays for canonical gates, without
    building per-gate tensors (the serving fast path)."""
    G = len(gates)
    desc = np.zeros(G, dtype=DESC_DTYPE)
    parts = []
    off = 0
    for i, g in enumerate(gates):
        if g.theta is None:
            mat = _FIXED.get(g.name)
            if mat is None:
                mat = _FIXED[g.name] = gate_matrix(g.name).reshape(-1)
        else:
            mat = gate_matrix(g.name, g.theta).reshape(-1)
        q = g.qubits
        desc[i] = (_KIND_CODE[_NAMED_KIND.get(g.name, DENSE)], len(q), q[0],
                   q[1] if len(q) > 1 else 0, off, 0, 1)
        parts.append(mat)
        off += mat.size
    mats = np.concatenate(parts) if parts else np.zeros(1, np.complex128)
    return desc, mats


def _circuit_desc(gates: Sequence[CircuitGate]):
    G = len(gates)
    desc = np.zeros(G, dtype=DESC_DTYPE)
    parts = []
    off = 0
    for i, g in enumerate(gates):
        mat = g.matrix.detach().numpy().astype(np.complex128, copy=False)
        d = mat.shape[-1]
        desc[i] = (_KIND_CODE[g.kind], len(g.qubits), g.qubits[0],
                   g.qubits[1] if len(g.qubits) > 1 else 0, off,
                   d * d if mat.ndim == 3 else 0,
                   mat.shape[0] if mat.ndim == 3 else 1)
        parts.append(mat.reshape(-1))
        off += mat.size
    mats = np.ascontiguousarray(np.concatenate(parts)) if parts else \
        np.zeros(1, np.complex128)
    return desc, mats


def native_plan(gates: Sequence[CircuitGate], n: int, m: int, c_min: int,
                rb: int, fuse: bool, dtype, desc=None,
                mats=None) -> Optional[dict]:
    """Plan with gbsv_plan (C++).  None when a matrix lives on the device
    (reading it would need a sync; the Python planner handles that)."""
    if desc is None:
        if any(g.matrix.is_cuda for g in gates):
            return None
        desc, mats = _circuit_desc(gates)
    G = len(desc)
    cdt = np.complex64 if dtype == torch.complex64 else np.complex128
    max_pool = max(16, sum(16 * max(1, int(x)) for x in desc["num_batch"]))
    ops = np.zeros(max(1, G), dtype=PLANOP_DTYPE)
    recs = np.zeros(max(1, G), dtype=FG_DTYPE)
    lays = np.zeros(max(1, G), dtype=LAYOUT_DTYPE)
    pool = np.zeros(max_pool, dtype=cdt)
    pl = _lib.Plan()
    pl.dtype = _core.complex_code(dtype)
    pl.ops, pl.max_ops = ops.ctypes.data, len(ops)
    pl.records, pl.max_records = recs.ctypes.data, len(recs)
    pl.layouts, pl.max_layouts = lays.ctypes.data, len(lays)
    pl.pool, pl.max_pool = pool.ctypes.data, len(pool)
    rc = _lib.load().gbsv_plan(desc.ctypes.data, G, mats.ctypes.data, n, m,
                               c_min, rb, int(bool(fuse)), ctypes.byref(pl))
    _lib.check(rc, "plan")
    return {"ops": ops[:pl.num_ops], "records": recs[:pl.num_records],
            "layouts": lays[:pl.num_layouts], "pool": pool[:pl.pool_len],
            "used_layouts": bool(pl.used_layouts)}


class Program:
    """A compiled circuit for one dtype/device (see module doc)."""

    def __init__(self, circuit: Circuit, dtype, device, fuse=True,
                 tile_qubits=None, min_contiguous=None, layouts=True,
                 native=True, tensor_cores=None):
        self.native = False
        self.tensor_cores = False
        self.n = n = circuit.num_qubits
        self.dtype = dtype
        self.device = device
        self.code = _core.complex_code(dtype)
        L = _lib.load()
        mmax = int(L.gbsv_fused_max_tile_qubits(self.code))
        self.rb = int(L.gbsv_fused_register_bits(self.code))
        if tile_qubits is None:
            # 12 tile qubits (32 KiB c64 tiles, 4 CTAs per SM) measured
            # fastest on the 30-qubit random circuit among m = 12..14
            tile_qubits = 12
        self.m = min(int(tile_qubits), mmax, n)
        if min_contiguous is None:
            min_contiguous = 4 if dtype == torch.complex64 else 3
        self.c_min = min(int(min_contiguous), self.m)
        # register-blocked stages need rb <= m and at most 512 threads
        self.use_layouts = bool(layouts) and self.rb <= self.m <= self.rb + 9
        self.batch = None  # per-state gate batch size, if any
        for g in circuit.gates:
            if g.matrix.dim() == 3:
                b = g.matrix.shape[0]
                if self.batch not in (None, b):
                    raise ValueError("per-state gates must share one batch "
                                     "size")
                self.batch = b
        # tensor-core stages: complex64, shared matrices held on the host
        # (their block products are formed there; matrices already on the
        # device stay on the register path, which needs no host copy)
        tc_ok = (fuse and dtype == torch.complex64 and n >= 12
                 and self.batch is None and tile_qubits in (None, 12)
                 and not any(g.matrix.is_cuda for g in circuit.gates))
        if tensor_cores is None:
            tensor_cores = tc_ok and layouts
        if tensor_cores:
            if not tc_ok:
                raise ValueError("tensor-core stages need complex64, at "
                                 "least 12 qubits, shared gate matrices on "
                                 "the host and 12 tile qubits")
            from . import tcplan
            self.m = tcplan.TC_M
            self._build_tc(tcplan.plan_tc(circuit.gates, n, self.c_min))
            return
        nat = None
        if native:
            nat = native_plan(circuit.gates, n, self.m, self.c_min,
                              self.rb if self.use_layouts else 0, fuse, dtype)
        if nat is not None and nat["used_layouts"] == self.use_layouts:
            self._build_native(nat, circuit.gates)
            return
        if fuse:
            raw = plan(circuit.gates, n, self.m, self.c_min)
        else:
            raw = [("plain", g) for g in circuit.gates]
        self._build(raw)

    @classmethod
    def from_gate_list(cls, gates: Sequence[NamedGate], num_qubits: int,
                       dtype=torch.complex64, device="cuda", fuse=True):
        """Compile canonical gates straight from their descriptors (the
        serving fast path: no per-gate tensors, native planner)."""
        prog = cls.__new__(cls)
        prog.native = False
        prog.n = n = num_qubits
        prog.dtype = dtype
        prog.device = torch.device(device)
        prog.code = _core.complex_code(dtype)
        L = _lib.load()
        mmax = int(L.gbsv_fused_max_tile_qubits(prog.code))
        prog.rb = int(L.gbsv_fused_register_bits(prog.code))
        prog.m = min(12, mmax, n)
        prog.c_min = min(4 if dtype == torch.complex64 else 3, prog.m)
        prog.use_layouts = prog.rb <= prog.m <= prog.rb + 9
        prog.batch = None
        desc, mats = gate_list_desc(gates)
        nat = native_plan(None, n, prog.m, prog.c_min,
                          prog.rb if prog.use_layouts else 0, fuse, dtype,
                          desc, mats)
        plain = [CircuitGate(torch.from_numpy(
            gate_matrix(g.name, g.theta)), g.qubits) for g in gates] \
            if any(int(o["type"]) == 0 for o in nat["ops"]) else gates
        prog._build_native(nat, plain)
        return prog

    def _build_native(self, nat, gates):
        dev, dt = self.device, self.dtype
        self.ops = []
        for op in nat["ops"]:
            t, c, first, count = (int(op["type"]), int(op["contiguous"]),
                                  int(op["first"]), int(op["count"]))
            if t == 0:
                g = gates[first]
                mat = g.matrix.to(dtype=dt).contiguous()
                if dev.type == "cuda":
                    mat = mat.pin_memory()
                self.ops.append(("plain", mat.to(dev, non_blocking=True),
                                 g.qubits))
                continue
            positions = (ctypes.c_int32 * self.m)(
                *[int(x) for x in op["positions"][:self.m]])
            self.ops.append(("layouts" if t == 2 else "stage", c, positions,
                             first, count))
        recs, lays = nat["records"], nat["layouts"]
        self.gate_records = _to_device(recs.view(np.uint8) if len(recs)
                                       else None, dev)
        self.layout_records = _to_device(lays.view(np.uint8) if len(lays)
                                         else None, dev)
        self.num_layouts = len(lays)
        pool = torch.from_numpy(nat["pool"]) if len(nat["pool"]) else \
            torch.zeros(1, dtype=dt)
        if dev.type == "cuda":
            pool = pool.pin_memory()
        self._staging = pool
        self.pool = pool.to(dev, non_blocking=True)
        self.num_stages = sum(1 for o in self.ops if o[0] != "plain")
        self.num_plain = sum(1 for o in self.ops if o[0] == "plain")
        self.native = True

    # -- packing ---------------------------------------------------------
    def _plain_op(self, g):
        mat = g.matrix.to(dtype=self.dtype).contiguous()
        if self.device.type == "cuda" and not mat.is_cuda:
            mat = mat.pin_memory()
        return ("plain", mat.to(self.device, non_blocking=True), g.qubits)

    def _build_tc(self, raw):
        """Tensor-core stages (tcplan) and single-gate launches."""
        from . import tcplan
        dev = self.device
        blocks, diags, images, factors = [], [], [], []
        self.ops = []
        for kind, item in raw:
            if kind == "plain":
                self.ops.append(self._plain_op(item))
                continue
            first = len(blocks)
            c, order = tcplan.encode_stage(item, self.n, blocks, diags,
                                           images, factors)
            positions = (ctypes.c_int32 * tcplan.TC_M)(*order)
            self.ops.append(("tc", c, positions, first, len(blocks) - first))
        self.tc_blocks = _to_device(
            np.stack(blocks).view(np.uint8) if blocks else None, dev)
        self.tc_diags = _to_device(
            np.stack(diags).view(np.uint8) if diags else None, dev)
        self.tc_images = _to_device(
            np.concatenate(images).view(np.uint8) if images else None, dev)
        self.tc_factors = _to_device(
            np.concatenate(factors).view(np.uint8) if factors else None, dev)
        self.tc_records = (blocks, diags, images, factors)  # host copies
        self.gate_records = self.layout_records = _to_device(None, dev)
        self.num_layouts = 0
        self.pool = torch.zeros(1, dtype=self.dtype, device=dev)
        self.num_stages = sum(1 for o in self.ops if o[0] != "plain")
        self.num_plain = sum(1 for o in self.ops if o[0] == "plain")
        self.tensor_cores = True

    def _build(self, raw):
        n, dev, dt = self.n, self.device, self.dtype
        records = []
        layouts = []
        pool_parts = []
        pool_len = 0

        self.gate_pool = {}  # id(gate) -> (pool offset, values per state)

        def add_pool(values: torch.Tensor, gate=None):
            """values (nv,) or (B, nv) -> (offset, bstride).  Host values
            stay on the host until one transfer at the end."""
            nonlocal pool_len
            v = values.to(dtype=dt)
            off = pool_len
            pool_parts.append(v.reshape(-1))
            pool_len += v.numel()
            if gate is not None:
                self.gate_pool[id(gate)] = (off, v.shape[-1])
            return off, (v.shape[1] if v.dim() == 2 else 0)

        self.ops = []
        for kind, item in raw:
            if kind == "plain":
                g = item
                mat = g.matrix.to(dtype=dt).contiguous()
                if dev.type == "cuda" and not mat.is_cuda:
                    mat = mat.pin_memory()
                mat = mat.to(dev, non_blocking=True)
                self.ops.append(("plain", mat, g.qubits))
                continue
            st: _Stage = item
            c = 0
            while c in st.tile:
                c += 1
            c = min(c, self.m)
            order = list(range(c)) + sorted(p for p in st.tile if p >= c)
            local = {p: i for i, p in enumerate(order)}
            positions = (ctypes.c_int32 * self.m)(*order)
            if self.use_layouts:
                first_layout = len(layouts)
                for rbits, lgates in _plan_layouts(st.gates, n, local,
                                                   self.m, self.rb):
                    first = len(records)
                    kreg = {b: k for k, b in enumerate(rbits)}
                    for g in lgates:
                        rec, vals = _record(g, n, local, kreg, self.rb)
                        off, bstride = add_pool(vals, g)
                        rec["mat"], rec["mat_bstride"] = off, bstride
                        records.append(rec)
                    lay = np.zeros((), dtype=LAYOUT_DTYPE)
                    lay["rb"][:len(rbits)] = rbits
                    lay["first_gate"], lay["num_gates"] = first, len(lgates)
                    layouts.append(lay)
                self.ops.append(("layouts", c, positions, first_layout,
                                 len(layouts) - first_layout))
                continue
            first = len(records)
            for g in st.gates:
                rec, vals = _record(g, n, local, None)
                off, bstride = add_pool(vals, g)
                rec["mat"], rec["mat_bstride"] = off, bstride
                records.append(rec)
            self.ops.append(("stage", c, positions, first, len(st.gates)))
        self.gate_records = _to_device(
            np.stack(records).view(np.uint8) if records else None, dev)
        self.layout_records = _to_device(
            np.stack(layouts).view(np.uint8) if layouts else None, dev)
        self.num_layouts = len(layouts)
        if not pool_parts:
            self.pool = torch.zeros(1, dtype=dt, device=dev)
        elif all(not p.is_cuda for p in pool_parts):
            host = torch.cat(pool_parts)
            if dev.type == "cuda":
                host = host.pin_memory()
            self.pool = host.to(dev, non_blocking=True)
            self._staging = host  # alive until the copy has run
        else:
            self.pool = torch.cat([p.to(dev) for p in pool_parts])
        self.num_stages = sum(1 for o in self.ops if o[0] != "plain")
        self.num_plain = sum(1 for o in self.ops if o[0] == "plain")

    @property
    def num_passes(self) -> int:
        """HBM passes over the state (one per stage or single-gate launch)."""
        return len(self.ops)

    # -- running ---------------------------------------------------------
    def run(self, state: torch.Tensor, inplace: bool = False,
            renorm_every: Optional[int] = None) -> torch.Tensor:
        """Apply the program to ``state`` (*batch, 2^n); a per-state gate
        batch must equal the flattened state batch.

        ``renorm_every=K`` adds a renormalisation checkpoint after every K
        passes (gbsv_renormalize): each state is rescaled to the squared
        norm it started with, measured in FP64 before the first pass.  A
        unitary circuit preserves the norm; rounding over thousands of gates
        drifts it.  ``renorm_drift()`` reports the largest relative drift
        the checkpoints removed."""
        _core.require_cuda(state)
        if state.dtype != self.dtype:
            raise RuntimeError(f"program compiled for {self.dtype}, state is "
                               f"{state.dtype}")
        if state.shape[-1] != 2 ** self.n:
            raise ValueError(f"state has {state.shape[-1]} amplitudes, "
                             f"program is for {self.n} qubits")
        B = state.numel() >> self.n
        if self.batch is not None and self.batch != B:
            raise ValueError(f"per-state gates have batch {self.batch}, "
                             f"state batch is {B}")
        if inplace:
            if not state.is_contiguous():
                raise ValueError("in-place run needs a contiguous state")
            out = state
        else:
            out = torch.empty_like(state, memory_format=torch.contiguous_format)
        src = state.contiguous()
        if B == 0:
            return out
        L = _lib.load()
        stream = _core.stream_of(state.device)
        N = 2 ** self.n
        cur = src
        if not self.ops and cur is not out:
            out.copy_(cur)
        self._renorm = []
        if renorm_every:
            from . import states as S
            target = S.norm_squared_fp64(src.reshape(B, N))
            nbytes = int(L.gbsv_reduce_scratch_bytes(B, N))
            scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8,
                                  device=state.device)
        for i, op in enumerate(self.ops):
            self._run_op(op, cur, out, B, N, L, stream)
            cur = out
            if (renorm_every and (i + 1) % int(renorm_every) == 0
                    and i + 1 < len(self.ops)):
                norms = torch.empty(B, dtype=torch.float64,
                                    device=state.device)
                rc = L.gbsv_renormalize(out.data_ptr(), self.code, B, N,
                                        target.data_ptr(), norms.data_ptr(),
                                        scratch.data_ptr(), nbytes, stream)
                _lib.check(rc, "renormalize")
                self._renorm.append((norms, target))
        return out

    def renorm_drift(self) -> float:
        """Largest |norm^2 / target - 1| seen at the last run's
        checkpoints (0 without checkpoints); synchronizes."""
        worst = 0.0
        for norms, target in getattr(self, "_renorm", []):
            d = (norms / target.clamp_min(1e-300) - 1).abs().max()
            worst = max(worst, float(d))
        return worst

    def run_op(self, op, state: torch.Tensor) -> None:
        """One pass of the program (an entry of ``ops``), in place on a
        contiguous state: for timing the stages one at a time."""
        B = state.numel() >> self.n
        self._run_op(op, state, state, B, 2 ** self.n, _lib.load(),
                     _core.stream_of(state.device))

    def _run_op(self, op, cur, out, B, N, L, stream):
        gp = self.gate_records.data_ptr()
        lp = self.layout_records.data_ptr()
        pool = self.pool.data_ptr()
        if op[0] == "stage":
            _, c, positions, first, count = op
            rc = L.gbsv_run_stage(cur.data_ptr(), out.data_ptr(),
                                  self.code, self.n, B, N, self.m, c,
                                  positions, gp + first * 48, count,
                                  pool, stream)
            _lib.check(rc, "run_stage")
        elif op[0] == "tc":
            _, c, positions, first, count = op
            rc = L.gbsv_run_stage_tc(
                cur.data_ptr(), out.data_ptr(), self.code, self.n, B, N,
                self.m, c, positions,
                self.tc_blocks.data_ptr() + first * 64, count,
                self.tc_diags.data_ptr(), self.tc_images.data_ptr(),
                self.tc_factors.data_ptr(), stream)
            _lib.check(rc, "run_stage_tc")
        elif op[0] == "layouts":
            _, c, positions, first, count = op
            rc = L.gbsv_run_stage_layouts(
                cur.data_ptr(), out.data_ptr(), self.code, self.n, B, N,
                self.m, c, positions, gp, lp + first * 32, count, pool,
                stream)
            _lib.check(rc, "run_stage_layouts")
        else:
            _, mat, qubits = op
            op_stride = 0 if mat.dim() == 2 else mat.shape[-1] ** 2
            wide = (cur.data_ptr() == out.data_ptr() and not
                    _core.inplace_ok(self.dtype, len(qubits), self.n,
                                     op_stride != 0))
            dst = torch.empty_like(out) if wide else out
            rc = L.gbsv_apply_operator(
                cur.data_ptr(), dst.data_ptr(), self.code, self.n, B, N,
                mat.data_ptr(), op_stride, _lib.qubit_array(qubits),
                len(qubits), stream)
            _lib.check(rc, "apply_operator")
            if wide:
                out.copy_(dst)
