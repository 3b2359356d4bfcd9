"""Planner for tensor-core stages (complex64, ``gbsv_run_stage_tc``).

A stage owns 12 tile bits (amplitude-index positions): the lowest
``c_min`` always, plus the bits its blocks need.  Within the stage the gates
are grouped, in circuit order, into blocks of at most 5 tile bits; a
block's gates multiply into one 32x32 complex matrix that the kernel
applies on the tensor cores.  A gate joins the open block when the union of
bits still fits in 5 (and the stage's tile in 12); otherwise the block
closes and the gate opens the next one, or, when the tile is full, the
stage closes.

Diagonal gates whose qubits avoid the open block's bits commute with it.
They become the block's "post-diagonals" (applied per amplitude after the
block, from thread-index bits and bits outside the tile, which need no
tile bit at all).  When a later gate of the block touches the qubits of a
post-diagonal, the post-diagonal moves into the block's matrix just before
that gate (it commutes with every block gate in between, whose bits were
disjoint from its own).

This is gate fusion in the sense of unitair's ``apply_to_qubits`` /
``fuse_single_qubit_operators`` (src/unitair/simulation/operations.py:
416-503, gates/matrix_algebra.py:6-51) extended from runs of one-qubit
gates on one qubit to any gates on up to 5 qubits.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

TC_M, TC_RB, TC_TB = 12, 5, 7
TC_MAX_BLOCKS = 64
TC_PAIRS = 1
BLOCK_DTYPE = np.dtype([("rspo", "<i2", (5,)), ("tspo", "<i2", (7,)),
                        ("mat", "<i4"), ("first_diag", "<i4"),
                        ("num_diag", "<i4"), ("flags", "<i4"), ("fac", "<i4"),
                        ("nout", "i1"), ("opos", "i1", (7,)),
                        ("pad", "<i4", (3,))])
TC_MAX_OUT = 5  # outside bits a block's factor table may depend on
DIAG_DTYPE = np.dtype([("nq", "<i4"), ("enc", "<i4", (2,)), ("reg", "<i4"),
                       ("d", "<f4", (8,))])
assert BLOCK_DTYPE.itemsize == 64 and DIAG_DTYPE.itemsize == 48
IMG_BYTES = 16384
IMG_ELEMS = IMG_BYTES // 2  # fp16 values per image: [Bl; Bh]


def tc_swz(l: int) -> int:
    """Tile swizzle (amplitude units) shared with the kernel."""
    return l ^ ((((l >> 4) ^ (l >> 7) ^ (l >> 10)) & 7) << 1)


def _image_index() -> np.ndarray:
    """fp16 element index of the K = 128 x N = 64 operand [Bl; Bh] (rows
    k < 64 Bl, k >= 64 Bh) in one 16 KiB image: core matrices of 8 rows (n)
    x 16 bytes (8 k), K-adjacent ones 128 bytes apart, 8-row groups 2048
    bytes apart."""
    k = np.arange(128)[:, None]
    n = np.arange(64)[None, :]
    off = (n % 8) * 16 + (k % 8) * 2 + (k // 8) * 128 + (n // 8) * 2048
    return off // 2


_IMG_IDX = _image_index()


@dataclass(eq=False)
class _Item:
    gate: object          # fusion.CircuitGate
    pos: frozenset        # amplitude-index positions it acts on
    order: int            # index in the circuit


@dataclass(eq=False)
class _Block:
    bits: set = field(default_factory=set)
    gates: List[_Item] = field(default_factory=list)
    post: List[_Item] = field(default_factory=list)


@dataclass
class TcStagePlan:
    tile: set
    blocks: List[_Block]


class _Stage:
    def __init__(self, low):
        self.tile = set(low)
        self.blocks: List[_Block] = []
        self.cur = _Block()

    def add(self, it: _Item, diag: bool) -> bool:
        cur = self.cur
        if diag and not (it.pos & cur.bits):
            cur.post.append(it)
            return True
        newbits = set(cur.bits) | it.pos
        moved, rest = [], list(cur.post)
        changed = True
        while changed:
            changed = False
            for p in rest:
                if p.pos & newbits:
                    moved.append(p)
                    rest.remove(p)
                    newbits |= p.pos
                    changed = True
                    break
        if len(newbits) <= TC_RB and len(self.tile | newbits) <= TC_M:
            cur.post = rest
            cur.gates += sorted(moved, key=lambda x: x.order) + [it]
            cur.bits = newbits
            self.tile |= newbits
            return True
        if (len(self.tile | it.pos) > TC_M
                or len(self.blocks) + 2 > TC_MAX_BLOCKS):
            return False
        self.blocks.append(cur)
        self.cur = _Block(set(it.pos), [it], [])
        self.tile |= it.pos
        return True

    def finish(self) -> TcStagePlan:
        blocks = self.blocks + [self.cur]
        return TcStagePlan(self.tile, blocks)


def plan_tc(gates: Sequence, n: int, c_min: int = 4):
    """Greedy plan: list of ('tc', TcStagePlan) / ('plain', gate).  Gates on
    more than 5 qubits, or with one matrix per state, run on their own."""
    from .fusion import DIAG
    ops = []
    st: Optional[_Stage] = None
    low = set(range(min(c_min, TC_M)))
    for idx, g in enumerate(gates):
        pos = frozenset(n - 1 - q for q in g.qubits)
        diag = g.kind == DIAG and len(pos) <= 2
        if (len(pos) > TC_RB or g.matrix.dim() == 3 or g.matrix.is_cuda
                or len(low | pos) > TC_M):
            if st is not None:
                ops.append(("tc", st.finish()))
                st = None
            ops.append(("plain", g))
            continue
        it = _Item(g, pos, idx)
        if st is None:
            st = _Stage(low)
        if not st.add(it, diag):
            ops.append(("tc", st.finish()))
            st = _Stage(low)
            ok = st.add(it, diag)
            assert ok
    if st is not None:
        ops.append(("tc", st.finish()))
    return ops


# ----------------------------------------------------------- encoding ----
def _host_matrix(g) -> np.ndarray:
    return g.matrix.detach().cpu().resolve_conj().numpy().astype(
        np.complex128)


def _classes(b: int) -> int:
    """Bank-bit image (low 4 amplitude-address bits) of tile bit b."""
    return tc_swz(1 << b) & 15


def _thread_order(tbits: List[int], pairs: bool) -> List[int]:
    """Order the 7 thread bits so the lowest lane bits hit distinct banks:
    8-byte accesses need the images of lane bits 0-3 independent, 16-byte
    (pair) accesses those of lane bits 0-2 in address bits 1-3."""
    mask = 14 if pairs else 15
    want = 3 if pairs else 4
    basis: List[int] = []
    chosen: List[int] = []

    def reduce(v):
        for b in basis:
            v = min(v, v ^ b)
        return v

    for b in sorted(tbits):
        if len(chosen) == want:
            break
        v = reduce(_classes(b) & mask)
        if v:
            basis.append(v)
            basis.sort(reverse=True)
            chosen.append(b)
    return chosen + [b for b in sorted(tbits) if b not in chosen]


def _embed(mat: np.ndarray, kbits: List[int]) -> np.ndarray:
    """32x32 matrix of a d-qubit gate whose qubit t (t = 0 the matrix MSB)
    is register bit kbits[t]."""
    d = len(kbits)
    i = np.arange(32)
    sub = np.zeros(32, dtype=np.int64)
    mask = 0
    for t, k in enumerate(kbits):
        sub |= ((i >> k) & 1) << (d - 1 - t)
        mask |= 1 << k
    same = (i[:, None] & ~mask) == (i[None, :] & ~mask)
    return np.where(same, mat[sub[:, None], sub[None, :]], 0)


def block_image(U: np.ndarray) -> np.ndarray:
    """fp16 image (8192 values, [Bl; Bh]) of the real form B of U^T:
    Bh = rint(1024 B) (integers), Bl = 1024 B - Bh."""
    Ur, Ui = U.real, U.imag
    B = np.empty((64, 64))
    B[0::2, 0::2] = Ur.T
    B[1::2, 0::2] = -Ui.T
    B[0::2, 1::2] = Ui.T
    B[1::2, 1::2] = Ur.T
    Bs = 1024.0 * B
    Bh = np.rint(Bs)
    Bl = Bs - Bh
    img = np.zeros(IMG_ELEMS, dtype=np.float16)
    img[_IMG_IDX[:64]] = Bl.astype(np.float16)
    img[_IMG_IDX[64:]] = Bh.astype(np.float16)
    return img


def image_matrix(img: np.ndarray) -> np.ndarray:
    """The real 64x64 matrix B an image stands for (Bh + Bl) / 1024,
    as float64 (test helper: what the kernel multiplies by)."""
    Bl = img[_IMG_IDX[:64]].astype(np.float64)
    Bh = img[_IMG_IDX[64:]].astype(np.float64)
    return (Bh + Bl) / 1024.0


def encode_stage(plan: TcStagePlan, n: int, blocks_out: list,
                 diags_out: list, images_out: list, factors_out: list):
    """Records of one stage appended to the program's arrays (factor tables
    to factors_out as complex64 arrays of 128 * 2^nout entries); returns
    (c, positions)."""
    tile = set(plan.tile)
    p = 0
    while len(tile) < TC_M:
        if p not in tile:
            tile.add(p)
        p += 1
    c = 0
    while c in tile:
        c += 1
    c = min(c, TC_M)
    order = list(range(c)) + sorted(q for q in tile if q >= c)
    local = {q: i for i, q in enumerate(order)}
    for blk in plan.blocks:
        lbits = sorted(local[q] for q in blk.bits)
        post_bits = set()
        for it in blk.post:
            post_bits |= {local[q] for q in it.pos if q in local}
        free = [b for b in range(TC_M) if b not in lbits]

        def covers(reg):
            cls = {_classes(b) & 14 for b in range(TC_M) if b not in reg}
            return {2, 4, 8} <= cls

        pads: List[int] = []
        for pref in (True, False):
            for b in sorted(free, reverse=True):
                if len(lbits) + len(pads) == TC_RB:
                    break
                if b in pads or (pref and b in post_bits):
                    continue
                if pref and not covers(set(lbits) | set(pads) | {b}):
                    continue
                pads.append(b)
        for b in sorted(free, reverse=True):  # last resort
            if len(lbits) + len(pads) == TC_RB:
                break
            if b not in pads:
                pads.append(b)
        rb = sorted(lbits + pads)
        pairs = 0 in rb
        tb = _thread_order([b for b in range(TC_M) if b not in rb], pairs)
        kpos = {order[b]: k for k, b in enumerate(rb)}
        U = np.eye(32, dtype=np.complex128)
        for it in blk.gates:
            g = it.gate
            mat = _host_matrix(g)
            kb = [kpos[n - 1 - q] for q in g.qubits]
            U = _embed(mat, kb) @ U
        # post-diagonals on thread bits and at most TC_MAX_OUT outside
        # positions fold into one table of per-thread factors; the rest
        # (a register bit, or more outside positions) stay a list
        opos: List[int] = []
        table_items, listed = [], []
        for it in blk.post:
            enc = []
            for q in it.gate.qubits:
                pq = n - 1 - q
                if pq in local:
                    lb = local[pq]
                    enc.append(("r", rb.index(lb)) if lb in rb
                               else ("t", tb.index(lb)))
                else:
                    enc.append(("o", pq))
            outs = [v for k, v in enc if k == "o"]
            new_out = [v for v in dict.fromkeys(outs) if v not in opos]
            if (all(k != "r" for k, _ in enc)
                    and len(opos) + len(new_out) <= TC_MAX_OUT):
                opos += new_out
                table_items.append((it, enc))
            else:
                listed.append((it, enc))
        fac = -1
        if table_items:
            r = np.arange(128)
            pat = np.arange(2 ** len(opos))
            tab = np.ones((len(pat), 128), dtype=np.complex128)
            for it, enc in table_items:
                vals = np.diagonal(_host_matrix(it.gate))
                idx = np.zeros((len(pat), 128), dtype=np.int64)
                for k, v in enc:
                    bit = (((r >> v) & 1)[None, :] if k == "t" else
                           ((pat >> opos.index(v)) & 1)[:, None])
                    idx = (idx << 1) | bit
                tab = tab * vals[idx]
            fac = sum(f.size for f in factors_out)
            factors_out.append(tab.astype(np.complex64).reshape(-1))
        first_diag = len(diags_out)
        for it, enc in listed:
            vals = np.diagonal(_host_matrix(it.gate)).astype(np.complex64)
            rec = np.zeros((), dtype=DIAG_DTYPE)
            rec["nq"] = len(enc)
            reg = 0
            for t, (k, v) in enumerate(enc):
                if k == "r":
                    rec["enc"][t] = v
                    reg = 1
                elif k == "t":
                    rec["enc"][t] = TC_RB + v
                else:
                    rec["enc"][t] = -1 - v
            rec["reg"] = reg
            d = np.zeros(8, dtype=np.float32)
            d[0:2 * len(vals):2] = vals.real
            d[1:2 * len(vals):2] = vals.imag
            rec["d"] = d
            diags_out.append(rec)
        brec = np.zeros((), dtype=BLOCK_DTYPE)
        brec["rspo"] = [tc_swz(1 << b) for b in rb]
        brec["tspo"] = [tc_swz(1 << b) for b in tb]
        brec["mat"] = len(images_out)
        brec["first_diag"] = first_diag
        brec["num_diag"] = len(diags_out) - first_diag
        brec["flags"] = TC_PAIRS if pairs else 0
        brec["fac"] = fac
        brec["nout"] = len(opos)
        brec["opos"][:len(opos)] = opos
        images_out.append(block_image(U))
        blocks_out.append(brec)
    return c, order
