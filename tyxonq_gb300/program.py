"""Tile-pass planning and execution of gate programs on the GPU.

A *program* is the gate list of one circuit cut into shared-memory tile
passes (``csrc/program.cu``).  ``plan_passes`` schedules gates greedily over
the gate DAG: each pass keeps the lowest ``nlow`` index bits local (for
coalesced HBM access) and adds up to ``t - nlow`` further qubits, taking every
ready gate whose qubits fit.  Within a forward pass single-qubit gates are
folded into neighbouring two-qubit gates (``fuse_pass``), so a pass costs one
HBM round trip plus a few shared-memory sweeps.  Gates that cannot run inside
a tile (k >= 3 dense unitaries, Z projections) split the program into
segments executed by the single-gate kernels.
"""
from __future__ import annotations

import ctypes
import threading
from collections import deque
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .ir import Gate

TILE_OP_DTYPE = np.dtype({
    "names": ["kind", "a", "b", "slot", "xm", "zm", "cm", "gxm", "gzm", "gcm", "gny", "pidx", "pscale", "gcoef",
              "zo", "fuse_next", "zg", "mf", "md"],
    "formats": ["<i4", "<i4", "<i4", "<i4", "<u4", "<u4", "<u4", "<u4", "<u4", "<u4", "<i4", "<i4", "<f8", "<f8",
                "<u4", "<i4", "<u8", ("<f4", 32), ("<f8", 32)],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 56, 64, 68, 72, 80, 208],
    "itemsize": 464,
})


def active_qubits(g: Gate) -> tuple:
    """Qubits that must be local for g to run inside a tile: a Pauli rotation
    needs only its X/Y qubits (its Z factors elsewhere become a sign)."""
    if g.kind == "prot":
        return tuple(q for q, p in g.pauli if p in ("X", "Y"))
    return tuple(g.qubits)
TOP = {"u1": 1, "d1": 2, "u2": 3, "cx": 4, "cz": 5, "swap": 6, "prot": 7}
TILE_KINDS = {"u1", "d1", "u2", "cx", "cz", "swap", "prot"}
MAX_BITS = 16
DEFAULT_NLOW = 5


class TilePass(ctypes.Structure):
    _fields_ = [("t", ctypes.c_int32), ("nlow", ctypes.c_int32), ("op_begin", ctypes.c_int32),
                ("op_end", ctypes.c_int32), ("pos", ctypes.c_int32 * MAX_BITS)]


def tileable(g: Gate) -> bool:
    if g.kind in TILE_KINDS:
        return True
    return g.kind == "uk" and len(g.qubits) <= 2


def _canon(g: Gate) -> Gate:
    if g.kind == "uk" and len(g.qubits) == 1:
        return Gate("u1", g.qubits, g.mat, rot=g.rot)
    if g.kind == "uk" and len(g.qubits) == 2:
        return Gate("u2", g.qubits, g.mat, rot=g.rot)
    return g


# ---------------------------------------------------------------- diagonal commuting
def _commutes_with_diag(h: Gate, q: int) -> bool:
    """Whether gate h commutes exactly with any diagonal single-qubit gate on q."""
    if q not in h.qubits:
        return True
    if h.kind in ("d1", "cz"):
        return True
    return h.kind == "cx" and h.qubits[0] == q  # a diagonal on the control commutes


def _is_1q_on(h: Gate, q: int) -> bool:
    return h.kind in ("u1", "d1") and len(h.qubits) == 1 and h.qubits[0] == q


def commute_diagonals(gates: Sequence[Gate]) -> list[int]:
    """An execution order in which each diagonal single-qubit gate sits next to
    a single-qubit gate on the same qubit whenever only gates it commutes with
    (gates on other qubits, CZ, CX controlled by it, other diagonals) stand
    between them: first moved back to the previous such gate, else forward to
    the next one.  Adjacent single-qubit gates on one qubit are fused into one
    2x2 by the pass encoder, so each move removes one register routine.  The
    order is a list of gate indices; the state it produces equals the
    original's up to rounding."""
    def backward(order: list[int], skip_merged: bool) -> list[int]:
        out: list[int] = []
        for gi in order:
            g = gates[gi]
            if g.kind == "d1" and len(g.qubits) == 1:
                q = g.qubits[0]
                if skip_merged and out and _is_1q_on(gates[out[-1]], q):
                    out.append(gi)
                    continue
                j = len(out) - 1
                while j >= 0 and not _is_1q_on(gates[out[j]], q) and _commutes_with_diag(gates[out[j]], q):
                    j -= 1
                if j >= 0 and _is_1q_on(gates[out[j]], q):
                    out.insert(j + 1, gi)
                    continue
            out.append(gi)
        return out

    order = backward(list(range(len(gates))), False)
    # forward moves: the same scan on the reversed order (merged diagonals stay)
    rev = backward(order[::-1], True)
    return rev[::-1]


# ---------------------------------------------------------------- planning
@dataclass
class PassPlan:
    qubits: list  # local qubits (sorted by bit position ascending)
    gates: list  # gate indices in execution order
    nlow: int = DEFAULT_NLOW  # the lowest nlow index bits are local


@dataclass
class Segment:
    kind: str  # 'tiles' or 'gate'
    passes: list = field(default_factory=list)  # list[PassPlan]
    gate: int = -1


def plan_passes(gates: Sequence[Gate], n: int, t: int, nlow: int = DEFAULT_NLOW,
                max_ops: int | None = None) -> list[Segment]:
    """Greedy DAG scheduling of `gates` into tile passes of t local qubits
    (at most max_ops gates per pass when given)."""
    t = min(t, n)

    def fits(g: Gate) -> bool:
        return tileable(g) and (len(set(active_qubits(g))) <= t - 1 or t == n)

    # keep room for the widest tile gate next to the always-local low bits
    maxw = max([len(set(active_qubits(g))) for g in gates if fits(g)] or [1])
    nlow = n if t == n else max(1, min(nlow, t - maxw))
    low = set(range(n - nlow, n))  # qubits whose bits are 0..nlow-1
    queues: list[deque] = [deque() for _ in range(n)]
    for i, g in enumerate(gates):
        for q in set(g.qubits):
            queues[q].append(i)
    done = [False] * len(gates)

    def is_ready(i: int) -> bool:
        return all(queues[q] and queues[q][0] == i for q in set(gates[i].qubits))

    ready = set(i for i in range(len(gates)) if is_ready(i))
    segments: list[Segment] = []
    remaining = len(gates)

    def execute(i: int):
        nonlocal remaining
        done[i] = True
        remaining -= 1
        ready.discard(i)
        for q in set(gates[i].qubits):
            queues[q].popleft()
            if queues[q]:
                h = queues[q][0]
                if not done[h] and is_ready(h):
                    ready.add(h)

    while remaining:
        # plain-kernel gates that are ready run first
        plain = sorted(i for i in ready if not fits(gates[i]))
        if plain:
            for i in plain:
                segments.append(Segment("gate", gate=i))
                execute(i)
            continue
        L = set(low)
        order: list[int] = []
        while max_ops is None or len(order) < max_ops:
            best, best_cost = None, None
            for i in ready:
                g = gates[i]
                if not fits(g):
                    continue
                new = set(active_qubits(g)) - L
                if len(L) + len(new) > t:
                    continue
                c = len(new)
                if best is None or c < best_cost or (c == best_cost and i < best):
                    best, best_cost = i, c
                    if c == 0:
                        break
            if best is None:
                break
            L |= set(active_qubits(gates[best]))
            order.append(best)
            execute(best)
        if not order:  # pragma: no cover - a ready tileable gate always fits an empty pass
            raise RuntimeError("tile planner made no progress")
        # pad the local set up to t with the lowest free bits (bigger, fewer tiles)
        for q in range(n - 1, -1, -1):
            if len(L) >= t:
                break
            L.add(q)
        qs = sorted(L, key=lambda q: n - 1 - q)
        if segments and segments[-1].kind == "tiles":
            segments[-1].passes.append(PassPlan(qs, order, min(nlow, len(qs))))
        else:
            segments.append(Segment("tiles", passes=[PassPlan(qs, order, min(nlow, len(qs)))]))
    return segments


# ---------------------------------------------------------------- fusion
def _kron_local(P: np.ndarray, which: int) -> np.ndarray:
    I = np.eye(2, dtype=np.complex128)
    return np.kron(P, I) if which == 0 else np.kron(I, P)


def _mat4(g: Gate) -> np.ndarray:
    from . import gates as G

    if g.kind == "u2":
        return g.mat
    return {"cx": G.gate_cx_4x4, "cz": G.gate_cz_4x4, "swap": G.gate_swap_4x4}[g.kind]()


def fuse_pass(gates: Sequence[Gate], absorb: bool = True) -> list[Gate]:
    """Merge runs of single-qubit gates; with absorb=True also fold them into
    neighbouring two-qubit gates (fewer shared-memory sweeps), with
    absorb=False keep CX/CZ/SWAP as permutations (fewer flops when ops run in
    registers).  Forward only."""
    out: list[Gate] = []
    pending: dict[int, np.ndarray] = {}
    last: dict[int, int] = {}
    for g0 in gates:
        g = _canon(g0)
        if g.kind in ("u1", "d1"):
            q = g.qubits[0]
            M = g.mat if g.kind == "u1" else np.diag(np.diag(g.mat))
            pending[q] = M @ pending[q] if q in pending else M.copy()
        elif g.kind in ("u2", "cx", "cz", "swap") and not absorb:
            for q in g.qubits:
                if q in pending:
                    out.append(_one_q(q, pending.pop(q)))
            out.append(g)
        elif g.kind in ("u2", "cx", "cz", "swap"):
            a, b = g.qubits
            pa, pb = pending.pop(a, None), pending.pop(b, None)
            if pa is None and pb is None:
                out.append(g)
            else:
                M = _mat4(g)
                if pa is not None:
                    M = M @ _kron_local(pa, 0)
                if pb is not None:
                    M = M @ _kron_local(pb, 1)
                out.append(Gate("u2", (a, b), M))
            last[a] = last[b] = len(out) - 1
        else:  # prot: flush its qubits first
            for q in g.qubits:
                if q in pending:
                    out.append(_one_q(q, pending.pop(q)))
                    last[q] = len(out) - 1
            out.append(g)
            for q in g.qubits:
                last[q] = len(out) - 1
    for q, P in pending.items():
        j = last.get(q) if absorb else None
        if j is not None and out[j].kind in ("u2", "cx", "cz", "swap"):
            tg = out[j]
            M = _mat4(tg)
            which = 0 if tg.qubits[0] == q else 1
            out[j] = Gate("u2", tg.qubits, _kron_local(P, which) @ M)
        else:
            out.append(_one_q(q, P))
    return out


def _one_q(q: int, M: np.ndarray) -> Gate:
    if abs(M[0, 1]) == 0 and abs(M[1, 0]) == 0:
        return Gate("d1", (q,), M)
    return Gate("u1", (q,), M)


# ---------------------------------------------------------------- encoding
_PH = [1.0, 1j, -1.0, -1j]


def _generator(g: Gate, loc: dict) -> tuple[int, int, int, int, float] | None:
    """(gxm, gzm, gcm, gny, coef) with dE/dangle = coef * Im<lam|G|psi>."""
    if g.rot is None:
        return None
    name = g.rot[0]
    if name in ("rx", "ry", "rz", "rxx", "ryy", "rzz"):
        from .ir import ROTATION_GENERATORS

        ps = ROTATION_GENERATORS[name]
        xm = zm = ny = 0
        for q, p in zip(g.qubits, ps):
            b = 1 << loc[q]
            if p in "XY":
                xm |= b
            if p in "YZ":
                zm |= b
            ny += p == "Y"
        return xm, zm, 0, ny, 1.0
    if name == "cry":
        c, tq_ = g.qubits
        return 1 << loc[tq_], 1 << loc[tq_], 1 << loc[c], 1, 1.0
    if name == "phase":
        return 0, 0, 1 << loc[g.qubits[0]], 0, -2.0
    if name == "prot":
        # Z factors outside `loc` enter through the op's zo / zg sign
        xm = zm = ny = 0
        for q, p in g.pauli:
            if q not in loc:
                continue
            b = 1 << loc[q]
            if p in "XY":
                xm |= b
            if p in "YZ":
                zm |= b
            ny += p == "Y"
        return xm, zm, 0, ny, 1.0
    return None


def _rotation_masks(g: Gate, loc: dict, outer: dict | None = None, n: int | None = None) -> tuple | None:
    """(xm, zm, cm, ny, zo, zg) of a Pauli-rotation gate (rx/ry/rz/rxx/ryy/rzz/cry/prot).
    X/Y qubits must be in `loc`; Z qubits outside it go to zo (local bit via
    `outer`, for register stages) or zg (global basis-index bit)."""
    from .ir import ROTATION_GENERATORS

    if g.rot is None:
        return None
    name = g.rot[0]
    if name in ROTATION_GENERATORS:
        pairs = list(zip(g.qubits, ROTATION_GENERATORS[name]))
        cm = 0
    elif name == "prot":
        pairs = list(g.pauli)
        cm = 0
    elif name == "cry":
        pairs = [(g.qubits[1], "Y")]
        cm = 1 << loc[g.qubits[0]]
    else:
        return None
    xm = zm = ny = zo = zg = 0
    for q, p in pairs:
        if q not in loc:
            if p != "Z":
                raise ValueError(f"qubit {q} ({p}) of a rotation is not local")
            if outer is not None and q in outer:
                zo |= 1 << outer[q]
            else:
                if n is None:
                    raise ValueError("a non-local Z factor needs the qubit count")
                zg |= 1 << (n - 1 - q)
            continue
        b = 1 << loc[q]
        if p in "XY":
            xm |= b
        if p in "YZ":
            zm |= b
        ny += p == "Y"
    return xm, zm, cm, ny, zo, zg


def op_fields(g: Gate, loc: dict, slot: int = -1, gen=None, pidx: int = -1, pscale: float = 1.0,
              gcoef: float = 0.0, as_rotation: bool = False, outer: dict | None = None,
              n: int | None = None) -> tuple:
    """Field values of one tq_tile_op: (kind, a, b, slot, xm, zm, cm, gxm, gzm,
    gcm, gny, pidx, pscale, gcoef, zo, zg, matrix entries or None).
    as_rotation=True encodes Pauli rotations (and cry) as kind 7, which is
    cheaper than a dense 4x4 sweep; pidx >= 0 makes the device build the
    rotation from theta[pidx] * pscale.  `outer` (local bits, for register
    stages) and `n` place Z factors of Pauli rotations outside `loc`."""
    g = _canon(g)
    rm = _rotation_masks(g, loc, outer, n) if (as_rotation or pidx >= 0 or g.kind == "prot") else None
    xm = zm = cm = zo = zg = 0
    if rm is not None:
        a = b = 0
        xm, zm, cm, ny, zo, zg = rm
        kind = TOP["prot"]
        ang = g.rot[1]
        c, s = np.cos(0.5 * ang), np.sin(0.5 * ang)
        m = np.array([c, -1j * s * _PH[ny & 3]], dtype=np.complex128)
    else:
        a = loc[g.qubits[0]]
        b = loc[g.qubits[1]] if len(g.qubits) > 1 else 0
        if g.kind in ("u1", "u2"):
            kind = TOP[g.kind]
            m = np.asarray(g.mat, dtype=np.complex128).reshape(-1)
        elif g.kind == "d1":
            kind = TOP["d1"]
            m = np.array([g.mat[0, 0], g.mat[1, 1]], dtype=np.complex128)
        else:
            kind = TOP[g.kind]
            m = None
    if pidx >= 0 and rm is None and not (g.rot is not None and g.rot[0] == "phase"):
        raise ValueError(f"gate '{g.kind}' cannot take a device-side angle")
    gx, gz, gc, gn = gen[:4] if gen is not None else (0, 0, 0, 0)
    return (kind, a, b, slot, xm, zm, cm, gx, gz, gc, gn, pidx, pscale, gcoef, zo, zg, m)


_SCALAR_FIELDS = ["kind", "a", "b", "slot", "xm", "zm", "cm", "gxm", "gzm", "gcm", "gny", "pidx", "pscale", "gcoef",
                  "zo", "zg"]


def pack_ops(fields: list) -> np.ndarray:
    """Column-wise fill of a tq_tile_op array from op_fields tuples (an optional
    18th entry is fuse_next)."""
    arr = np.zeros(len(fields), dtype=TILE_OP_DTYPE)
    if not fields:
        return arr
    for k, name in enumerate(_SCALAR_FIELDS):
        arr[name] = [f[k] for f in fields]
    arr["fuse_next"] = [f[17] if len(f) > 17 else 0 for f in fields]
    for size in (2, 4, 16):
        idx = [i for i, f in enumerate(fields) if f[16] is not None and f[16].size == size]
        if idx:
            M = np.stack([fields[i][16] for i in idx])
            flat = np.stack([M.real, M.imag], axis=-1).reshape(len(idx), -1)
            arr["md"][idx, : 2 * size] = flat
            arr["mf"][idx, : 2 * size] = flat.astype(np.float32)
    return arr


@dataclass
class EncodedTiles:
    passes: ctypes.Array
    n_passes: int
    ops_host: np.ndarray
    ops_dev: torch.Tensor | None = None

    def device_ops(self, device) -> torch.Tensor:
        if self.ops_dev is None or self.ops_dev.device != torch.device(device):
            raw = self.ops_host.tobytes() or bytes(TILE_OP_DTYPE.itemsize)
            self.ops_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)
        return self.ops_dev


def _fuse_around_params(gl: list, idx: list, params: dict | None) -> list:
    """Fuse maximal runs of fixed gates; parametrised gates stay single ops.
    Returns [(gate, gate index or None)]."""
    out, run = [], []
    for gi, g in zip(idx, gl):
        if params is not None and gi in params:
            out += [(x, None) for x in fuse_pass(run)]
            run = []
            out.append((g, gi))
        else:
            run.append(g)
    out += [(x, None) for x in fuse_pass(run)]
    return out


def encode_passes(n: int, plans: Sequence[PassPlan], gates: Sequence[Gate], *, fuse: bool, reverse: bool = False,
                  slots: dict | None = None, params: dict | None = None,
                  nlow: int = DEFAULT_NLOW) -> tuple[EncodedTiles, list]:
    """Encode pass plans.  reverse=True lists passes and ops in reverse.
    `slots` maps gate index -> gradient slot; `params` maps gate index ->
    (pidx, pscale) for angles read from device theta.  Returns the encoded
    tiles and [(slot, coef)] with dE/d(angle) = coef * Im<lam|G|psi>."""
    fields = []
    passes = []
    coefs = []
    seq = list(reversed(plans)) if reverse else list(plans)
    for pp in seq:
        qs = pp.qubits
        loc = {q: j for j, q in enumerate(qs)}
        t = len(qs)
        idx = list(reversed(pp.gates)) if reverse else list(pp.gates)
        gl = [gates[i] for i in idx]
        begin = len(fields)
        if fuse and not reverse:
            for g, gi in _fuse_around_params(gl, idx, params):
                if gi is None:
                    fields.append(op_fields(g, loc, n=n))
                else:
                    pidx, psc = params[gi]
                    fields.append(op_fields(g, loc, pidx=pidx, pscale=psc, as_rotation=True, n=n))
        else:
            for gi, g in zip(idx, gl):
                slot = -1
                gen = None
                pidx, psc = params[gi] if (params is not None and gi in params) else (-1, 1.0)
                gcoef = 0.0
                if slots is not None and gi in slots:
                    slot = slots[gi]
                    gen = _generator(g, loc)
                    coefs.append((slot, gen[4]))
                    gcoef = gen[4] * psc
                fields.append(op_fields(g, loc, slot, gen, pidx=pidx, pscale=psc, gcoef=gcoef, as_rotation=True,
                                        n=n))
        p = TilePass()
        p.t = t
        p.nlow = min(pp.nlow, t)
        p.op_begin = begin
        p.op_end = len(fields)
        for j, q in enumerate(qs):
            p.pos[j] = n - 1 - q
        passes.append(p)
    arr = (TilePass * max(len(passes), 1))(*passes)
    return EncodedTiles(arr, len(passes), pack_ops(fields)), coefs


# ---------------------------------------------------------------- execution
def default_tile_bits(n: int, dtype: torch.dtype, adjoint: bool = False) -> int:
    from .autotune import tile_bits_for

    return tile_bits_for(n, dtype, adjoint)


@dataclass
class ForwardProgram:
    n: int
    segments: list  # list of ('tiles', EncodedTiles) | ('gate', Gate)
    n_gates: int
    n_passes: int

    def run(self, psi: torch.Tensor, theta: torch.Tensor | None = None, ws: dict | None = None) -> torch.Tensor:
        """Apply the program in place; theta (float64 device tensor) feeds the
        ops compiled with device-side angles.  ws: the caller's workspace dict
        for the specialised passes' op records (needed when callers on
        different streams share this program)."""
        from .engine import execute_plain

        dt = K.dtype_tag(psi)
        th = ctypes.c_void_p(theta.data_ptr()) if theta is not None else None
        for kind, obj in self.segments:
            if kind == "gate":
                execute_plain(psi, [obj])
            elif kind == "staged" and obj.jit is not None:
                from . import jit

                jit.run_staged(obj.jit, obj, psi, self.n, dt, th, K.stream_ptr(psi.device), ws)
            elif kind == "staged" and obj.rb > STAGE_BITS:  # pragma: no cover - never built without kernels
                raise RuntimeError("a 5-bit staged segment needs its specialised kernels")
            elif kind == "staged":
                st, ops = obj.device_tables(psi.device)
                nat.call("tq_sv_run_staged", ctypes.c_void_p(psi.data_ptr()), self.n, dt, obj.passes, obj.n_passes,
                         ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(ops.data_ptr()), th,
                         K.stream_ptr(psi.device))
            else:
                ops = obj.device_ops(psi.device)
                nat.call("tq_sv_run_tiles", ctypes.c_void_p(psi.data_ptr()), self.n, dt, obj.passes, obj.n_passes,
                         ctypes.c_void_p(ops.data_ptr()), th, K.stream_ptr(psi.device))
        return psi

    def specialise(self, dtype, device="cuda", stage_bits: int = 5) -> int:
        """Compile circuit-specialised kernels (runtime CUDA compilation, cached
        per structure) for every register-staged segment; returns the number of
        passes that run them.  stage_bits=5: segments re-encoded with 5-bit
        register stages (32 amplitudes per thread: fewer shared-memory sweeps
        per pass) where every pass takes a specialised kernel; 4-bit stages
        otherwise."""
        import warnings

        from . import jit

        count = 0
        for si, (kind, obj) in enumerate(self.segments):
            if kind != "staged":
                continue
            try:
                if obj.jit is None and stage_bits == 5 and obj.rb == STAGE_BITS:
                    wide = jit.specialise_wide(obj, dtype, device)
                    if wide is not None:
                        self.segments[si] = (kind, wide)
                        obj = wide
                if obj.jit is None and obj.rb == STAGE_BITS:
                    obj.jit = jit.specialise(obj, dtype, device)
            except (nat.TqError, OSError) as e:
                # a runtime compilation that fails leaves the segment on the
                # interpreting kernel: the same results, slower
                warnings.warn(f"specialised pass kernels unavailable, interpreting kernel used: {e}")
            if obj.jit is not None:
                count += obj.jit.n_kernels
        return count


# ---------------------------------------------------------------- register stages
STAGE_DTYPE = np.dtype({"names": ["bits", "op_begin", "op_end"], "formats": [("<i4", 4), "<i4", "<i4"],
                        "offsets": [0, 16, 20], "itemsize": 24})
STAGE_BITS = 4
STAGED_MIN_T = 9


def plan_stages(op_bits: Sequence[tuple], t: int, rb: int = STAGE_BITS,
                dep_bits: Sequence[tuple] | None = None) -> list[tuple[list, list]]:
    """Group ops (given as tuples of local bits, in a valid order) into stages
    of at most `rb` local bits by greedy DAG scheduling; each stage's bit set
    is padded to exactly rb bits with the highest unused local bits.
    dep_bits (default op_bits): the bits that order an op against others (a
    Pauli rotation's Z qubits order it but need not be in the stage)."""
    dep = list(dep_bits) if dep_bits is not None else list(op_bits)
    queues: list[deque] = [deque() for _ in range(t)]
    for i, bs in enumerate(dep):
        for b in set(bs):
            queues[b].append(i)
    done = [False] * len(op_bits)

    def is_ready(i):
        return all(queues[b] and queues[b][0] == i for b in set(dep[i]))

    ready = set(i for i in range(len(op_bits)) if is_ready(i))
    stages = []
    left = len(op_bits)
    while left:
        S: set = set()
        order: list = []
        while True:
            # fewest new bits first; among equals prefer an op on the same bits as
            # the last one (runs of single-qubit ops on one qubit can be fused), then
            # the lowest index
            best, bk = None, None
            last = tuple(sorted(set(op_bits[order[-1]]))) if order else None
            for i in ready:
                new = set(op_bits[i]) - S
                if len(S) + len(new) > rb:
                    continue
                key = (len(new), 0 if tuple(sorted(set(op_bits[i]))) == last else 1, i)
                if best is None or key < bk:
                    best, bk = i, key
            if best is None:
                break
            S |= set(op_bits[best])
            order.append(best)
            done[best] = True
            left -= 1
            ready.discard(best)
            for b in set(dep[best]):
                queues[b].popleft()
                if queues[b] and not done[queues[b][0]] and is_ready(queues[b][0]):
                    ready.add(queues[b][0])
        if not order:  # pragma: no cover - every op has at most rb bits
            raise RuntimeError("stage planner made no progress")
        for b in range(t - 1, -1, -1):
            if len(S) >= rb:
                break
            S.add(b)
        stages.append((sorted(S), order))
    return stages


def _single_bit(f: tuple) -> int | None:
    """Register bit of an op (op_fields tuple) that acts on one register bit with
    no sign from outside the stage, else None (the device's op_mat2 rule)."""
    kind, a, _, _, xm, zm, cm = f[:7]
    zo, zg = f[14], f[15]
    if zo or zg:
        return None
    if kind in (TOP["u1"], TOP["d1"]):
        return a
    if kind == TOP["prot"] and cm == 0:
        if xm and xm & (xm - 1) == 0 and zm & ~xm == 0:
            return xm.bit_length() - 1
        if xm == 0 and zm and zm & (zm - 1) == 0:
            return zm.bit_length() - 1
    return None


def _mark_fusion(fields: list, b: int, e: int) -> None:
    """Set fuse_next on the first op of each run of consecutive single-bit ops on
    the same register bit in fields[b:e] (one stage, forward order)."""
    k = b
    while k < e:
        K = _single_bit(fields[k])
        j = k + 1
        if K is not None:
            while j < e and j - k < 16 and _single_bit(fields[j]) == K:
                j += 1
        if j - k > 1:
            fields[k] = fields[k][:17] + (j - k - 1,)
        k = j


@dataclass
class EncodedStaged:
    passes: ctypes.Array
    n_passes: int
    stages_host: np.ndarray
    ops_host: np.ndarray
    _dev: tuple | None = None
    jit: object | None = None  # jit.JitStaged: circuit-specialised kernels for these passes
    rb: int = STAGE_BITS  # register bits per stage
    stage_bits: list | None = None  # every stage's register bits (host; the device table holds at most 4)
    source: tuple | None = None  # (plans, gates, params, slots) it was encoded from

    def device_tables(self, device):
        if self._dev is None or self._dev[0].device != torch.device(device):
            st = torch.frombuffer(bytearray(self.stages_host.tobytes() or bytes(24)), dtype=torch.uint8).to(device)
            op = torch.frombuffer(bytearray(self.ops_host.tobytes() or bytes(TILE_OP_DTYPE.itemsize)),
                                  dtype=torch.uint8).to(device)
            self._dev = (st, op)
        return self._dev


def encode_staged(n: int, plans: Sequence[PassPlan], gates: Sequence[Gate], params: dict | None = None,
                  slots: dict | None = None, rb: int = STAGE_BITS) -> EncodedStaged:
    """Encode passes as register stages.  Forward (slots None): single-qubit
    runs merged, two-qubit gates kept as permutations / dense 4x4,
    parametrised gates as device-side rotations.  Adjoint (slots given, gates
    already in reverse order): one op per gate, gradient slot = slots[gate],
    generator masks and coefficient in register space."""
    fields, stage_rows, passes = [], [], []
    for pp in plans:
        qs = pp.qubits
        loc = {q: j for j, q in enumerate(qs)}
        t = len(qs)
        idx = list(pp.gates)
        gl = [gates[i] for i in idx]
        items = []  # (gate, pidx, pscale, gate index or None)
        if slots is not None:
            for gi, g in zip(idx, gl):
                pidx, psc = params[gi] if (params is not None and gi in params) else (-1, 1.0)
                items.append((g, pidx, psc, gi))
        else:
            run = []
            for gi, g in zip(idx, gl):
                if params is not None and gi in params:
                    items += [(x, -1, 1.0, None) for x in fuse_pass(run, absorb=False)]
                    run = []
                    items.append((g, params[gi][0], params[gi][1], gi))
                else:
                    run.append(g)
            items += [(x, -1, 1.0, None) for x in fuse_pass(run, absorb=False)]
        # stage bits: qubits that must sit in registers; dependency bits: every local qubit touched
        op_bits = [tuple(loc[q] for q in active_qubits(g)) for g, _, _, _ in items]
        dep_bits = [tuple(loc[q] for q in g.qubits if q in loc) for g, _, _, _ in items]
        st_begin = len(stage_rows)
        for bits, order in plan_stages(op_bits, t, rb=rb, dep_bits=dep_bits):
            reg = {b: k for k, b in enumerate(bits)}
            qreg = {q: reg[loc[q]] for q in qs if loc[q] in reg}
            ob = len(fields)
            for k in order:
                g, pidx, psc, gi = items[k]
                if slots is not None and gi in slots:
                    gen = _generator(g, qreg)
                    fields.append(op_fields(g, qreg, slots[gi], gen, pidx=pidx, pscale=psc, gcoef=gen[4] * psc,
                                            as_rotation=True, outer=loc, n=n))
                else:
                    fields.append(op_fields(g, qreg, pidx=pidx, pscale=psc, as_rotation=pidx >= 0 or slots is not None,
                                            outer=loc, n=n))
            if slots is None:
                _mark_fusion(fields, ob, len(fields))
            stage_rows.append((bits, ob, len(fields)))
        p = TilePass()
        p.t = t
        p.nlow = min(pp.nlow, t)
        p.op_begin = st_begin
        p.op_end = len(stage_rows)
        for j, q in enumerate(qs):
            p.pos[j] = n - 1 - q
        passes.append(p)
    st = np.zeros(len(stage_rows), dtype=STAGE_DTYPE)
    for i, (bits, b, e) in enumerate(stage_rows):
        bl = list(bits)[:STAGE_BITS]
        st[i] = (bl + [-1] * (STAGE_BITS - len(bl)), b, e)
    arr = (TilePass * max(len(passes), 1))(*passes)
    enc = EncodedStaged(arr, len(passes), st, pack_ops(fields))
    enc.rb = rb
    enc.stage_bits = [list(bits) for bits, _, _ in stage_rows]
    enc.source = (list(plans), gates, params, slots, n)
    return enc


def compile_forward(gates: Sequence[Gate], n: int, dtype=torch.complex64, t: int | None = None,
                    nlow: int = DEFAULT_NLOW, fuse: bool = True, params: dict | None = None,
                    staged: bool | None = None) -> ForwardProgram:
    """Plan and encode a forward program.  params: gate index -> (pidx, pscale)
    for gates whose angle is read from device theta at run time.  staged:
    register-staged passes (default when the tile has >= 9 bits)."""
    if any(g.kind == "kraus" for g in gates):
        raise NotImplementedError("Kraus channels are stochastic steps between programs (GpuStatevectorEngine)")
    gates = [_canon(g) for g in gates]
    if fuse:
        order = commute_diagonals(gates)
        if order != list(range(len(gates))):
            gates = [gates[i] for i in order]
            if params is not None:
                where = {old: new for new, old in enumerate(order)}
                params = {where[gi]: v for gi, v in params.items()}
    if t is None:
        t = default_tile_bits(n, dtype)
    t = min(t, n)
    if staged is None:
        staged = (fuse and STAGED_MIN_T <= t <= (13 if dtype == torch.complex64 else 12)
                  and all(len(set(active_qubits(g))) <= STAGE_BITS for g in gates))
    segs = plan_passes(gates, n, t, nlow)
    out = []
    npass = 0
    for s in segs:
        if s.kind == "gate":
            if params is not None and s.gate in params:
                raise NotImplementedError("a device-angle gate must fit a tile (X/Y support <= t-1 qubits)")
            out.append(("gate", gates[s.gate]))
        elif staged:
            enc = encode_staged(n, s.passes, gates, params=params)
            out.append(("staged", enc))
            npass += enc.n_passes
        else:
            enc, _ = encode_passes(n, s.passes, gates, fuse=fuse, params=params, nlow=nlow)
            out.append(("tiles", enc))
            npass += enc.n_passes
    return ForwardProgram(n, out, len(gates), npass)


_FUSED_CACHE: "OrderedDict" = None  # gate-list key -> ForwardProgram (engine calls of the same circuit)
_FUSED_CACHE_MAX = 64
_FUSED_LOCK = threading.Lock()


def _gate_key(g: Gate) -> tuple:
    return (g.kind, tuple(g.qubits), None if g.mat is None else np.asarray(g.mat).tobytes(),
            None if g.rot is None else (g.rot[0], float(g.rot[1])), g.pauli)


def execute_fused(psi: torch.Tensor, gates: Sequence[Gate]) -> torch.Tensor:
    """Run the gates as a fused program; programs of circuits seen before (same
    gates, angles and matrices, size, dtype and device) are reused from a
    small LRU cache instead of being planned and encoded again."""
    global _FUSED_CACHE
    from collections import OrderedDict

    n = K._check_state(psi)
    if n == 0:
        return psi
    key = (n, psi.dtype, str(psi.device), tuple(_gate_key(g) for g in gates))
    with _FUSED_LOCK:
        if _FUSED_CACHE is None:
            _FUSED_CACHE = OrderedDict()
        prog = _FUSED_CACHE.get(key)
        if prog is not None:
            _FUSED_CACHE.move_to_end(key)
    if prog is None:
        prog = compile_forward(gates, n, psi.dtype)
        with _FUSED_LOCK:
            _FUSED_CACHE[key] = prog
            while len(_FUSED_CACHE) > _FUSED_CACHE_MAX:
                _FUSED_CACHE.popitem(last=False)
    return prog.run(psi)
