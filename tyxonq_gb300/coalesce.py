"""Continuous batching of small VQE requests into one device launch.

Requests of up to `res1_max` qubits (13 by default) keep psi and lam in one
CTA's shared memory (the batched path's resident size classes,
`tq_batch_run`), so requests of *different* sessions -- different circuits,
Hamiltonians and sizes -- can share one persistent launch per size class.
The device tables of every registered session live in append-only arenas:

  * op records: each distinct (n, circuit structure) is encoded once
    (forward list with fused single-qubit runs, adjoint list with parameter
    slots) and shared by every session with that structure;
  * Pauli groups and terms of each session's Hamiltonian.

A micro-batch is then one packed host buffer -- the instance table (56 B
per request), per-class work lists, per-class counters and the
concatenated angle vectors -- copied to the device in one transfer, one
`tq_batch_run` launch per size class present, and one copy of the energies
and gradients back.  Nothing is re-encoded per request: a new parameter
vector is data.

The reference evaluates one circuit per call (`devices/base.py:378-381`);
batching across clients is new.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .batch import INST_DTYPE, Schedule, encode_resident, structure_gates
from .hamiltonian import GROUP_DTYPE, TERM_DTYPE
from .program import TILE_OP_DTYPE

_CLASSES = ("res1", "res2", "res4", "res8")  # launch order: largest instances first


class _Arena:
    """Append-only device array of structured records with a host copy.

    Growing reallocates the device buffer; the old one goes to the caller's
    `retired` list so that it stays alive until the launches that read it
    have completed."""

    def __init__(self, dtype: np.dtype, device, capacity: int = 1024):
        self.dtype = dtype
        self.device = device
        self.host = np.zeros(capacity, dtype=dtype)
        self.dev = torch.zeros(capacity * dtype.itemsize, dtype=torch.uint8, device=device)
        self.size = 0

    def append(self, arr: np.ndarray, retired: list) -> int:
        """Copy arr to the end (host and device); returns its first index."""
        n = len(arr)
        base = self.size
        if base + n > len(self.host):
            cap = len(self.host)
            while base + n > cap:
                cap *= 2
            host = np.zeros(cap, dtype=self.dtype)
            host[:base] = self.host[:base]
            dev = torch.zeros(cap * self.dtype.itemsize, dtype=torch.uint8, device=self.device)
            dev[:base * self.dtype.itemsize].copy_(self.dev[:base * self.dtype.itemsize])
            retired.append(self.dev)
            self.host, self.dev = host, dev
        if n:
            self.host[base:base + n] = arr
            raw = torch.from_numpy(self.host[base:base + n].view(np.uint8).copy())
            it = self.dtype.itemsize
            self.dev[base * it:(base + n) * it].copy_(raw.to(self.device))
        self.size = base + n
        return base

    def ptr(self) -> ctypes.c_void_p:
        return ctypes.c_void_p(self.dev.data_ptr())


@dataclass
class SmallSession:
    n: int
    n_params: int
    fwd_begin: int
    fwd_count: int
    adj_begin: int
    adj_count: int
    group_begin: int
    group_count: int
    n_terms: int
    cls: str
    cost: int


class ResidentBatcher:
    """Registers small sessions and evaluates micro-batches of their requests
    (energy and adjoint gradient of each) with one launch per size class."""

    def __init__(self, device="cuda", dtype=torch.complex64, schedule: Schedule | None = None):
        self.device = torch.device(device)
        self.dtype = dtype
        self.dt = K._DT[dtype]
        self.sched = schedule or Schedule.default(dtype, self.device)
        self.res_max = self.sched.res1_max
        self.ops = _Arena(TILE_OP_DTYPE, self.device, 4096)
        self.groups = _Arena(GROUP_DTYPE, self.device, 4096)
        self.terms = _Arena(TERM_DTYPE, self.device, 8192)
        self.structs: dict = {}
        self.sessions: dict[str, SmallSession] = {}
        self.retired: list = []  # device buffers replaced by a grow, freed after the next sync
        lib = nat.load()
        bound = {"res8": self.sched.res8_max, "res4": self.sched.res4_max, "res2": self.sched.res2_max,
                 "res1": self.sched.res1_max}
        self.cls_info = {}
        for name in _CLASSES:
            _, G, T = self.sched.class_of(bound[name])
            self.cls_info[name] = (G, T, int(lib.tq_batch_smem_bytes(self.dt, bound[name], G, 0)))
        self.grid = torch.cuda.get_device_properties(self.device).multi_processor_count

    def fits(self, n: int) -> bool:
        return 1 <= n <= self.res_max

    def table_bytes(self, n: int, n_gates: int, n_groups: int, n_terms: int) -> int:
        """Device bytes one session adds (op records of both lists, groups, terms)."""
        return (2 * n_gates * TILE_OP_DTYPE.itemsize + n_groups * GROUP_DTYPE.itemsize
                + n_terms * TERM_DTYPE.itemsize)

    def register(self, key: str, n: int, structure, n_params: int, H) -> SmallSession:
        """Encode (once per structure) and upload a session's tables."""
        if key in self.sessions:
            return self.sessions[key]
        if not self.fits(n):
            raise ValueError(f"{n} qubits do not fit a resident class (<= {self.res_max})")
        skey = (int(n), tuple((nm, tuple(int(q) for q in qs), p) for nm, qs, p in structure))
        ent = self.structs.get(skey)
        if ent is None:
            gates, params = structure_gates(structure)
            f_ops, a_ops = encode_resident(n, gates, params)
            fb = self.ops.append(f_ops, self.retired)
            ab = self.ops.append(a_ops, self.retired)
            ent = (fb, len(f_ops), ab, len(a_ops))
            self.structs[skey] = ent
        g, t = H.pack()
        tb = self.terms.append(t, self.retired)
        g2 = g.copy()
        g2["first_term"] += tb
        gb = self.groups.append(g2, self.retired)
        cls = self.sched.class_of(n)[0]
        cost = (1 << n) * (ent[1] + ent[3] + 4 * len(t))
        s = SmallSession(int(n), int(n_params), ent[0], ent[1], ent[2], ent[3], gb, len(g2), len(t), cls, cost)
        self.sessions[key] = s
        return s

    def launch(self, items, stream) -> dict:
        """Enqueue one micro-batch on `stream`: items = [(session key, theta)].
        Returns a ticket: event, pinned host results and per-item slices."""
        sess = [self.sessions[k] for k, _ in items]
        m = len(items)
        insts = np.zeros(m, dtype=INST_DTYPE)
        theta_off = np.zeros(m + 1, dtype=np.int64)
        for i, s in enumerate(sess):
            theta_off[i + 1] = theta_off[i] + s.n_params
        for i, s in enumerate(sess):
            r = insts[i]
            r["n"] = s.n
            r["streamed"] = 0
            r["fwd_begin"], r["fwd_count"], r["adj_begin"], r["adj_count"] = (s.fwd_begin, s.fwd_count,
                                                                               s.adj_begin, s.adj_count)
            r["group_begin"], r["group_count"] = s.group_begin, s.group_count
            r["theta_offset"] = r["grad_offset"] = theta_off[i]
            r["basis"] = 0
        work = {c: sorted((i for i in range(m) if sess[i].cls == c), key=lambda i: -sess[i].cost)
                for c in _CLASSES}
        present = [c for c in _CLASSES if work[c]]
        # one packed upload: insts | work lists | counters | theta (8-byte aligned parts)
        parts = [insts.view(np.uint8)]
        offs = {}
        pos = insts.nbytes
        for c in present:
            w = np.asarray(work[c], dtype=np.int32)
            offs[c] = pos
            pad = (-w.nbytes) % 8
            parts.append(w.view(np.uint8))
            parts.append(np.zeros(pad, np.uint8))
            pos += w.nbytes + pad
        cnt_off = pos
        parts.append(np.zeros(8 * max(len(present), 1), np.uint8))
        pos += 8 * max(len(present), 1)
        th_off = pos
        th = np.concatenate([np.asarray(t, dtype=np.float64).reshape(-1) for _, t in items]) if theta_off[-1] else \
            np.zeros(1)
        parts.append(th.view(np.uint8))
        blob_h = torch.from_numpy(np.concatenate(parts)).pin_memory()
        n_out = m + int(theta_off[-1])
        stream.wait_stream(torch.cuda.current_stream(self.device))  # arena uploads
        with torch.cuda.stream(stream):
            blob = torch.empty(blob_h.numel(), dtype=torch.uint8, device=self.device)
            blob.copy_(blob_h, non_blocking=True)
            out = torch.zeros(max(n_out, 1), dtype=torch.float64, device=self.device)
            base = blob.data_ptr()
            P = ctypes.c_void_p
            grads_ptr = out.data_ptr() + 8 * m
            s = P(stream.cuda_stream)
            for k, c in enumerate(present):
                G, T, smem = self.cls_info[c]
                nat.call("tq_batch_run", self.dt, P(base), P(base + offs[c]), len(work[c]), 0, G, T, self.grid,
                         smem, None, self.ops.ptr(), self.groups.ptr(), self.terms.ptr(), P(base + th_off), None,
                         P(out.data_ptr()), P(grads_ptr), P(base + cnt_off + 4 * k), s)
            out_h = torch.empty(out.numel(), dtype=torch.float64, pin_memory=True)
            out_h.copy_(out, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return {"event": ev, "out": out_h, "keep": (blob, blob_h, out), "m": m, "theta_off": theta_off}

    @staticmethod
    def results(ticket) -> list[tuple[float, np.ndarray]]:
        """(energy, gradient) per item of a completed ticket."""
        o = ticket["out"].numpy()
        m, to = ticket["m"], ticket["theta_off"]
        return [(float(o[i]), o[m + to[i]:m + to[i + 1]].copy()) for i in range(m)]

    def release_retired(self) -> None:
        """Drop grown-out device buffers (call when no batch is in flight)."""
        self.retired.clear()
