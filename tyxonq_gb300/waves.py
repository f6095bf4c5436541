"""L2-resident waves for the large instances of a batch (host side of csrc/wave.cu).

Instances too large for one CTA's shared memory are grouped into waves whose
psi and lam fit together in L2 (``budget`` bytes).  A wave runs as a short
sequence of grid-wide launches over (instance, tile) work items:

  forward pass k of every wave instance  (kind 0, register stages; pass 0
                                          also writes |basis>)
  lam = H psi, energy partials          (kind 1)
  adjoint pass k of every wave instance  (kind 2, gradient partials)
  fixed-order reductions of the partials into energies and gradients.

All tables (passes, stages, ops, items, reduction rows) are built once; the
state pool and partial buffer are reused by every wave, so device memory is
one wave's footprint.  Circuit structures are encoded once and shared by all
instances with the same structure; angles are read from theta on the device.
"""
from __future__ import annotations

import ctypes
import warnings
from collections import defaultdict

import numpy as np
import torch

from . import _native as nat
from .program import STAGE_DTYPE, TILE_OP_DTYPE, PassPlan, encode_staged, plan_passes

WAVE_ITEM_DTYPE = np.dtype({
    "names": ["psi_off", "lam_off", "pass", "tile", "theta_off", "part_off", "n", "group_begin", "group_count",
              "basis_lo"],
    "formats": ["<i8", "<i8", "<i4", "<i4", "<i4", "<i4", "<i4", "<i4", "<i4", "<i4"],
    "offsets": [0, 8, 16, 20, 24, 28, 32, 36, 40, 44],
    "itemsize": 48,
})
ROP_JOB_DTYPE = np.dtype({"names": ["op_begin", "n_ops", "theta_off", "flags", "out_record"],
                          "formats": ["<i4", "<i4", "<i4", "<i4", "<i8"], "offsets": [0, 4, 8, 12, 16],
                          "itemsize": 24})


def rop_jobs(items: list, launches, passes: list, stages: np.ndarray) -> tuple[list, np.ndarray]:
    """Op-record jobs (tq_rop_job) for the forward and adjoint items: one per
    distinct (kind, pass, instance angles); returns the items with
    group_begin = the first record of their job and group_count = its op
    count, and the job table."""
    index: dict = {}
    jobs = []
    nrec = 0
    out = list(items)
    for L in launches:
        if L[0] != "run" or L[1] not in (0, 2):
            continue
        kind = L[1]
        for i in range(L[2], L[2] + L[3]):
            row = out[i]
            key = (kind, int(row[2]), int(row[4]))
            if key not in index:
                pa = passes[int(row[2])]
                sb, se = int(pa[2]), int(pa[3])
                op0 = int(stages[sb]["op_begin"]) if se > sb else 0
                nops = int(stages[se - 1]["op_end"]) - op0 if se > sb else 0
                index[key] = (nrec, nops)
                jobs.append((op0, nops, int(row[4]), 1 if kind == 2 else 0, nrec))
                nrec += nops
            out[i] = tuple(row[:7]) + index[key] + tuple(row[9:])
    tab = np.zeros(len(jobs), dtype=ROP_JOB_DTYPE)
    for k, j in enumerate(jobs):
        tab[k] = j
    if nrec >= 2 ** 31:
        raise NotImplementedError("too many op records for one wave plan")
    return out, tab


# passes of a wave keep at least this many contiguous low bits (the kernels'
# offset table holds 2^(t - WAVE_MIN_NLOW) entries)
WAVE_MIN_NLOW = 4
PASS_DTYPE = np.dtype({"names": ["t", "nlow", "op_begin", "op_end", "pos"],
                       "formats": ["<i4", "<i4", "<i4", "<i4", ("<i4", 16)], "itemsize": 80})


def _max_pass_ops(enc) -> int:
    """Largest op count of one pass of an EncodedStaged."""
    st = enc.stages_host
    best = 0
    for p in range(enc.n_passes):
        ps = enc.passes[p]
        if ps.op_end > ps.op_begin:
            best = max(best, int(st[ps.op_end - 1]["op_end"] - st[ps.op_begin]["op_begin"]))
    return best


def _dev(arr: np.ndarray, device) -> torch.Tensor:
    return torch.frombuffer(bytearray(arr.tobytes() or b"\0" * 16), dtype=torch.uint8).to(device)


MAX_FORK = 8  # side-by-side sub-launches of one wave launch


class WavePlan:
    def __init__(self, entries, dtype, device, t: int = 12, hbits: int = 12, budget: int = 48 << 20,
                 max_ops: int = 256, lanes: int = 1, adj_stage_bits: int = 4, jit: bool = False,
                 fork: bool = True):
        """entries: list of dicts with keys idx (instance index), n, gates,
        params, key (structure key), theta_off, grad_offset, basis,
        group_begin, group_count.  Waves are dealt round-robin to `lanes`
        independent launch sequences with disjoint pool and partial ranges,
        which may run on separate streams (each lane's wave fits `budget`)."""
        self.lanes = max(1, int(lanes))
        self.adj_rb = int(adj_stage_bits)
        self.dtype = dtype
        self.dt = 0 if dtype == torch.complex64 else 1
        self.t = t
        self.hbits = hbits
        self.max_ops = max_ops
        S = 8 if dtype == torch.complex64 else 16
        self.passes, self.stages, self.ops = [], [], []
        self.adj_max_ops = 1
        self.fwd_max_ops = 1
        self._np = self._ns = self._no = 0
        cache = {}
        for e in entries:
            if e["key"] not in cache:
                cache[e["key"]] = self._encode(e["n"], e["gates"], e["params"])
            e["enc"] = cache[e["key"]]
        self.n_structures = len(cache)
        # waves: largest first, packed up to the L2 budget
        order = sorted(entries, key=lambda e: -e["n"])
        waves, cur, used = [], [], 0
        for e in order:
            need = 2 * S << e["n"]
            if cur and used + need > budget:
                waves.append(cur)
                cur, used = [], 0
            cur.append(e)
            used += need
        if cur:
            waves.append(cur)
        self.waves = waves
        items, launches, rows = [], [], []
        norm_rows, norm_lane = [], []
        self.hpsi_alg_bytes = 0
        item_lane, row_lane, self.launch_lanes = [], [], []
        lane_pool = [0] * self.lanes
        lane_part = [0] * self.lanes
        for wi, wv in enumerate(waves):
            lane = wi % self.lanes
            n_items0, n_rows0, n_launch0 = len(items), len(rows), len(launches)
            off = 0
            for e in wv:
                e["psi_off"], e["lam_off"] = off, off + (1 << e["n"])
                off += 2 << e["n"]
            lane_pool[lane] = max(lane_pool[lane], off)
            part = 0
            # energy partial slots first, then gradient partials
            for e in wv:
                e["epart"] = part
                part += 1 << max(0, e["n"] - min(hbits, e["n"]))
            # forward phases
            nf = max(len(e["enc"]["fwd"]) for e in wv)
            for k in range(nf):
                b = len(items)
                for e in wv:
                    if k >= len(e["enc"]["fwd"]):
                        continue
                    pid = e["enc"]["fwd"][k]
                    for tile in range(1 << (e["n"] - self.t)):
                        items.append((e["psi_off"], e["lam_off"], pid, tile, e["theta_off"], 0, e["n"], 0, 0,
                                      e["basis"] if k == 0 else -1))
                launches.append(("run", 0, b, len(items) - b))
            b = len(items)
            for e in wv:
                hb = min(hbits, e["n"])
                self.hpsi_alg_bytes += (1 << (e["n"] - hb)) * (int(e.get("partner_tiles", 1)) + 1) * (S << hb)
                for tile in range(1 << (e["n"] - hb)):
                    items.append((e["psi_off"], e["lam_off"], 0, tile, e["theta_off"], e["epart"] + tile, e["n"],
                                  e["group_begin"], e["group_count"], -1))
            launches.append(("run", 1, b, len(items) - b))
            na = max(len(e["enc"]["adj"]) for e in wv)
            grad_rows = []
            for k in range(na):
                b = len(items)
                for e in wv:
                    if k >= len(e["enc"]["adj"]):
                        continue
                    pid, nops, pslots = e["enc"]["adj"][k]
                    ntile = 1 << (e["n"] - self.t)
                    base = part
                    for tile in range(ntile):
                        items.append((e["psi_off"], e["lam_off"], pid, tile, e["theta_off"], base + tile * nops,
                                      e["n"], 0, 0, -1))
                    part += ntile * nops
                    for kk, slot, coef in pslots:
                        grad_rows.append((base + kk, ntile, nops, coef, e["grad_offset"] + slot))
                launches.append(("run", 2, b, len(items) - b))
            lane_part[lane] = max(lane_part[lane], part)
            erow = [(e["epart"], 1 << (e["n"] - min(hbits, e["n"])), 1, 1.0, e["idx"]) for e in wv]
            rb = len(rows)
            rows += erow
            launches.append(("reduce_e", rb, len(erow)))
            # split gradient rows so that no launch writes one output twice
            seen = defaultdict(int)
            layers = defaultdict(list)
            for r in grad_rows:
                layers[seen[r[4]]].append(r)
                seen[r[4]] += 1
            for lay in sorted(layers):
                rb = len(rows)
                rows += layers[lay]
                launches.append(("reduce_g", rb, len(layers[lay])))
            # energies and gradients divided by <psi|psi> (norm partials of the H psi items)
            nb = len(norm_rows)
            norm_rows += [(e["epart"], 1 << (e["n"] - min(hbits, e["n"])), e["idx"], e["grad_offset"],
                           int(e.get("n_params", 0))) for e in wv]
            norm_lane += [lane] * len(wv)
            launches.append(("normalize", nb, len(wv)))
            item_lane += [lane] * (len(items) - n_items0)
            row_lane += [lane] * (len(rows) - n_rows0)
            self.launch_lanes += [lane] * (len(launches) - n_launch0)
        self.launches = launches
        self.n_items = len(items)
        # circuit-specialised kernels: one per distinct pass body; the items of each
        # forward / adjoint launch are grouped by body, one sub-launch per group
        self.jit_sub: dict = {}
        self.device = torch.device(device)
        self._aux: dict = {}  # lane -> side streams for the sub-launches of one launch
        self.fork = bool(fork)
        # op records of the forward and adjoint items, compiled once per evaluation
        # (compile_rops) for the specialised kernels instead of once per tile
        st_all = np.concatenate(self.stages) if self.stages else np.zeros(0, STAGE_DTYPE)
        items, jobs = rop_jobs(items, launches, self.passes, st_all)
        self.rop_jobs_dev = _dev(jobs if len(jobs) else np.zeros(1, ROP_JOB_DTYPE), device)
        self.n_rop_jobs = len(jobs)
        n_rec = int(jobs["out_record"][-1] + jobs["n_ops"][-1]) if len(jobs) else 0
        self.rops_buf = torch.empty(max(int(nat.load().tq_jit_rops_bytes(self.dt, n_rec)), 16), dtype=torch.uint8,
                                    device=device)
        if jit and items:
            try:
                self._specialise(items, device)
            except (nat.TqError, OSError) as e:
                # a runtime compilation that fails leaves every item on the library's
                # interpreting kernels: the same results, slower
                warnings.warn(f"specialised wave kernels unavailable, interpreting kernels used: {e}")
                self.jit_sub, self.jit_kernels, self.jit_bodies = {}, {}, 0
        pool_base = np.concatenate([[0], np.cumsum(lane_pool)]).astype(np.int64)
        part_base = np.concatenate([[0], np.cumsum(lane_part)]).astype(np.int64)
        pool_need, part_need = int(pool_base[-1]), int(part_base[-1])
        it = np.zeros(len(items), dtype=WAVE_ITEM_DTYPE)
        if items:
            cols = list(zip(*items))
            for name, col in zip(WAVE_ITEM_DTYPE.names, cols):
                it[name] = col
            il = np.asarray(item_lane)
            it["psi_off"] += pool_base[il]
            it["lam_off"] += pool_base[il]
            it["part_off"] += part_base[il].astype(np.int32)
        rows = [(r[0] + int(part_base[l]),) + tuple(r[1:]) for r, l in zip(rows, row_lane)]
        norm_rows = [(r[0] + int(part_base[l]),) + tuple(r[1:]) for r, l in zip(norm_rows, norm_lane)]
        self.n_first = torch.tensor([x[0] for x in norm_rows] or [0], dtype=torch.int32, device=device)
        self.n_count = torch.tensor([x[1] for x in norm_rows] or [0], dtype=torch.int32, device=device)
        self.n_inst = torch.tensor([x[2] for x in norm_rows] or [0], dtype=torch.int32, device=device)
        self.n_goff = torch.tensor([x[3] for x in norm_rows] or [0], dtype=torch.int32, device=device)
        self.n_gcount = torch.tensor([x[4] for x in norm_rows] or [0], dtype=torch.int32, device=device)
        self.items_dev = _dev(it, device)
        r = np.array(rows, dtype=object) if rows else np.zeros((0, 5))
        self.r_first = torch.tensor([x[0] for x in rows] or [0], dtype=torch.int32, device=device)
        self.r_count = torch.tensor([x[1] for x in rows] or [0], dtype=torch.int32, device=device)
        self.r_stride = torch.tensor([x[2] for x in rows] or [0], dtype=torch.int32, device=device)
        self.r_scale = torch.tensor([x[3] for x in rows] or [0.0], dtype=torch.float64, device=device)
        self.r_out = torch.tensor([x[4] for x in rows] or [0], dtype=torch.int32, device=device)
        del r
        pa = np.zeros(len(self.passes), dtype=PASS_DTYPE)
        for k, (tt, nl, b0, e0, pos) in enumerate(self.passes):
            pa[k] = (tt, nl, b0, e0, pos)
        self.passes_dev = _dev(pa, device)
        self.stages_dev = _dev(np.concatenate(self.stages) if self.stages else np.zeros(1, STAGE_DTYPE), device)
        self.ops_dev = _dev(np.concatenate(self.ops) if self.ops else np.zeros(1, TILE_OP_DTYPE), device)
        self.pool = torch.empty(max(pool_need, 2), dtype=dtype, device=device)
        self.partials = torch.zeros(max(part_need, 1), dtype=torch.float64, device=device)
        self.norm_partials = torch.zeros(max(part_need, 1), dtype=torch.float64, device=device)
        self.pool_bytes = self.pool.numel() * S

    def _specialise(self, items: list, device) -> None:
        from . import jit as J

        st = np.concatenate(self.stages) if self.stages else np.zeros(0, STAGE_DTYPE)
        ops = np.concatenate(self.ops) if self.ops else np.zeros(0, TILE_OP_DTYPE)
        double = self.dt == 1
        used = {0: {}, 2: {}}
        for L in self.launches:
            if L[0] == "run" and L[1] in (0, 2) and L[3] > 0:
                for row in items[L[2]:L[2] + L[3]]:
                    used[L[1]][row[2]] = self.passes[row[2]]
        kern = {0: J.wave_kernels(0, self.t, st, ops, used[0], double, self.fwd_max_ops, device)}
        if self.adj_rb == 4:
            kern[2] = J.wave_kernels(2, self.t, st, ops, used[2], double, self.adj_max_ops, device)
        else:
            kern[2] = {}
        self.jit_kernels = kern
        for li, L in enumerate(self.launches):
            if L[0] != "run" or L[1] not in (0, 2) or L[3] == 0:
                continue
            kind, b, c = L[1], L[2], L[3]
            block = items[b:b + c]
            key = [kern[kind].get(row[2], 0) for row in block]
            order = sorted(range(c), key=lambda i: key[i])
            items[b:b + c] = [block[i] for i in order]
            subs, i = [], 0
            while i < c:
                j = i
                while j < c and key[order[j]] == key[order[i]]:
                    j += 1
                subs.append((b + i, j - i, key[order[i]]))
                i = j
            self.jit_sub[li] = subs
        self.jit_bodies = len({h for d in kern.values() for h in d.values()})

    # ------------------------------------------------------------ encoding
    def _add_staged(self, enc) -> list[int]:
        """Append an EncodedStaged's passes/stages/ops to the global tables; return pass ids."""
        st = enc.stages_host.copy()
        st["op_begin"] += self._no
        st["op_end"] += self._no
        ids = []
        for p in range(enc.n_passes):
            ps = enc.passes[p]
            self.passes.append((ps.t, ps.nlow, ps.op_begin + self._ns, ps.op_end + self._ns, list(ps.pos)))
            ids.append(len(self.passes) - 1)
        self.stages.append(st)
        self.ops.append(enc.ops_host)
        self._ns += len(st)
        self._no += len(enc.ops_host)
        return ids

    def _encode(self, n, gates, params) -> dict:
        t = self.t
        segs = plan_passes(gates, n, t, max_ops=self.max_ops)
        fwd = []
        for s in segs:
            if s.kind != "tiles":
                raise NotImplementedError("wave path needs tileable gates")
            enc = encode_staged(n, s.passes, gates, params=params)
            fwd += self._add_staged(enc)
            self.fwd_max_ops = max(self.fwd_max_ops, _max_pass_ops(enc))
        if not fwd:  # no gates: one empty pass writes |basis>
            qs = list(range(n - 1, n - 1 - t, -1))
            fwd += self._add_staged(encode_staged(n, [PassPlan(qs, [], 5)], gates))
        rg = list(reversed(gates))
        G = len(gates)
        rparams = {G - 1 - gi: v for gi, v in params.items()}
        slots = {ri: rparams[ri][0] for ri in rparams}
        adj = []
        for s in plan_passes(rg, n, t, max_ops=self.max_ops):
            if s.kind != "tiles":
                raise NotImplementedError("wave path needs tileable gates")
            for pp in s.passes:
                enc = encode_staged(n, [pp], rg, params=rparams, slots=slots, rb=self.adj_rb)
                pid = self._add_staged(enc)[0]
                ops = enc.ops_host
                pslots = [(k, int(ops[k]["slot"]), float(ops[k]["gcoef"])) for k in range(len(ops))
                          if ops[k]["slot"] >= 0]
                adj.append((pid, len(ops), pslots))
                self.adj_max_ops = max(self.adj_max_ops, len(ops))
        for pid in fwd + [a[0] for a in adj]:
            if self.passes[pid][1] < WAVE_MIN_NLOW:
                raise NotImplementedError(f"wave pass keeps {self.passes[pid][1]} contiguous low bits "
                                          f"(at least {WAVE_MIN_NLOW} needed)")
        return {"fwd": fwd, "adj": adj}

    # ------------------------------------------------------------ execution
    def compile_rops(self, theta, stream) -> None:
        """Build the op records of every forward and adjoint (pass, instance) pair
        from theta (one launch; the specialised wave kernels copy them per item)."""
        if self.n_rop_jobs:
            P = ctypes.c_void_p
            nat.call("tq_wave_rops", self.dt, P(self.rop_jobs_dev.data_ptr()), self.n_rop_jobs,
                     P(self.ops_dev.data_ptr()), P(theta.data_ptr()), P(self.rops_buf.data_ptr()), stream)

    def _fork(self, lane: int, stream, width: int):
        """(the launching stream, [it and width - 1 side streams of this lane that wait on it])."""
        aux = self._aux.setdefault(lane, [])
        while len(aux) < width - 1:
            aux.append(torch.cuda.Stream(self.device))
        ptr = stream.value if isinstance(stream, ctypes.c_void_p) else stream
        base = (torch.cuda.ExternalStream(int(ptr), device=self.device) if ptr
                else torch.cuda.default_stream(self.device))  # a null handle is the default stream
        ev = torch.cuda.Event()
        ev.record(base)
        for a in aux[:width - 1]:
            a.wait_event(ev)
        return base, [base] + aux[:width - 1]

    @staticmethod
    def _join(base, branch) -> None:
        for a in branch[1:]:
            ev = torch.cuda.Event()
            ev.record(a)
            base.wait_event(ev)

    def launch(self, groups_dev, terms_dev, theta, energies, grads, stream, lane_streams=None,
               kinds=(0, 1, 2), on_launch=None) -> None:
        """Enqueue every launch; lane l's on lane_streams[l] when given, else all on `stream`.
        kinds: the phases to run (0 forward, 1 H psi + energy reduction, 2 adjoint +
        gradient reductions).  on_launch(when, kind, n_items, jit): called before
        ("start") and after ("end") each kernel launch (profiling on one stream)."""
        P = ctypes.c_void_p
        isz = WAVE_ITEM_DTYPE.itemsize
        cb = on_launch or (lambda *a: None)
        for li, (L, lane) in enumerate(zip(self.launches, self.launch_lanes)):
            if lane_streams is not None:
                stream = lane_streams[lane]
            phase = L[1] if L[0] == "run" else (1 if L[0] in ("reduce_e", "normalize") else 2)
            if phase not in kinds:
                continue
            if L[0] == "run" and li in self.jit_sub:
                kind = L[1]
                subs = self.jit_sub[li]
                # the sub-launches of one launch touch disjoint items: without a profiler
                # they run side by side (fork on side streams, join before the next launch),
                # so a launch split by kernel still fills the GPU like one launch
                fork = self.fork and on_launch is None and len(subs) > 1
                if fork:
                    base, branch = self._fork(lane, stream, min(len(subs), MAX_FORK))
                for si, (b0, c0, k) in enumerate(subs):
                    if fork:
                        stream = ctypes.c_void_p(branch[si % len(branch)].cuda_stream)
                    cb("start", kind, c0, bool(k))
                    if k:
                        nat.call("tq_jit_wave_run", P(k), kind, self.dt, P(self.items_dev.data_ptr() + isz * b0), c0,
                                 self.t, P(self.passes_dev.data_ptr()), P(self.stages_dev.data_ptr()),
                                 P(self.ops_dev.data_ptr()), P(theta.data_ptr()), P(self.rops_buf.data_ptr()),
                                 P(self.pool.data_ptr()),
                                 P(self.partials.data_ptr()), self.fwd_max_ops if kind == 0 else self.adj_max_ops,
                                 stream)
                    else:
                        nat.call("tq_wave_run", kind, self.dt, P(self.items_dev.data_ptr() + isz * b0), c0, self.t,
                                 self.hbits, self.adj_rb if kind == 2 else 4, P(self.passes_dev.data_ptr()),
                                 P(self.stages_dev.data_ptr()), P(self.ops_dev.data_ptr()), None, None,
                                 P(theta.data_ptr()), P(self.pool.data_ptr()), P(self.partials.data_ptr()), None,
                                 self.fwd_max_ops if kind == 0 else self.adj_max_ops, stream)
                    cb("end", kind, c0, bool(k))
                if fork:
                    self._join(base, branch)
                    stream = ctypes.c_void_p(base.cuda_stream)
            elif L[0] == "run":
                _, kind, b, c = L
                if c == 0:
                    continue
                cb("start", kind, c, False)
                nat.call("tq_wave_run", kind, self.dt, P(self.items_dev.data_ptr() + isz * b), c, self.t,
                         self.hbits, self.adj_rb if kind == 2 else 4, P(self.passes_dev.data_ptr()),
                         P(self.stages_dev.data_ptr()),
                         P(self.ops_dev.data_ptr()), P(groups_dev.data_ptr()), P(terms_dev.data_ptr()),
                         P(theta.data_ptr()), P(self.pool.data_ptr()), P(self.partials.data_ptr()),
                         P(self.norm_partials.data_ptr()) if kind == 1 else None,
                         self.fwd_max_ops if kind == 0 else self.adj_max_ops, stream)
                cb("end", kind, c, False)
            elif L[0] == "normalize":
                _, b, c = L
                nat.call("tq_wave_normalize", P(self.norm_partials.data_ptr()), P(self.n_first.data_ptr() + 4 * b),
                         P(self.n_count.data_ptr() + 4 * b), P(self.n_inst.data_ptr() + 4 * b),
                         P(self.n_goff.data_ptr() + 4 * b), P(self.n_gcount.data_ptr() + 4 * b), c,
                         P(energies.data_ptr()), P(grads.data_ptr()), stream)
            else:
                kind, b, c = L
                out = energies if kind == "reduce_e" else grads
                nat.call("tq_wave_reduce", P(self.partials.data_ptr()), P(self.r_first.data_ptr() + 4 * b),
                         P(self.r_count.data_ptr() + 4 * b), P(self.r_stride.data_ptr() + 4 * b),
                         P(self.r_scale.data_ptr() + 8 * b), P(self.r_out.data_ptr() + 4 * b), c,
                         P(out.data_ptr()), 0 if kind == "reduce_e" else 1, stream)
