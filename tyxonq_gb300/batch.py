"""Batched VQE energy + adjoint gradient for thousands of uneven instances.

``BatchedVQE`` compiles a set of parametrised circuits (any qubit count,
depth and Pauli-sum Hamiltonian) once into device tables and evaluates all
energies and gradients with a few persistent launches of
``tq_batch_run`` (csrc/batch.cu), one per size class:

  class        qubits   thread groups / CTA   where psi, H psi live
  res8         <= 10    8 x 128 threads       shared memory
  res4         11       4 x 256               shared memory
  res2         12       2 x 512               shared memory
  res1         13       1 x 1024              shared memory
  streamed     >= 14    1 x 1024              HBM pool, tile passes

(complex64; complex128 shifts every boundary down by one qubit).  Angles live
on the device (ops read theta[pidx]), so a new parameter vector costs one
H2D copy; the whole step (memsets + launches) can be captured in a CUDA graph
(``capture``) and replayed.  The class boundaries, wave tile width, L2 budget,
lanes and stage widths are the schedule the autotuner
(tyxonq_gb300.autotune.tune_batched) searches; ``Schedule.default`` is the
tuned one for the current GPU when it was saved.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .hamiltonian import GROUP_DTYPE, TERM_DTYPE, PauliSum, order_groups_for_tiles, sort_terms_by_class
from .ir import Gate, _rot_gate
from .program import TILE_OP_DTYPE, PassPlan, TilePass, encode_passes, plan_passes

INST_DTYPE = np.dtype({
    "names": ["n", "streamed", "fwd_begin", "fwd_count", "adj_begin", "adj_count", "group_begin", "group_count",
              "theta_offset", "grad_offset", "scratch_offset", "basis"],
    "formats": ["<i4"] * 10 + ["<i8", "<i8"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 48],
    "itemsize": 56,
})
PASS_DTYPE = np.dtype({"names": ["t", "nlow", "op_begin", "op_end", "pos"],
                       "formats": ["<i4", "<i4", "<i4", "<i4", ("<i4", 16)], "itemsize": 80})


@dataclass
class Schedule:
    """Launch schedule: size-class boundaries and tile widths."""

    res8_max: int = 10
    res4_max: int = 11
    res2_max: int = 12
    res1_max: int = 13
    t_fwd: int = 13
    t_adj: int = 12
    max_pass_ops: int = 512
    large: str = "waves"  # instances above res1_max: "waves" (L2-resident grid-wide phases) or "cta"
    wave_t: int = 12
    wave_hbits: int = 12
    wave_budget: int = 64 << 20  # per lane
    wave_lanes: int = 2  # waves in flight at once, each lane on its own stream
    wave_max_ops: int = 256
    wave_adj_stage_bits: int = 4  # register bits per adjoint stage (3: 8 amplitudes of psi and of lam per thread)
    wave_jit: int = 1  # circuit-specialised wave kernels (runtime-compiled per distinct pass body)
    wave_fork: int = 0  # the per-kernel sub-launches of one wave launch run side by side (1) or in order (0)

    @classmethod
    def builtin(cls, dtype) -> "Schedule":
        """The untuned schedule (shared-memory capacity rules)."""
        if dtype == torch.complex128:
            return cls(res8_max=9, res4_max=10, res2_max=11, res1_max=12, t_fwd=12, t_adj=11)
        return cls()

    @classmethod
    def default(cls, dtype, device=None) -> "Schedule":
        """The autotuned schedule for this GPU when one was saved
        (tyxonq_gb300.autotune), else the builtin one."""
        from dataclasses import replace

        from .autotune import load_schedule

        base = cls.builtin(dtype)
        tuned = load_schedule(dtype, device)
        return replace(base, **tuned) if tuned else base

    def class_of(self, n: int) -> tuple[str, int, int]:
        """(class name, groups per CTA, threads per CTA)."""
        if n <= self.res8_max:
            return "res8", 8, 1024
        if n <= self.res4_max:
            return "res4", 4, 1024
        if n <= self.res2_max:
            return "res2", 2, 1024
        if n <= self.res1_max:
            return "res1", 1, 1024
        return "streamed", 1, 1024


def _jit_enabled() -> bool:
    """Circuit-specialised kernels are on unless TYXONQ_GB300_JIT=0."""
    import os

    return os.environ.get("TYXONQ_GB300_JIT", "1") != "0"


def structure_gates(structure) -> tuple[list[Gate], dict]:
    """[(name, qubits, param index or None)] -> gates and {gate index: (pidx, 1.0)}."""
    gates, params = [], {}
    for i, (name, qs, p) in enumerate(structure):
        qs = tuple(int(q) for q in qs)
        if p is None:
            gates.append(Gate(name, qs) if name in ("cx", "cz", "swap") else _fixed(name, qs))
        else:
            gates.append(_rot_gate(name, qs, 0.0))
            params[i] = (int(p), 1.0)
    return gates, params


def _fixed(name, qs):
    from . import gates as G

    m = {"h": G.gate_h, "x": G.gate_x, "y": G.gate_y, "z": G.gate_z}[name]()
    return Gate("u1", qs, m)


@dataclass
class _Class:
    name: str
    groups: int
    threads: int
    work: list = field(default_factory=list)
    max_n: int = 0
    smem: int = 0
    work_dev: torch.Tensor | None = None


class BatchedVQE:
    """Energies and adjoint gradients of many parametrised circuits at once.

    instances: objects with ``n``, ``n_params``, ``structure()`` (list of
    (gate name, qubits, param index or None)) and ``H`` (PauliSum); optional
    ``basis`` (initial basis index).
    """

    def __init__(self, instances: Sequence, dtype=torch.complex64, device="cuda", schedule: Schedule | None = None,
                 grid: int | None = None):
        self.dtype = dtype
        self.dt = K._DT[dtype]
        self.device = torch.device(device)
        self.sched = schedule or Schedule.default(dtype)
        self.count = len(instances)
        sm = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.grid = grid or sm
        ops_all, passes_all, groups_all, terms_all = [], [], [], []
        pass_is_fwd: list[bool] = []
        self._pass_is_fwd = pass_is_fwd
        insts = np.zeros(self.count, dtype=INST_DTYPE)
        theta_off = 0
        pool_off = 0
        self.classes: dict[str, _Class] = {}
        self.n_params = []
        S = 8 if dtype == torch.complex64 else 16
        cache: dict = {}
        self._nops = 0
        wave_entries = []
        n_groups_total = n_terms_total = 0
        gate_cache: dict = {}
        for i, inst in enumerate(instances):
            n = int(inst.n)
            cname, G, T = self.sched.class_of(n)
            skey = tuple(inst.structure())
            if skey not in gate_cache:
                gate_cache[skey] = structure_gates(inst.structure())
            gates, params = gate_cache[skey]
            H: PauliSum = inst.H
            g, t = H.pack()
            if cname == "streamed" and self.sched.large == "waves":
                t = sort_terms_by_class(g, t, self.sched.wave_hbits)
                # groups whose flips share the bits above the H psi tile read the same
                # partner tile: neighbours in the loop, so it is staged once; inside such a
                # run, one-term groups of one sign class run back to back
                g = order_groups_for_tiles(g, t, self.sched.wave_hbits)
                wave_entries.append({"idx": i, "n": n, "gates": gates, "params": params, "key": (n, skey),
                                     "theta_offset": theta_off, "theta_off": theta_off, "grad_offset": theta_off,
                                     "basis": int(getattr(inst, "basis", 0)), "group_begin": n_groups_total,
                                     "group_count": len(g), "n_params": int(inst.n_params),
                                     "partner_tiles": int(len(np.unique(g["flip"] >> np.uint64(
                                         min(self.sched.wave_hbits, n))))) if len(g) else 0})
                insts[i]["n"] = n
                insts[i]["streamed"] = 2
                theta_off += int(inst.n_params)
                self.n_params.append(int(inst.n_params))
                g2 = g.copy()
                g2["first_term"] += n_terms_total
                groups_all.append(g2)
                terms_all.append(t)
                n_groups_total += len(g)
                n_terms_total += len(t)
                continue
            cl = self.classes.setdefault(cname, _Class(cname, G, T))
            streamed = cname == "streamed"
            rec = insts[i]
            rec["n"] = n
            rec["streamed"] = int(streamed)
            rec["basis"] = int(getattr(inst, "basis", 0))
            rec["theta_offset"] = theta_off
            rec["grad_offset"] = theta_off
            theta_off += int(inst.n_params)
            self.n_params.append(int(inst.n_params))
            # instances with the same circuit structure share one encoded op block
            # (angles are read from theta on the device, so ops do not depend on them)
            key = (n, streamed, tuple(inst.structure()))
            ent = cache.get(key)
            if ent is None:
                ent = self._encode_structure(n, gates, params, streamed, ops_all, passes_all, pass_is_fwd)
                cache[key] = ent
            rec["fwd_begin"], rec["fwd_count"], rec["adj_begin"], rec["adj_count"] = ent
            if streamed:
                rec["scratch_offset"] = pool_off
                pool_off += 2 << n
            rec["group_begin"] = n_groups_total
            rec["group_count"] = len(g)
            g2 = g.copy()
            g2["first_term"] += n_terms_total
            groups_all.append(g2)
            terms_all.append(t)
            n_groups_total += len(g)
            n_terms_total += len(t)
            cost = (1 << n) * (rec["fwd_count"] + rec["adj_count"] + 4 * H.n_terms)
            cl.work.append((cost, i))
            cl.max_n = max(cl.max_n, n)
        self.n_structures = len(cache)
        self.insts_host = insts
        self.ops_host = np.concatenate(ops_all) if ops_all else np.zeros(1, TILE_OP_DTYPE)
        self.n_theta = theta_off
        dev = self.device
        self.insts_dev = _to_dev(insts, dev)
        self.ops_dev = _to_dev(self.ops_host, dev)
        if passes_all:
            pa = np.zeros(len(passes_all), dtype=PASS_DTYPE)
            for k, (t, nl, b, e, pos) in enumerate(passes_all):
                pa[k] = (t, nl, b, e, pos)
            self.passes_dev = _to_dev(pa, dev)
        else:
            self.passes_dev = None
        self.groups_dev = _to_dev(np.concatenate(groups_all), dev)
        self.terms_dev = _to_dev(np.concatenate(terms_all), dev)
        self.pool = torch.empty(max(pool_off, 2), dtype=dtype, device=dev) if pool_off else None
        self.theta = torch.zeros(max(theta_off, 1), dtype=torch.float64, device=dev)
        self.grads = torch.zeros_like(self.theta)
        self.energies = torch.zeros(self.count, dtype=torch.float64, device=dev)
        self.counters = torch.zeros(max(len(self.classes), 1), dtype=torch.int32, device=dev)
        self.waves = None
        if wave_entries:
            from .waves import WavePlan

            sc = self.sched
            self.waves = WavePlan(wave_entries, dtype, dev, t=sc.wave_t, hbits=sc.wave_hbits, budget=sc.wave_budget,
                                  lanes=sc.wave_lanes, adj_stage_bits=sc.wave_adj_stage_bits,
                                  max_ops=sc.wave_max_ops, jit=bool(sc.wave_jit) and _jit_enabled(),
                                  fork=bool(sc.wave_fork))
            self.n_structures += self.waves.n_structures
        lib = nat.load()
        order = ["streamed", "res1", "res2", "res4", "res8"]
        self.launch_order = [self.classes[c] for c in order if c in self.classes]
        for cl in self.launch_order:
            cl.work.sort(reverse=True)
            cl.work_dev = torch.tensor([i for _, i in cl.work], dtype=torch.int32, device=dev)
            if cl.name == "streamed":
                # exact need: max over passes of tiles + offset table + op accumulators,
                # and at least the H psi tiles of the adjoint width (kernel layout after 256 B)
                need = 256 + 2 * S * (1 << self.sched.t_adj)
                for k, (t, nl, b, e, _) in enumerate(passes_all):
                    fwd_like = 256 + S * (1 << t) + 8 * (1 << (t - nl))
                    adj_like = 256 + 2 * S * (1 << t) + 8 * (1 << (t - nl)) + 8 * (e - b)
                    need = max(need, fwd_like if self._pass_is_fwd[k] else adj_like)
                cl.smem = int((need + 255) & ~255)
                if cl.smem > 227 * 1024:
                    raise ValueError(f"streamed schedule needs {cl.smem} B of shared memory")
            else:
                cl.smem = int(lib.tq_batch_smem_bytes(self.dt, cl.max_n, cl.groups, 0))
        self.graph = None

    def _add_ops(self, ops_all: list, arr: np.ndarray) -> int:
        base = self._nops
        ops_all.append(arr)
        self._nops += len(arr)
        return base

    def _encode_structure(self, n, gates, params, streamed, ops_all, passes_all, pass_is_fwd) -> tuple:
        """Encode one circuit structure; returns (fwd_begin, fwd_count, adj_begin, adj_count):
        op ranges for resident instances, pass ranges for streamed ones.
        The adjoint list is the reversed gate list; its slots are parameter indices."""
        rgates = list(reversed(gates))
        Gn = len(gates)
        rparams = {Gn - 1 - gi: v for gi, v in params.items()}
        slots = {ri: rparams[ri][0] for ri in rparams}
        if not streamed:
            f_ops, a_ops = encode_resident(n, gates, params)
            fb = self._add_ops(ops_all, f_ops)
            ab = self._add_ops(ops_all, a_ops)
            return fb, len(f_ops), ab, len(a_ops)
        out = []
        for which, gl, pr, sl in (("fwd", gates, params, None), ("adj", rgates, rparams, slots)):
            t = self.sched.t_fwd if which == "fwd" else self.sched.t_adj
            segs = plan_passes(gl, n, t, max_ops=self.sched.max_pass_ops)
            begin = len(passes_all)
            for s in segs:
                if s.kind != "tiles":
                    raise NotImplementedError("batched instances need tileable gates")
                enc, _ = encode_passes(n, s.passes, gl, fuse=(which == "fwd"), slots=sl, params=pr)
                base = self._add_ops(ops_all, enc.ops_host)
                for p in range(enc.n_passes):
                    ps = enc.passes[p]
                    passes_all.append((ps.t, ps.nlow, ps.op_begin + base, ps.op_end + base, list(ps.pos)))
                    pass_is_fwd.append(which == "fwd")
            out += [begin, len(passes_all) - begin]
        return tuple(out)

    # ------------------------------------------------------------ execution
    def set_theta(self, theta) -> None:
        """Copy a flat parameter vector (host array or device tensor) in."""
        if isinstance(theta, torch.Tensor):
            self.theta.copy_(theta.reshape(-1).to(self.theta.dtype), non_blocking=True)
        else:
            self.theta.copy_(torch.from_numpy(np.ascontiguousarray(theta, dtype=np.float64)).reshape(-1),
                             non_blocking=True)

    def launch(self) -> None:
        """Enqueue one evaluation (memsets + persistent launches) on the current stream."""
        self.grads.zero_()
        self.counters.zero_()
        main = torch.cuda.current_stream(self.device)
        P = ctypes.c_void_p
        # persistent size-class kernels run on a side stream, concurrently with the waves
        if self.waves is not None and self.launch_order:
            if getattr(self, "_side", None) is None:
                self._side = torch.cuda.Stream(self.device)
            side = self._side
            side.wait_stream(main)
        else:
            side = main
        s = ctypes.c_void_p(side.cuda_stream)
        for k, cl in enumerate(self.launch_order):
            nat.call("tq_batch_run", self.dt, P(self.insts_dev.data_ptr()), P(cl.work_dev.data_ptr()),
                     int(cl.work_dev.numel()), int(cl.name == "streamed"), cl.groups, cl.threads, self.grid,
                     cl.smem, P(self.passes_dev.data_ptr()) if self.passes_dev is not None else None,
                     P(self.ops_dev.data_ptr()), P(self.groups_dev.data_ptr()), P(self.terms_dev.data_ptr()),
                     P(self.theta.data_ptr()), P(self.pool.data_ptr()) if self.pool is not None else None,
                     P(self.energies.data_ptr()), P(self.grads.data_ptr()),
                     P(self.counters.data_ptr() + 4 * k), s)
        if self.waves is not None:
            self.waves.compile_rops(self.theta, ctypes.c_void_p(main.cuda_stream))
            lanes = [main]
            if self.waves.lanes > 1:
                if getattr(self, "_lane_streams", None) is None:
                    self._lane_streams = [torch.cuda.Stream(self.device) for _ in range(self.waves.lanes - 1)]
                for ls in self._lane_streams:
                    ls.wait_stream(main)
                lanes += self._lane_streams
            self.waves.launch(self.groups_dev, self.terms_dev, self.theta, self.energies, self.grads,
                              ctypes.c_void_p(main.cuda_stream), [ctypes.c_void_p(x.cuda_stream) for x in lanes])
            for ls in lanes[1:]:
                main.wait_stream(ls)
        if side is not main:
            main.wait_stream(side)

    def kernel_launches(self) -> int:
        """Kernel launches of one evaluation (persistent class kernels, wave passes,
        wave reductions)."""
        n = len(self.launch_order)
        if self.waves is not None:
            for li, L in enumerate(self.waves.launches):
                if li in self.waves.jit_sub:
                    n += len(self.waves.jit_sub[li])
                elif L[0] != "run" or L[3] > 0:
                    n += 1
        return n

    def profile_waves(self) -> dict:
        """One evaluation of the wave launches alone, serialised on the current
        stream with CUDA events around every kernel: per phase (forward, hpsi,
        adjoint) the launches, items, total device ms and the algorithmic bytes
        moved (forward 2 * 2^t * S per item, adjoint 4 * 2^t * S -- psi and lam
        tiles read and written once -- and H psi (1 + partner tiles) * 2^hb * S
        read plus 2^hb * S written per item)."""
        if self.waves is None:
            return {}
        main = torch.cuda.current_stream(self.device)
        marks = []

        def cb(when, kind, items, jit):
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(main)
            marks.append((when, kind, items, jit, ev))

        self.grads.zero_()
        self.launch_waves_only(main, cb)
        torch.cuda.synchronize(self.device)
        out: dict = {}
        names = {0: "forward", 1: "hpsi", 2: "adjoint"}
        S = 8 if self.dtype == torch.complex64 else 16
        for (w0, kind, items, jit, a), (w1, _, _, _, b) in zip(marks[0::2], marks[1::2]):
            d = out.setdefault(names[kind], {"launches": 0, "items": 0, "ms": 0.0, "specialised_launches": 0})
            d["launches"] += 1
            d["items"] += items
            d["ms"] += a.elapsed_time(b)
            d["specialised_launches"] += int(jit)
        t = self.waves.t
        if "forward" in out:
            out["forward"]["alg_bytes"] = out["forward"]["items"] * 2 * (S << t)
        if "adjoint" in out:
            out["adjoint"]["alg_bytes"] = out["adjoint"]["items"] * 4 * (S << t)
        if "hpsi" in out:
            out["hpsi"]["alg_bytes"] = int(self.waves.hpsi_alg_bytes)
        return out

    def launch_waves_only(self, stream, on_launch=None) -> None:
        self.waves.compile_rops(self.theta, ctypes.c_void_p(stream.cuda_stream))
        self.waves.launch(self.groups_dev, self.terms_dev, self.theta, self.energies, self.grads,
                          ctypes.c_void_p(stream.cuda_stream), None, on_launch=on_launch)

    def capture(self) -> None:
        """Capture launch() into a CUDA graph (replayed by run())."""
        self.launch()  # warm-up (sets smem attributes outside capture)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g

    def run(self, theta=None) -> tuple[torch.Tensor, torch.Tensor]:
        """Evaluate all instances; returns (energies, flat gradients) on the device."""
        if theta is not None:
            self.set_theta(theta)
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self.energies, self.grads

    def split_grads(self, grads: np.ndarray) -> list[np.ndarray]:
        out, o = [], 0
        for p in self.n_params:
            out.append(grads[o:o + p])
            o += p
        return out


def encode_resident(n: int, gates: list, params: dict) -> tuple[np.ndarray, np.ndarray]:
    """Op records of a shared-memory-resident instance: the forward list (runs of
    single-qubit ops fused) and the adjoint list (reversed gates, slots =
    parameter indices), bit positions global (the whole state is one tile)."""
    rgates = list(reversed(gates))
    Gn = len(gates)
    rparams = {Gn - 1 - gi: v for gi, v in params.items()}
    slots = {ri: rparams[ri][0] for ri in rparams}
    allq = list(range(n - 1, -1, -1))  # bit 0 first: local bit = global bit
    enc_f, _ = encode_passes(n, [PassPlan(allq, list(range(Gn)), n)], gates, fuse=True, params=params)
    enc_a, _ = encode_passes(n, [PassPlan(allq, list(range(Gn)), n)], rgates, fuse=False, slots=slots,
                             params=rparams)
    return enc_f.ops_host, enc_a.ops_host


def _to_dev(arr: np.ndarray, device) -> torch.Tensor:
    raw = arr.tobytes() or b"\0" * 16
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)


# ---------------------------------------------------------------- plain engine comparison
def _plain_gates(inst):
    theta = np.asarray(inst.theta, dtype=np.float64)
    gates, params = [], []
    for name, qs, p in inst.structure():
        qs = tuple(int(q) for q in qs)
        if p is None:
            gates.append(Gate(name, qs) if name in ("cx", "cz", "swap") else _fixed(name, qs))
            params.append(None)
        else:
            gates.append(_rot_gate(name, qs, float(theta[p])))
            params.append(int(p))
    return gates, params


class PlainEngine:
    """The plain single-circuit GPU engine on one instance: one kernel launch per
    gate forward, H psi, <psi|H psi>, then per gate in reverse one generator
    reduction (tq_sv_generator_im) and two inverse-gate launches.  Buffers are
    allocated once; ``capture`` records the whole evaluation in a CUDA graph so
    that replays are bound by the GPU, not by the host loop that issues the
    launches."""

    def __init__(self, inst, dtype=torch.complex64, device="cuda"):
        from .program import _generator

        self.inst = inst
        self.n = n = int(inst.n)
        self.dtype = dtype
        self.device = torch.device(device)
        self.gates, self.params = _plain_gates(inst)
        self.psi = torch.empty(1 << n, dtype=dtype, device=self.device)
        self.lam = torch.empty_like(self.psi)
        self.buf = torch.zeros(max(len(self.gates), 1), dtype=torch.float64, device=self.device)
        self.energy = torch.zeros(1, dtype=torch.float64, device=self.device)
        loc = {q: n - 1 - q for q in range(n)}
        self.outs = []
        self.gen = {}
        for gi, g in enumerate(self.gates):
            if self.params[gi] is not None:
                gx, gz, gc, _, coef = _generator(g, loc)
                self.gen[gi] = (gx, gz, gc)
                self.outs.append((gi, self.params[gi], coef))
        self.inv = [g if g.kind in ("cx", "cz", "swap") else Gate(g.kind, g.qubits, np.conj(g.mat).T)
                    for g in self.gates]
        self.graph = None

    def launch(self) -> None:
        from .engine import execute_plain

        lib = nat.load()
        n, dev = self.n, self.device
        st = K.stream_ptr(dev)
        nat.call("tq_sv_init_basis", ctypes.c_void_p(self.psi.data_ptr()), n, K.dtype_tag(self.psi),
                 int(getattr(self.inst, "basis", 0)), st)
        execute_plain(self.psi, self.gates)
        K.apply_pauli_sum(self.psi, self.inst.H, out=self.lam)
        p_ws, cap = K._ws(lib.tq_sv_inner_workspace_bytes(n), dev)
        nat.call("tq_sv_inner_re", ctypes.c_void_p(self.psi.data_ptr()), ctypes.c_void_p(self.lam.data_ptr()), n,
                 K.dtype_tag(self.psi), ctypes.c_void_p(self.energy.data_ptr()), p_ws, cap, st)
        for gi in range(len(self.gates) - 1, -1, -1):
            if gi in self.gen:
                gx, gz, gc = self.gen[gi]
                nat.call("tq_sv_generator_im", ctypes.c_void_p(self.psi.data_ptr()),
                         ctypes.c_void_p(self.lam.data_ptr()), n, K.dtype_tag(self.psi), gx, gz, gc,
                         ctypes.c_void_p(self.buf.data_ptr() + 8 * gi), p_ws, cap, st)
            execute_plain(self.psi, [self.inv[gi]])
            execute_plain(self.lam, [self.inv[gi]])

    def capture(self) -> None:
        self.launch()  # warm-up: device tables and workspaces exist before capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g

    def run(self) -> None:
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()

    def result(self) -> tuple[float, np.ndarray]:
        vals = self.buf.cpu().numpy()
        grad = np.zeros(int(self.inst.n_params))
        for gi, p, coef in self.outs:
            grad[p] += coef * vals[gi]
        return float(self.energy.item()), grad


def plain_energy_and_grad(inst, dtype=torch.complex64, device="cuda") -> tuple[float, np.ndarray]:
    """One evaluation of the plain single-circuit engine (launches issued from
    the host, no graph)."""
    eng = PlainEngine(inst, dtype, device)
    eng.launch()
    return eng.result()
