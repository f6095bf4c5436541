"""Adjoint (reverse-sweep) energy gradients on the GPU.

For psi = U_G ... U_1 |psi0> and E = <psi|H|psi>:
  forward:  psi (fused tile passes), lam = H psi, E = Re <psi|lam>;
  reverse:  for g = G..1: dE/dtheta_g += coef_g * Im <lam|G_g|psi>, then
            psi <- U_g^dag psi, lam <- U_g^dag lam,
which is the reference's CI-space reverse loop (energy_and_grad_civector,
chem_libs/quantum_chem_library/civector_ops.py:141-200) generalised to gates
and Pauli rotations.  The reverse sweep runs as adjoint tile passes
(``tq_sv_adjoint_tiles``) carrying psi and lam together, gradient reductions
fused in.  ``AdjointEnergy`` wraps it as a torch.autograd.Function, the
replacement for the reference's autograd through per-gate einsums
(numerics/backends/pytorch_backend.py:446-564).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any, Sequence

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .hamiltonian import PauliSum, as_pauli_sum
from .ir import Gate, lower_ops
from .program import DEFAULT_NLOW, TILE_OP_DTYPE, _canon, compile_forward, encode_passes, plan_passes, tileable

TILE_OP_RECORD_BYTES = TILE_OP_DTYPE.itemsize


@dataclass
class ParamGate:
    """Gate whose angle = scale * theta[param] + shift (param None = fixed)."""

    gate: Gate
    param: int | None = None
    scale: float = 1.0


@dataclass
class AdjointProgram:
    n: int
    dtype: torch.dtype
    forward: Any
    reverse: list  # ('tiles', EncodedTiles) | ('gate', Gate)
    n_slots: int
    slot_param: np.ndarray  # slot -> param index
    slot_coef: np.ndarray  # slot -> coef * scale
    n_params: int


def _build(pgates: Sequence[ParamGate], n: int, n_params: int, dtype, t_fwd=None, t_adj=None) -> AdjointProgram:
    from .autotune import tile_bits_for

    gates = [_canon(p.gate) for p in pgates]
    for g in gates:
        if not tileable(g):
            raise NotImplementedError(f"adjoint gradient through a '{g.kind}' gate is not supported")
    fwd = compile_forward(gates, n, dtype, t=t_fwd)
    t_adj = t_adj or tile_bits_for(n, dtype, adjoint=True)
    segs = plan_passes(list(reversed(gates)), n, t_adj, DEFAULT_NLOW)
    # plan_passes on the reversed list gives the reverse sweep order directly;
    # indices refer to the reversed list.
    rgates = list(reversed(gates))
    slots = {}
    slot_param = []
    slot_scale = []
    G = len(gates)
    for ri, g in enumerate(rgates):
        pg = pgates[G - 1 - ri]
        if pg.param is not None:
            slots[ri] = len(slot_param)
            slot_param.append(pg.param)
            slot_scale.append(pg.scale)
    rev = []
    coef = np.zeros(len(slot_param))
    for s in segs:
        if s.kind == "gate":  # pragma: no cover - tileable check above
            raise NotImplementedError
        enc, coefs = encode_passes(n, s.passes, rgates, fuse=False, reverse=False, slots=slots)
        for sl, c in coefs:
            coef[sl] = c
        rev.append(("tiles", enc))
    return AdjointProgram(n, dtype, fwd, rev, len(slot_param), np.asarray(slot_param, dtype=np.int64),
                          coef * np.asarray(slot_scale, dtype=np.float64), n_params)


def _with_angles(pgates: Sequence[ParamGate], theta: np.ndarray) -> list[ParamGate]:
    """Rebuild parametrised gate matrices for new angles."""
    from .ir import _rot_gate, pauli_rotation

    out = []
    for p in pgates:
        if p.param is None:
            out.append(p)
            continue
        a = p.scale * float(theta[p.param])
        g = p.gate
        if g.kind == "prot":
            ng = pauli_rotation(g.pauli, a)
        elif g.rot is not None and g.rot[0] == "phase":
            ng = Gate("d1", g.qubits, np.diag([1.0, np.exp(1j * a)]), rot=("phase", a, a))
        else:
            ng = _rot_gate(g.rot[0], g.qubits, a)
        out.append(ParamGate(ng, p.param, p.scale))
    return out


def reverse_sweep(prog: AdjointProgram, psi: torch.Tensor, lam: torch.Tensor,
                  theta: torch.Tensor | None = None) -> torch.Tensor:
    """Run the adjoint passes in place on (psi, lam); returns slot values (device, FP64).
    theta feeds ops compiled with device-side angles."""
    dt = K.dtype_tag(psi)
    out = torch.zeros(max(prog.n_slots, 1), dtype=torch.float64, device=psi.device)
    lib = nat.load()
    th = ctypes.c_void_p(theta.data_ptr()) if theta is not None else None
    for kind, enc in prog.reverse:
        ops = enc.device_ops(psi.device)
        # slots of this segment only are written; other segments' slots must be kept
        seg_out = torch.empty_like(out)
        p, cap = K._ws(lib.tq_sv_adjoint_tiles_workspace_bytes(prog.n, prog.n_slots), psi.device)
        nat.call("tq_sv_adjoint_tiles", ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(lam.data_ptr()), prog.n, dt,
                 enc.passes, enc.n_passes, ctypes.c_void_p(ops.data_ptr()), th, prog.n_slots,
                 ctypes.c_void_p(seg_out.data_ptr()), p, cap, K.stream_ptr(psi.device))
        out += seg_out
    return out[: prog.n_slots]


def build_parametric(pgates: Sequence[ParamGate], n: int, n_params: int, dtype, t_fwd=None,
                     t_adj=None) -> AdjointProgram:
    """Compile once for any angles: parametrised gates read theta[param] * scale
    on the device, so a new parameter vector needs no re-planning."""
    from .autotune import tile_bits_for

    gates = [_canon(p.gate) for p in pgates]
    for g in gates:
        if not tileable(g):
            raise NotImplementedError(f"adjoint gradient through a '{g.kind}' gate is not supported")
    params = {i: (p.param, p.scale) for i, p in enumerate(pgates) if p.param is not None}
    fwd = compile_forward(gates, n, dtype, t=t_fwd, params=params)
    t_adj = t_adj or tile_bits_for(n, dtype, adjoint=True)
    rgates = list(reversed(gates))
    G = len(gates)
    rparams = {G - 1 - gi: v for gi, v in params.items()}
    slots, slot_param, slot_scale = {}, [], []
    for ri in sorted(rparams):
        slots[ri] = len(slot_param)
        slot_param.append(rparams[ri][0])
        slot_scale.append(rparams[ri][1])
    rev = []
    coef = np.zeros(len(slot_param))
    for s in plan_passes(rgates, n, t_adj, DEFAULT_NLOW):
        if s.kind != "tiles":
            raise NotImplementedError("every gate of an adjoint program must fit a tile")
        enc, coefs = encode_passes(n, s.passes, rgates, fuse=False, slots=slots, params=rparams)
        for sl, c in coefs:
            coef[sl] = c
        rev.append(("tiles", enc))
    return AdjointProgram(n, dtype, fwd, rev, len(slot_param), np.asarray(slot_param, dtype=np.int64),
                          coef * np.asarray(slot_scale, dtype=np.float64), n_params)


# From this size up the reverse sweep of ParametricEstimator runs as
# register-staged adjoint passes (the batched path's wave kernels on a
# one-instance plan) instead of the shared-memory tile passes, unless more
# than STAGED_ADJOINT_MAX_COLD of its gates may have no register routine there
# (rotations with two or more X/Y qubits, ZZ rotations, controlled rotations,
# dense 4x4 gates: they
# run from shared memory, which measured slower than the tile passes for
# UCCSD's Pauli-string exponentials at 16 qubits).
STAGED_ADJOINT_MIN_N = 14
STAGED_ADJOINT_MAX_COLD = 0.1


def _cold_in_staged_adjoint(g: Gate) -> bool:
    from .ir import ROTATION_GENERATORS

    if g.rot is None:
        return g.kind == "u2"
    name = g.rot[0]
    if name == "cry":
        return True
    letters = [p for _, p in g.pauli] if name == "prot" else list(ROTATION_GENERATORS.get(name, ""))
    nxy = sum(p in "XY" for p in letters)
    # register routines: one X/Y qubit (Z factors become signs), or a single Z
    return not (nxy == 1 or (nxy == 0 and len(letters) == 1))


class _StagedReverse:
    """The reverse sweep of one state as wave adjoint passes (kind 2 of
    tq_wave_run): the passes are encoded as the batched path encodes an
    instance, the work items (one per tile and pass) and the fixed-order
    gradient reductions are built with numpy, psi and lam live in one pool
    (psi_off 0, lam_off 2^n), and the reductions write dE/dtheta per
    parameter."""

    def __init__(self, n: int, pgates: Sequence[ParamGate], n_params: int, dtype, device):
        from collections import defaultdict

        from .program import STAGE_DTYPE, TILE_OP_DTYPE
        from .waves import PASS_DTYPE, ROP_JOB_DTYPE, WAVE_ITEM_DTYPE, WavePlan, _dev

        gates = [_canon(p.gate) for p in pgates]
        for g in gates:
            if not tileable(g):
                raise NotImplementedError(f"adjoint gradient through a '{g.kind}' gate is not supported")
        params = {i: (int(p.param), float(p.scale)) for i, p in enumerate(pgates) if p.param is not None}
        t = min(n, 13 if dtype == torch.complex64 else 12)
        enc_plan = WavePlan([], dtype, device, t=t, hbits=min(12, n), max_ops=256)  # tables only
        enc = enc_plan._encode(n, gates, params)
        self.t, self.dt, self.rb = t, enc_plan.dt, enc_plan.adj_rb
        self.max_ops = enc_plan.adj_max_ops
        N = 1 << n
        ntile = 1 << (n - t)
        blocks, rows, base = [], [], 0
        self.runs = []  # (first item, item count) per adjoint pass
        self.run_pids = []  # pass id of each run
        self.kernels: dict = {}  # pass id -> specialised kernel (specialise())
        for pid, nops, pslots in enc["adj"]:
            self.run_pids.append(pid)
            it = np.zeros(ntile, dtype=WAVE_ITEM_DTYPE)
            it["lam_off"] = N
            it["pass"] = pid
            it["tile"] = np.arange(ntile)
            it["part_off"] = base + np.arange(ntile) * nops
            it["n"] = n
            it["basis_lo"] = -1
            self.runs.append((ntile * len(blocks), ntile))
            blocks.append(it)
            rows += [(base + kk, ntile, nops, coef, slot) for kk, slot, coef in pslots]
            base += ntile * nops
        if base >= 2 ** 31:
            raise NotImplementedError("too many gradient partials for one reverse sweep")
        # a parameter shared by several ops gets one row per op: rows of one
        # reduction launch must write distinct outputs
        seen, layers = defaultdict(int), defaultdict(list)
        for r in rows:
            layers[seen[r[4]]].append(r)
            seen[r[4]] += 1
        rows = [r for lay in sorted(layers) for r in layers[lay]]
        self.layers = []
        o = 0
        for lay in sorted(layers):
            self.layers.append((o, len(layers[lay])))
            o += len(layers[lay])
        items = np.concatenate(blocks) if blocks else np.zeros(0, dtype=WAVE_ITEM_DTYPE)
        # op records of every adjoint pass, compiled once per sweep (tq_wave_rops):
        # one job per pass (one instance), its items point at the job's records
        st_all = np.concatenate(enc_plan.stages) if enc_plan.stages else np.zeros(0, STAGE_DTYPE)
        jobs = np.zeros(len(self.runs), dtype=ROP_JOB_DTYPE)
        nrec = 0
        for r, ((first, count), pid) in enumerate(zip(self.runs, self.run_pids)):
            pa = enc_plan.passes[pid]
            sb, se = int(pa[2]), int(pa[3])
            op0 = int(st_all[sb]["op_begin"]) if se > sb else 0
            nops = int(st_all[se - 1]["op_end"]) - op0 if se > sb else 0
            jobs[r] = (op0, nops, 0, 1, nrec)
            items["group_begin"][first:first + count] = nrec
            items["group_count"][first:first + count] = nops
            nrec += nops
        n_rec = nrec
        self.rop_jobs_dev = _dev(jobs if len(jobs) else np.zeros(1, ROP_JOB_DTYPE), device)
        self.n_rop_jobs = len(jobs)
        self.rops_buf = torch.empty(max(int(nat.load().tq_jit_rops_bytes(enc_plan.dt, n_rec)), 16), dtype=torch.uint8,
                                    device=device)
        pa = np.zeros(len(enc_plan.passes), dtype=PASS_DTYPE)
        for k, (tt, nl, b0, e0, pos) in enumerate(enc_plan.passes):
            pa[k] = (tt, nl, b0, e0, pos)
        self._host = (np.concatenate(enc_plan.stages) if enc_plan.stages else np.zeros(0, STAGE_DTYPE),
                      np.concatenate(enc_plan.ops) if enc_plan.ops else np.zeros(0, TILE_OP_DTYPE),
                      list(enc_plan.passes))
        self.device = torch.device(device)
        self.items_dev = _dev(items, device)
        self.passes_dev = _dev(pa, device)
        self.stages_dev = _dev(np.concatenate(enc_plan.stages) if enc_plan.stages else np.zeros(1, STAGE_DTYPE),
                               device)
        self.ops_dev = _dev(np.concatenate(enc_plan.ops) if enc_plan.ops else np.zeros(1, TILE_OP_DTYPE), device)
        self.r_first = torch.tensor([r[0] for r in rows] or [0], dtype=torch.int32, device=device)
        self.r_count = torch.tensor([r[1] for r in rows] or [0], dtype=torch.int32, device=device)
        self.r_stride = torch.tensor([r[2] for r in rows] or [0], dtype=torch.int32, device=device)
        self.r_scale = torch.tensor([r[3] for r in rows] or [0.0], dtype=torch.float64, device=device)
        self.r_out = torch.tensor([r[4] for r in rows] or [0], dtype=torch.int32, device=device)
        self.partials = torch.zeros(max(base, 1), dtype=torch.float64, device=device)
        self.pool = torch.empty(2 * N, dtype=dtype, device=device)
        self.psi, self.lam = self.pool[:N], self.pool[N:]
        self.grads = torch.zeros(max(n_params, 1), dtype=torch.float64, device=device)
        self.n_params = n_params

    def specialise(self) -> int:
        """Circuit-specialised kernels for the adjoint passes (4-bit stages);
        returns how many passes have one.  Safe to call from another thread:
        run() takes each kernel once it is in place."""
        from . import jit

        if self.rb != 4:
            return 0
        stages, ops, passes = self._host
        rows = {pid: passes[pid] for pid in self.run_pids}
        kern = jit.wave_kernels(2, self.t, stages, ops, rows, self.dt == 1, self.max_ops, self.device)
        self.kernels = kern
        return len(kern)

    def run(self, theta: torch.Tensor) -> torch.Tensor:
        from .waves import WAVE_ITEM_DTYPE

        P = ctypes.c_void_p
        st = K.stream_ptr(self.grads.device)
        isz = WAVE_ITEM_DTYPE.itemsize
        self.grads.zero_()
        kern = self.kernels
        if kern and self.n_rop_jobs:
            nat.call("tq_wave_rops", self.dt, P(self.rop_jobs_dev.data_ptr()), self.n_rop_jobs,
                     P(self.ops_dev.data_ptr()), P(theta.data_ptr()), P(self.rops_buf.data_ptr()), st)
        for (first, count), pid in zip(self.runs, self.run_pids):
            k = kern.get(pid)
            if k:
                nat.call("tq_jit_wave_run", P(k), 2, self.dt, P(self.items_dev.data_ptr() + isz * first), count,
                         self.t, P(self.passes_dev.data_ptr()), P(self.stages_dev.data_ptr()),
                         P(self.ops_dev.data_ptr()), P(theta.data_ptr()), P(self.rops_buf.data_ptr()),
                         P(self.pool.data_ptr()), P(self.partials.data_ptr()), self.max_ops, st)
                continue
            nat.call("tq_wave_run", 2, self.dt, P(self.items_dev.data_ptr() + isz * first), count, self.t, 12,
                     self.rb, P(self.passes_dev.data_ptr()), P(self.stages_dev.data_ptr()),
                     P(self.ops_dev.data_ptr()), None, None, P(theta.data_ptr()), P(self.pool.data_ptr()),
                     P(self.partials.data_ptr()), None, self.max_ops, st)
        for b, c in self.layers:
            nat.call("tq_wave_reduce", P(self.partials.data_ptr()), P(self.r_first.data_ptr() + 4 * b),
                     P(self.r_count.data_ptr() + 4 * b), P(self.r_stride.data_ptr() + 4 * b),
                     P(self.r_scale.data_ptr() + 8 * b), P(self.r_out.data_ptr() + 4 * b), c,
                     P(self.grads.data_ptr()), 1, st)
        return self.grads[:self.n_params]


def estimate_footprint(n: int, n_gates: int, n_param_ops: int, n_groups: int, n_terms: int, grad: bool, dtype,
                       staged_reverse: bool | None = None) -> int:
    """Device bytes of one estimator session: psi (and lam for gradients),
    the forward and reverse op tables, the Pauli tables, the tiled H psi
    workspace and, for the register-staged reverse sweep (n >= 14), its FP64
    gradient partials (one per parametrised op and tile of 2^t amplitudes)."""
    S = 8 if dtype == torch.complex64 else 16
    N = 1 << int(n)
    b = (2 if grad else 1) * S * N
    b += 2 * n_gates * TILE_OP_RECORD_BYTES + n_groups * 16 + n_terms * 32
    if n >= K.TILED_MIN_N:
        b += int(nat.load().tq_sv_pauli_sum_tiled_workspace_bytes(int(n), 0 if S == 8 else 1, int(n_groups), 1))
    if staged_reverse is None:
        staged_reverse = n >= STAGED_ADJOINT_MIN_N
    if grad and staged_reverse:
        t = min(int(n), 13 if S == 8 else 12)
        b += 8 * n_param_ops * (1 << (int(n) - t))
    return int(b)


class ParametricEstimator:
    """Energy / adjoint gradient of one circuit structure, compiled once; each
    call takes a parameter vector (host array or float64 device tensor)."""

    def __init__(self, n: int, pgates: Sequence[ParamGate], n_params: int, hamiltonian, dtype=torch.complex64,
                 device="cuda", init_basis: int = 0, prog: AdjointProgram | None = None):
        """prog: a program already compiled for this structure (build_parametric
        of the same pgates, n, n_params and dtype); its tables are read-only and
        may be shared by estimators on one device."""
        self.n = int(n)
        self.n_params = int(n_params)
        self.H = as_pauli_sum(hamiltonian, self.n)
        self.dtype = dtype
        self.device = torch.device(device)
        self.init_basis = int(init_basis)
        self._pgates = list(pgates)
        self.prog = prog if prog is not None else build_parametric(pgates, self.n, self.n_params, dtype)
        self.theta = torch.zeros(max(self.n_params, 1), dtype=torch.float64, device=self.device)
        self._staged = None
        cold = sum(_cold_in_staged_adjoint(_canon(p.gate)) for p in pgates) / max(len(pgates), 1)
        # built on the first gradient call (energy-only use never pays for it)
        self._staged_pending = (list(pgates) if self.n >= STAGED_ADJOINT_MIN_N and self.device.type == "cuda"
                                and cold <= STAGED_ADJOINT_MAX_COLD else None)
        self.psi = torch.empty(1 << self.n, dtype=dtype, device=self.device)
        self.lam = None
        self._jit_ws: dict = {}  # this session's op-record workspaces of the specialised passes

    def footprint_bytes(self, grad: bool) -> int:
        """Device bytes a session of this estimator holds: see estimate_footprint."""
        n_param_ops = sum(1 for pg in self._pgates if pg.param is not None)
        staged = self._staged is not None or self._staged_pending is not None
        return estimate_footprint(self.n, len(self._pgates), n_param_ops, self.H.n_groups, self.H.n_terms, grad,
                                  self.dtype, staged_reverse=staged)

    def _ensure_staged(self) -> None:
        if self._staged_pending is None:
            return
        pg, self._staged_pending = self._staged_pending, None
        try:
            self._staged = _StagedReverse(self.n, pg, self.n_params, self.dtype, self.device)
        except NotImplementedError:  # a pass the wave kernels do not take: tile passes instead
            return
        self.psi, self.lam = self._staged.psi, self._staged.lam

    def _forward(self, theta) -> torch.Tensor:
        if isinstance(theta, torch.Tensor) and theta.is_cuda:
            self.theta.copy_(theta.reshape(-1), non_blocking=True)
        else:
            self.theta.copy_(torch.as_tensor(np.asarray(theta, dtype=np.float64)).reshape(-1), non_blocking=True)
        nat.call("tq_sv_init_basis", ctypes.c_void_p(self.psi.data_ptr()), self.n, K.dtype_tag(self.psi),
                 self.init_basis, K.stream_ptr(self.device))
        return self.prog.forward.run(self.psi, self.theta, self._jit_ws)

    def specialise(self) -> int:
        """Circuit-specialised kernels for the forward passes and, when built,
        the staged reverse sweep.  Meant to run on a worker thread while the
        session already serves requests with the library kernels: each pass
        switches to its specialised kernel once that is in place (the program
        may be shared with other sessions; op records use this session's
        workspace).  Returns the number of specialised passes."""
        cnt = self.prog.forward.specialise(self.dtype, self.device, stage_bits=4)
        staged = self._staged
        if staged is not None:
            cnt += staged.specialise()
        return cnt

    def energy_async(self, theta) -> torch.Tensor:
        """Enqueue an energy evaluation on the current stream; returns a device
        scalar <psi|H|psi> / <psi|psi> (the circuit is unitary, so the division
        only removes the norm drift of rounded complex64 rotations)."""
        psi = self._forward(theta)
        return K.pauli_expectation(psi, self.H) / K.norm2(psi)

    def energy_and_grad_async(self, theta) -> tuple[torch.Tensor, torch.Tensor]:
        """Enqueue energy + adjoint gradient; returns (device energy, device
        slot values -- per-parameter gradients on the staged path), both divided
        by <psi|psi> as in energy_async."""
        self._ensure_staged()
        psi = self._forward(theta)
        if self.lam is None:
            self.lam = torch.empty_like(self.psi)
        K.apply_pauli_sum(psi, self.H, out=self.lam)
        q = K.norm2(psi)
        e = K.inner_re(psi, self.lam) / q
        if self._staged is not None:
            return e, self._staged.run(self.theta) / q
        sv = reverse_sweep(self.prog, psi, self.lam, self.theta)
        return e, sv / q

    def grad_from_slots(self, slot_vals: np.ndarray) -> np.ndarray:
        if self._staged is not None:
            return np.asarray(slot_vals, dtype=np.float64).copy()
        return slots_to_grad(self.prog, slot_vals)

    def energy(self, theta) -> float:
        return float(self.energy_async(theta).item())

    def energy_and_grad(self, theta) -> tuple[float, np.ndarray]:
        e, sv = self.energy_and_grad_async(theta)
        return float(e.item()), self.grad_from_slots(sv.cpu().numpy())


def slots_to_grad(prog: AdjointProgram, slot_vals: np.ndarray) -> np.ndarray:
    g = np.zeros(prog.n_params, dtype=np.float64)
    np.add.at(g, prog.slot_param, prog.slot_coef * slot_vals)
    return g


class AdjointEstimator:
    """Energy and adjoint gradient of one parametrised circuit and Pauli sum.

    `pgates` fixes the structure; angles come from theta at each call.  The
    structure (pass plans) is compiled once and reused across calls.
    """

    def __init__(self, n: int, pgates: Sequence[ParamGate], n_params: int, hamiltonian, dtype=torch.complex64,
                 device="cuda", init_basis: int = 0):
        self.n = int(n)
        self.pgates = list(pgates)
        self.n_params = int(n_params)
        self.H = as_pauli_sum(hamiltonian, self.n)
        self.dtype = dtype
        self.device = torch.device(device)
        self.init_basis = int(init_basis)
        self._lam = None

    def _program(self, theta):
        pg = _with_angles(self.pgates, np.asarray(theta, dtype=np.float64))
        return _build(pg, self.n, self.n_params, self.dtype)

    def state(self, theta) -> torch.Tensor:
        prog = self._program(theta)
        psi = K.init_statevector(self.n, self.dtype, self.device, self.init_basis)
        return prog.forward.run(psi)

    def energy(self, theta) -> float:
        psi = self.state(theta)
        return float(K.pauli_expectation(psi, self.H).item())

    def energy_and_grad(self, theta) -> tuple[float, np.ndarray]:
        prog = self._program(theta)
        psi = K.init_statevector(self.n, self.dtype, self.device, self.init_basis)
        prog.forward.run(psi)
        lam = K.apply_pauli_sum(psi, self.H)
        e = K.inner_re(psi, lam)
        sv = reverse_sweep(prog, psi, lam)
        e_h = float(e.item())
        return e_h, slots_to_grad(prog, sv.cpu().numpy())


class AdjointEnergy(torch.autograd.Function):
    """E(theta) with an adjoint-kernel backward: use as AdjointEnergy.apply(theta, estimator)."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, est: AdjointEstimator):
        e, g = est.energy_and_grad(theta.detach().cpu().numpy())
        ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
        return torch.tensor(e, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout * g, None


class PauliEnergyFn(torch.autograd.Function):
    """E = Re <psi|H|psi> of a device state for a Pauli-sum H, differentiable in
    psi (backward: dE/dpsi = 2 H psi in torch's complex-gradient convention, the
    input _StateFn's adjoint backward takes).  Replaces dynamics.expectation
    with a dense H (dynamics.py:117-126) without forming the 2^n x 2^n matrix."""

    @staticmethod
    def forward(ctx, psi: torch.Tensor, H):
        ctx.save_for_backward(psi)
        ctx.H = H
        return K.pauli_expectation(psi.detach().contiguous(), H).reshape(())

    @staticmethod
    def backward(ctx, gout):
        (psi,) = ctx.saved_tensors
        hpsi = K.apply_pauli_sum(psi.detach().contiguous(), ctx.H)
        scale = (2.0 * gout).to(hpsi.real.dtype)
        return scale * hpsi, None


def pauli_energy(psi, H):
    """Differentiable <psi|H|psi> of a device state (torch) or a host state (numpy: float)."""
    if isinstance(psi, torch.Tensor) and psi.is_cuda:
        return PauliEnergyFn.apply(psi, H)
    arr = psi.detach().cpu().numpy() if isinstance(psi, torch.Tensor) else np.asarray(psi)
    dev = K.from_array(arr, dtype=torch.complex128 if arr.dtype == np.complex128 else torch.complex64)
    return float(K.pauli_expectation(dev, H).item())


# ---------------------------------------------------------------- circuit-level autograd
def _angle_leaves(circuit) -> tuple[list, list]:
    """(angle tensors requiring grad, (op index, arg position) for each)."""
    leaves, where = [], []
    for oi, op in enumerate(getattr(circuit, "ops", [])):
        if isinstance(op, (list, tuple)):
            for ai, a in enumerate(op[1:], start=1):
                if isinstance(a, torch.Tensor) and a.requires_grad:
                    leaves.append(a)
                    where.append((oi, ai))
    return leaves, where


class _StateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, engine, circuit, pgates, n, *angles):
        prog = _build(pgates, n, len(angles), engine.dtype)
        psi = K.init_statevector(n, engine.dtype, engine.device)
        prog.forward.run(psi)
        ctx.prog = prog
        ctx.save_for_backward(psi.clone())
        ctx.n_angles = len(angles)
        return psi

    @staticmethod
    def backward(ctx, gout):
        (psi,) = ctx.saved_tensors
        prog = ctx.prog
        lam = gout.detach().to(dtype=psi.dtype).contiguous().clone()
        ps = psi.clone()
        sv = reverse_sweep(prog, ps, lam).cpu().numpy()
        g = 0.5 * slots_to_grad(prog, sv)  # dL/dtheta = 1/2 Im<grad|G|psi>
        grads = [torch.tensor(float(x), dtype=torch.float64, device=gout.device) for x in g]
        return (None, None, None, None, *grads)


def state_with_grad(engine, circuit) -> torch.Tensor:
    """Final state as a differentiable function of the circuit's tensor angles."""
    n = int(circuit.num_qubits)
    if getattr(circuit, "_initial_state", None) is not None:
        raise NotImplementedError("autograd with a custom initial state")
    gates, _ = lower_ops(circuit, mode="state", extended=engine.extended_gates)
    leaves, where = _angle_leaves(circuit)
    leaf_id = {id(t): k for k, t in enumerate(leaves)}
    pgates = []
    for g in gates:
        src = g.rot[2] if g.rot is not None else None
        if isinstance(src, torch.Tensor) and id(src) in leaf_id:
            pgates.append(ParamGate(g, leaf_id[id(src)], 1.0))
        else:
            pgates.append(ParamGate(g, None))
    out = _StateFn.apply(engine, circuit, pgates, n, *leaves)
    return out
