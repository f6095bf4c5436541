"""Continuous-batching VQE serving on one GPU.

Requests (energy, or energy + adjoint gradient) of 10-26+ qubits arrive
over time.  The server

  * admits a request when a stream slot is free and its session's device
    footprint (psi, plus lam for gradients: 2^n * 8 B each in complex64; op
    and Pauli tables, H psi workspace, reverse-sweep partials) fits the HBM
    budget -- evicting idle sessions least-recently-used first;
  * keeps each session's statevectors and compiled circuit resident across
    its optimizer iterations (angles are read on the device, so a new
    parameter vector costs one small copy, no re-planning); a new session's
    estimator is built on a worker thread (the loop keeps admitting and
    polling), and sessions with the same circuit structure share one compiled
    program;
  * gathers requests small enough for the shared-memory-resident classes
    (up to 13 qubits) across sessions into micro-batches: one launch per
    size class evaluates every waiting small request (coalesce.py);
  * enqueues every other admitted request on its own CUDA stream, so the work
    of requests that arrive while others run overlaps on the device, and
    completes requests by polling their events;
  * records arrival / admission / completion times for p50 / p99 latency.

Requests of one session run in arrival order (they share its buffers).  A
request whose footprint alone exceeds the budget fails with an error instead
of waiting forever.  The reference has no serving layer; this is new.
"""
from __future__ import annotations

import threading
import time
from collections import OrderedDict, deque
from concurrent.futures import Future, ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np
import torch


@dataclass
class VqeRequest:
    session: str
    n: int
    structure: list  # [(gate name, qubits, parameter index or None)]
    n_params: int
    H: object  # PauliSum
    theta: np.ndarray
    grad: bool = False
    arrival: float = 0.0
    # results
    energy: float | None = None
    gradient: np.ndarray | None = None
    error: str | None = None
    admitted: float | None = None
    done: float | None = None

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


_PROGRAMS: "OrderedDict" = OrderedDict()  # structure key -> (param gates, compiled program)
_PROGRAMS_LOCK = threading.Lock()
_PROGRAMS_MAX = 256


def default_estimator_factory(req: VqeRequest, dtype, device):
    """A session estimator; sessions with the same circuit structure share one
    compiled program (structure-keyed cache: only angles and H differ)."""
    from .adjoint import ParamGate, ParametricEstimator, build_parametric
    from .batch import structure_gates

    key = (int(req.n), tuple((nm, tuple(int(q) for q in qs), p) for nm, qs, p in req.structure),
           int(req.n_params), str(dtype), str(device))
    with _PROGRAMS_LOCK:
        hit = _PROGRAMS.get(key)
        if hit is not None:
            _PROGRAMS.move_to_end(key)
    if hit is None:
        gates, params = structure_gates(req.structure)
        pg = [ParamGate(g, params[i][0] if i in params else None) for i, g in enumerate(gates)]
        hit = (pg, build_parametric(pg, req.n, req.n_params, dtype))
        with _PROGRAMS_LOCK:
            _PROGRAMS[key] = hit
            while len(_PROGRAMS) > _PROGRAMS_MAX:
                _PROGRAMS.popitem(last=False)
    pg, prog = hit
    est = ParametricEstimator(req.n, pg, req.n_params, req.H, dtype=dtype, device=device, prog=prog)
    if req.grad:
        est._ensure_staged()  # the reverse sweep's tables, here rather than on the serving loop
    return est


@dataclass
class _Session:
    est: object
    bytes: int
    busy: bool = False
    pending: deque = field(default_factory=deque)
    building: Future | None = None  # estimator under construction on the compile worker
    jit: Future | None = None  # circuit-specialised kernels under construction
    small: bool = False  # tables in the micro-batch arenas (coalesce.ResidentBatcher)


class VqeServer:
    def __init__(self, device="cuda", dtype=torch.complex64, hbm_budget: int | None = None, max_inflight: int = 8,
                 estimator_factory: Callable | None = None, streams: Sequence | None = None,
                 compile_workers: int = 1, specialise: bool = True, coalesce: bool = True,
                 max_batch: int = 256):
        """compile_workers > 0: new sessions' estimators are built on a worker
        thread while the loop keeps admitting and polling other requests.
        specialise: each session's circuit-specialised kernels are compiled on
        another worker thread; until they are in place its requests run the
        library's kernels.
        coalesce: requests small enough for the shared-memory-resident classes
        (coalesce.ResidentBatcher) are gathered across sessions into
        micro-batches of up to max_batch requests, one launch per size class."""
        self.device = torch.device(device)
        self.dtype = dtype
        if hbm_budget is None:
            free, _total = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(free * 0.8)
        self.budget = int(hbm_budget)
        self.factory = estimator_factory or default_estimator_factory
        self.streams = list(streams) if streams is not None else [torch.cuda.Stream(self.device)
                                                                   for _ in range(max_inflight)]
        self.free_streams = deque(range(len(self.streams)))
        self.sessions: OrderedDict[str, _Session] = OrderedDict()
        self.queue: deque = deque()
        self.inflight: list = []
        self.used = 0
        self.completed: list[VqeRequest] = []
        self.pool = ThreadPoolExecutor(compile_workers) if compile_workers > 0 else None
        self.jit_pool = ThreadPoolExecutor(1) if specialise else None
        self.batcher = None
        if coalesce and self.device.type == "cuda":
            from .coalesce import ResidentBatcher

            self.batcher = ResidentBatcher(self.device, dtype)
        self.max_batch = int(max_batch)
        self.small_wait: list = []  # (req, sess) admitted, waiting for the next micro-batch
        self.batches: list = []  # (stream slot, ticket, [(req, sess)])
        self.batch_sizes: list[int] = []

    def _small(self, req: VqeRequest) -> bool:
        return self.batcher is not None and self.batcher.fits(req.n)

    def busy(self) -> bool:
        """Requests queued, waiting for a micro-batch or running."""
        return bool(self.queue or self.inflight or self.small_wait or self.batches)

    # ------------------------------------------------------------ memory
    def _footprint(self, req: VqeRequest) -> int:
        """Device bytes of the request's session: states, op and Pauli tables,
        H psi workspace and reverse-sweep partials (adjoint.estimate_footprint)."""
        from .adjoint import estimate_footprint

        if self._small(req):
            # states live in shared memory: the session's tables only, in the batcher's
            # append-only arenas (twice the tables: an arena grows by doubling), once
            if req.session in self.batcher.sessions:
                return 0
            return 2 * self.batcher.table_bytes(req.n, len(req.structure), req.H.n_groups, req.H.n_terms)
        n_param = sum(1 for _, _, p in req.structure if p is not None)
        return estimate_footprint(req.n, len(req.structure), n_param, req.H.n_groups, req.H.n_terms, req.grad,
                                  self.dtype)

    def _evict_for(self, need: int) -> bool:
        for key in list(self.sessions):
            if self.used + need <= self.budget:
                break
            s = self.sessions[key]
            if not s.busy and not s.pending and not s.small:  # arena tables are never freed
                self.used -= s.bytes
                del self.sessions[key]
        return self.used + need <= self.budget

    # ------------------------------------------------------------ API
    def submit(self, req: VqeRequest) -> None:
        if not req.arrival:
            req.arrival = time.perf_counter()
        self.queue.append(req)

    def step(self) -> int:
        """Admit what fits, poll running work; returns the number completed now."""
        self._admit()
        done = self._poll()
        if self.batcher is not None:
            done += self._poll_batches()
            self._launch_batch()
        return done

    def drain(self, timeout: float = 600.0) -> None:
        t0 = time.perf_counter()
        while self.busy():
            if not self.step():
                time.sleep(0.0002)
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("serving loop did not drain")

    # ------------------------------------------------------------ internals
    def _admit(self) -> None:
        keep = deque()
        while self.queue:
            req = self.queue.popleft()
            sess = self.sessions.get(req.session)
            if sess is not None and sess.busy:
                keep.append(req)  # same-session requests run in order
                continue
            small = self._small(req)
            if not small and not self.free_streams:
                keep.append(req)
                continue
            need = self._footprint(req)
            if sess is not None:
                need = max(0, need - sess.bytes)
            if self._footprint(req) > self.budget:
                req.error = f"request needs {self._footprint(req)} B, above the {self.budget} B budget"
                req.done = time.perf_counter()
                self.completed.append(req)
                continue
            if self.used + need > self.budget and not self._evict_for(need):
                keep.append(req)
                continue
            self._start(req, need)
        self.queue = keep

    def _start(self, req: VqeRequest, need: int) -> None:
        sess = self.sessions.get(req.session)
        if sess is None:
            sess = _Session(None, 0)
            self.sessions[req.session] = sess
        sess.bytes += need
        self.used += need
        self.sessions.move_to_end(req.session)
        sess.busy = True
        req.admitted = time.perf_counter()
        if self._small(req):
            sess.small = True
            if sess.est is None and sess.building is None:
                reg = (self.batcher.register, req.session, req.n, req.structure, req.n_params, req.H)
                if self.pool is not None:
                    sess.building = self.pool.submit(*reg)
                else:
                    sess.est = reg[0](*reg[1:])
            self.small_wait.append((req, sess))
            return
        si = self.free_streams.popleft()
        if sess.est is None and self.pool is not None:
            # build off the loop; launched by _poll once the estimator exists
            sess.building = self.pool.submit(self.factory, req, self.dtype, self.device)
            self.inflight.append((req, si, None, None, None, sess))
            return
        ev, e_h, sv_h = self._launch(sess, req, si)
        self.inflight.append((req, si, ev, e_h, sv_h, sess))

    def _specialise(self, sess: _Session) -> None:
        """Queue the session's kernel specialisation (once, and once more when its
        reverse sweep appears after an energy-only start)."""
        if self.jit_pool is None or not hasattr(sess.est, "specialise"):
            return
        staged = getattr(sess.est, "_staged", None)
        if sess.jit is None or (sess.jit.done() and staged is not None and not staged.kernels):
            sess.jit = self.jit_pool.submit(sess.est.specialise)

    def _launch(self, sess: _Session, req: VqeRequest, si: int):
        """Enqueue the request's device work on stream si; returns (event, host
        energy buffer, host slot-value buffer or None)."""
        stream = self.streams[si]
        stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(stream):
            if sess.est is None:
                sess.est = self.factory(req, self.dtype, self.device)
            self._specialise(sess)
            if req.grad:
                e, sv = sess.est.energy_and_grad_async(req.theta)
            else:
                e, sv = sess.est.energy_async(req.theta), None
            e_h = torch.empty(1, dtype=torch.float64, pin_memory=True)
            e_h.copy_(e.reshape(-1)[:1], non_blocking=True)
            sv_h = None
            if sv is not None:
                sv_h = torch.empty(sv.numel(), dtype=torch.float64, pin_memory=True)
                sv_h.copy_(sv, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev, e_h, sv_h

    def _ready(self, ev) -> bool:
        return ev.query()

    # ------------------------------------------------------------ micro-batches
    def _launch_batch(self) -> None:
        """One micro-batch of every waiting small request whose session tables
        are in place, on a free stream."""
        if not self.small_wait or not self.free_streams:
            return
        ready, rest = [], []
        for req, sess in self.small_wait:
            if sess.est is None and sess.building is not None and sess.building.done():
                try:
                    sess.est = sess.building.result()
                except Exception as exc:  # a session whose tables cannot be built fails its request
                    req.error = f"{type(exc).__name__}: {exc}"
                    req.done = time.perf_counter()
                    sess.busy = False
                    self.completed.append(req)
                    sess.building = None
                    continue
                sess.building = None
            if sess.est is not None and len(ready) < self.max_batch:
                ready.append((req, sess))
            else:
                rest.append((req, sess))
        self.small_wait = rest
        if not ready:
            return
        if not self.batches:
            self.batcher.release_retired()
        si = self.free_streams.popleft()
        ticket = self.batcher.launch([(r.session, r.theta) for r, _ in ready], self.streams[si])
        self.batches.append((si, ticket, ready))
        self.batch_sizes.append(len(ready))

    def _poll_batches(self) -> int:
        done = 0
        still = []
        for si, ticket, members in self.batches:
            if not self._ready(ticket["event"]):
                still.append((si, ticket, members))
                continue
            now = time.perf_counter()
            for (req, sess), (e, g) in zip(members, self.batcher.results(ticket)):
                req.energy = e
                if req.grad:
                    req.gradient = g
                req.done = now
                sess.busy = False
                self.completed.append(req)
                done += 1
            self.free_streams.append(si)
        self.batches = still
        return done

    def _poll(self) -> int:
        done = 0
        still = []
        for item in self.inflight:
            req, si, ev, e_h, sv_h, sess = item
            if ev is None:  # estimator still being built
                if not sess.building.done():
                    still.append(item)
                    continue
                try:
                    sess.est = sess.building.result()
                except Exception as exc:  # a session that cannot be built fails its request
                    sess.building = None
                    req.error = f"{type(exc).__name__}: {exc}"
                    req.done = time.perf_counter()
                    sess.busy = False
                    self.free_streams.append(si)
                    self.completed.append(req)
                    done += 1
                    continue
                sess.building = None
                ev, e_h, sv_h = self._launch(sess, req, si)
                still.append((req, si, ev, e_h, sv_h, sess))
                continue
            if not self._ready(ev):
                still.append(item)
                continue
            req.energy = float(e_h[0])
            if sv_h is not None:
                req.gradient = sess.est.grad_from_slots(sv_h.numpy())
            req.done = time.perf_counter()
            sess.busy = False
            self.free_streams.append(si)
            self.completed.append(req)
            done += 1
        self.inflight = still
        return done


def make_trace(count: int, rate: float, seed: int = 5, n_range=(10, 26), depth_range=(2, 10),
               terms_range=(20, 1000), grad_fraction: float = 0.3, iterations: int = 1) -> list[VqeRequest]:
    """Poisson arrivals (mean rate `rate` per second) of HEA requests; each
    session issues `iterations` requests (optimizer steps) in sequence."""
    from .hamiltonian import random_pauli_sum
    from .workloads import hea_rz_ops_params

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    sessions = max(1, count // iterations)
    for s in range(sessions):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        d = int(rng.integers(depth_range[0], depth_range[1] + 1))
        K = int(rng.integers(terms_range[0], terms_range[1] + 1))
        H = random_pauli_sum(n, K, rng)
        struct = hea_rz_ops_params(n, d)
        npar = 2 * n * d
        grad = bool(rng.random() < grad_fraction)
        for it in range(iterations):
            t += float(rng.exponential(1.0 / rate))
            out.append(VqeRequest(f"s{s}", n, struct, npar, H, rng.uniform(0, 2 * np.pi, npar), grad, arrival=t))
    return out


def replay(server: VqeServer, trace: Sequence[VqeRequest], timeout: float = 600.0) -> dict:
    """Feed requests at their (relative) arrival times; returns latency stats."""
    t0 = time.perf_counter()
    pending = deque(sorted(trace, key=lambda r: r.arrival))
    for r in pending:
        r.arrival = t0 + r.arrival
    while pending or server.busy():
        now = time.perf_counter()
        while pending and pending[0].arrival <= now:
            server.submit(pending.popleft())
        if not server.step():
            time.sleep(0.0001)
        if now - t0 > timeout:
            raise TimeoutError("trace replay did not finish")
    wall = time.perf_counter() - t0
    lat = np.array([r.latency for r in trace if r.error is None])
    return {"requests": len(trace), "errors": sum(r.error is not None for r in trace), "wall_s": wall,
            "throughput_rps": len(trace) / wall, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "micro_batches": len(getattr(server, "batch_sizes", [])),
            "batched_requests": int(sum(getattr(server, "batch_sizes", [])))}
