"""Serving loop: admission by HBM footprint, LRU eviction of idle sessions,
per-session ordering, over-budget rejection (host logic, CPU, fake device
work); and on the GPU, each request's result is the same alone and in the
concurrent mix."""
import numpy as np
import pytest
import torch

from tyxonq_gb300.serving import VqeRequest, VqeServer, make_trace, replay


class _FakeEst:
    def __init__(self, n):
        self.n = n

    def grad_from_slots(self, sv):
        return np.asarray(sv) * 2


class _FakeServer(VqeServer):
    """Device work replaced by tickets that complete after `delay` polls."""

    def __init__(self, delay=2, **kw):
        kw.setdefault("compile_workers", 0)
        kw.setdefault("estimator_factory", lambda r, d, dev: _FakeEst(r.n))
        super().__init__(device="cpu", **kw)
        self.delay = delay
        self.max_concurrent = 0

    def _launch(self, sess, req, si):
        if sess.est is None:
            sess.est = self.factory(req, self.dtype, self.device)
        self.max_concurrent = max(self.max_concurrent, len(self.inflight) + 1)
        ticket = {"left": self.delay}
        e_h = torch.tensor([float(req.n)], dtype=torch.float64)
        sv_h = torch.ones(3, dtype=torch.float64) if req.grad else None
        return ticket, e_h, sv_h

    def _ready(self, ticket):
        ticket["left"] -= 1
        return ticket["left"] < 0

    def _footprint(self, req):
        # admission logic under test: states only (psi, plus lam for gradients)
        return (2 if req.grad else 1) * (8 << req.n)


def _req(session, n, grad=False):
    return VqeRequest(session, n, [], 3, None, np.zeros(3), grad)


def test_admission_respects_budget_and_overlaps_requests():
    S = 8
    srv = _FakeServer(hbm_budget=3 * (S << 12), streams=[None] * 4)
    for k in range(6):
        srv.submit(_req(f"s{k}", 12))
    srv.drain()
    assert len(srv.completed) == 6 and all(r.error is None for r in srv.completed)
    assert srv.max_concurrent == 3  # three 12-qubit sessions fit the budget at once
    assert srv.used <= srv.budget


def test_lru_eviction_and_session_reuse():
    S = 8
    srv = _FakeServer(hbm_budget=2 * (S << 10), streams=[None] * 2)
    srv.submit(_req("a", 10))
    srv.drain()
    srv.submit(_req("b", 10))
    srv.drain()
    assert set(srv.sessions) == {"a", "b"}
    srv.submit(_req("c", 10))  # evicts the least recently used idle session ("a")
    srv.drain()
    assert set(srv.sessions) == {"b", "c"}
    est_b = srv.sessions["b"].est
    srv.submit(_req("b", 10))  # resident session reused, no new estimator
    srv.drain()
    assert srv.sessions["b"].est is est_b


def test_same_session_runs_in_order_and_gradients_complete():
    srv = _FakeServer(hbm_budget=1 << 30, streams=[None] * 4)
    reqs = [_req("s", 8, grad=(k % 2 == 0)) for k in range(5)]
    for r in reqs:
        srv.submit(r)
    srv.drain()
    assert srv.max_concurrent == 1  # one session -> serialized
    times = [r.admitted for r in reqs]
    assert times == sorted(times)
    for k, r in enumerate(reqs):
        assert (r.gradient is not None) == (k % 2 == 0)


def test_oversized_request_is_rejected_not_hung():
    srv = _FakeServer(hbm_budget=1 << 10, streams=[None])
    r = _req("big", 20, grad=True)
    srv.submit(r)
    srv.drain(timeout=5)
    assert r.error is not None and "budget" in r.error


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix():
    """Library kernels only (specialise=False): the mix changes no bit.  With
    specialised kernels a session switches kernels once they are compiled, so
    results then agree within the complex64 tolerance (next test)."""
    trace = make_trace(16, rate=1e6, seed=3, n_range=(10, 17), depth_range=(2, 4), terms_range=(20, 120),
                       grad_fraction=0.5, iterations=2)
    alone = {}
    srv1 = VqeServer(max_inflight=1, specialise=False)
    for r in trace:
        rr = VqeRequest(r.session, r.n, r.structure, r.n_params, r.H, r.theta, r.grad)
        srv1.submit(rr)
        srv1.drain()
        alone[id(r)] = rr
    srv = VqeServer(max_inflight=8, specialise=False)
    stats = replay(srv, trace)
    assert stats["errors"] == 0
    for r in trace:
        a = alone[id(r)]
        # FP64 accumulation in a fixed order: the mix changes nothing (tolerance 1e-9 absolute)
        assert abs(r.energy - a.energy) <= 1e-9
        if r.grad:
            np.testing.assert_allclose(r.gradient, a.gradient, atol=1e-9)
    # and against the batched engine / oracle for the energies
    from oracle import sv

    for r in trace[:6]:
        psi, _ = sv.run_ops(r.n, [(nm, *qs) if p is None else (nm, *qs, float(r.theta[p])) for nm, qs, p in r.structure])
        e_ref = sv.pauli_expectation(psi, r.H.codes, r.H.coeffs)
        assert abs(r.energy - e_ref) < 1e-5 * r.H.one_norm()


@pytest.mark.gpu
def test_specialised_sessions_match_the_oracle():
    """Sessions whose kernels are compiled while they serve: every request of
    a trace (three optimizer steps per session, 14-18 qubits, half with
    gradients) against the oracle, complex64 tolerances (1e-5 absolute energies,
    1e-4 gradients), and the kernels in place by the end."""
    from oracle import sv

    trace = make_trace(12, rate=1e6, seed=8, n_range=(14, 18), depth_range=(2, 3), terms_range=(20, 80),
                       grad_fraction=0.5, iterations=3)
    srv = VqeServer(max_inflight=4)
    stats = replay(srv, trace)
    assert stats["errors"] == 0
    for sess in srv.sessions.values():
        if sess.jit is not None:
            assert sess.jit.result() > 0
    for r in trace:
        gates = [(nm, list(qs), p, 1.0) for nm, qs, p in r.structure]
        e_ref, g_ref = sv.grad_adjoint(r.n, gates, r.theta, r.H.codes, r.H.coeffs)
        assert abs(r.energy - e_ref) < 1e-5
        if r.grad:
            np.testing.assert_allclose(r.gradient, g_ref, atol=1e-4)


def test_footprint_counts_tables_workspace_and_partials():
    """The admission footprint of a gradient session covers psi, lam, the op and
    Pauli tables, the tiled H psi workspace and the reverse-sweep partials."""
    from tyxonq_gb300.adjoint import TILE_OP_RECORD_BYTES, estimate_footprint
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.workloads import hea_rz_ops_params

    n = 20
    H = random_pauli_sum(n, 500, np.random.default_rng(1))
    struct = hea_rz_ops_params(n, 4)
    n_param = sum(1 for _, _, p in struct if p is not None)
    e = estimate_footprint(n, len(struct), n_param, H.n_groups, H.n_terms, False, torch.complex64)
    g = estimate_footprint(n, len(struct), n_param, H.n_groups, H.n_terms, True, torch.complex64)
    states = 8 << n
    tables = 2 * len(struct) * TILE_OP_RECORD_BYTES + 16 * H.n_groups + 32 * H.n_terms
    partials = 8 * n_param * (1 << (n - 13))
    assert e > states + tables  # plus the H psi workspace
    assert g - e == states + partials
    srv = VqeServer(device="cpu", hbm_budget=1 << 40, streams=[None])
    req = VqeRequest("s", n, struct, n_param, H, np.zeros(n_param), True)
    assert srv._footprint(req) == g


def test_slow_estimator_builds_do_not_block_other_requests():
    """A new session's estimator is built on the compile worker: a request of a
    resident session admitted meanwhile completes before the slow build ends."""
    import threading

    gate = threading.Event()

    def factory(req, dtype, device):
        if req.session == "slow":
            gate.wait(5)
        return _FakeEst(req.n)

    srv = _FakeServer(hbm_budget=1 << 30, streams=[None] * 4, compile_workers=1, estimator_factory=factory)
    srv.submit(_req("fast", 8))
    srv.drain()  # "fast" is resident now
    slow, fast = _req("slow", 8), _req("fast", 8)
    srv.submit(slow)
    srv.submit(fast)
    for _ in range(200):
        srv.step()
        if fast.done is not None:
            break
    assert fast.done is not None and slow.done is None  # not blocked by the build
    gate.set()
    srv.drain()
    assert slow.error is None and slow.energy == 8.0



class _FakeBatcher:
    """Micro-batch device work replaced by tickets (energy = n, gradient = 2 theta)."""

    def __init__(self, res_max=12, delay=1):
        self.res_max, self.delay = res_max, delay
        self.sessions = {}
        self.launched = []

    def fits(self, n):
        return n <= self.res_max

    def table_bytes(self, n, n_gates, n_groups, n_terms):
        return 1000

    def register(self, key, n, structure, n_params, H):
        self.sessions[key] = n
        return n

    def release_retired(self):
        pass

    def launch(self, items, stream):
        self.launched.append([k for k, _ in items])
        return {"event": {"left": self.delay}, "res": [(float(self.sessions[k]), np.asarray(t) * 2) for k, t in items]}

    @staticmethod
    def results(ticket):
        return ticket["res"]


def test_small_requests_are_coalesced_across_sessions():
    """Waiting small requests of different sessions share one micro-batch;
    requests of one session stay in order (one per batch); each request gets
    its own results; large requests keep their own streams."""
    srv = _FakeServer(hbm_budget=1 << 30, streams=[None] * 4, delay=1)
    srv.batcher = _FakeBatcher()
    reqs = []
    for k in range(6):
        r = VqeRequest(f"s{k}", 10 + (k % 3), [], 3, None, np.arange(3.0) + k, grad=(k % 2 == 0))
        reqs.append(r)
    reqs += [VqeRequest("s0", 10, [], 3, None, np.ones(3), grad=True)]  # second request of s0
    big = _req("big", 16, grad=True)
    for r in reqs + [big]:
        srv.submit(r)
    srv.drain()
    assert all(r.error is None and r.done is not None for r in reqs + [big])
    first = srv.batcher.launched[0]
    assert sorted(first) == sorted(f"s{k}" for k in range(6))  # one launch for six sessions
    assert srv.batcher.launched[1] == ["s0"]  # the same session's next request: the next batch
    assert srv.batch_sizes == [6, 1]
    for r in reqs:
        assert r.energy == float(r.n)
        if r.grad:
            np.testing.assert_array_equal(r.gradient, np.asarray(r.theta) * 2)
        else:
            assert r.gradient is None
    assert big.energy == 16.0  # through the per-request path
    assert srv.used <= srv.budget


@pytest.mark.gpu
def test_coalesced_small_requests_match_the_oracle():
    """Small requests (8-12 qubits) of many sessions evaluated in shared
    micro-batches: every energy and gradient against the oracle (complex64
    tolerances), and fewer launches than requests."""
    from oracle import sv

    trace = make_trace(48, rate=1e6, seed=11, n_range=(8, 12), depth_range=(2, 4), terms_range=(20, 120),
                       grad_fraction=0.5, iterations=2)
    srv = VqeServer(max_inflight=4)
    assert srv.batcher is not None
    stats = replay(srv, trace)
    assert stats["errors"] == 0
    assert stats["batched_requests"] == len(trace)
    assert stats["micro_batches"] < len(trace)
    for r in trace:
        gates = [(nm, list(qs), p, 1.0) for nm, qs, p in r.structure]
        e_ref, g_ref = sv.grad_adjoint(r.n, gates, r.theta, r.H.codes, r.H.coeffs)
        assert abs(r.energy - e_ref) < 1e-5
        if r.grad:
            np.testing.assert_allclose(r.gradient, g_ref, atol=1e-4)
        else:
            assert r.gradient is None


def test_table_arena_appends_grows_and_keeps_retired_buffers():
    """The micro-batch table arena (host and device copies, device "cpu" here):
    appends return consecutive offsets, growth doubles the capacity, keeps the
    contents and hands the replaced device buffer to the retired list."""
    from tyxonq_gb300.coalesce import _Arena
    from tyxonq_gb300.hamiltonian import TERM_DTYPE

    ar = _Arena(TERM_DTYPE, torch.device("cpu"), capacity=4)
    retired = []
    a = np.zeros(3, dtype=TERM_DTYPE)
    a["zy"] = [1, 2, 3]
    b = np.zeros(4, dtype=TERM_DTYPE)
    b["zy"] = [4, 5, 6, 7]
    assert ar.append(a, retired) == 0 and retired == []
    old = ar.dev
    assert ar.append(b, retired) == 3
    assert len(retired) == 1 and retired[0] is old and len(ar.host) == 8
    dev = np.frombuffer(ar.dev.numpy().tobytes(), dtype=TERM_DTYPE)
    assert list(dev["zy"][:7]) == [1, 2, 3, 4, 5, 6, 7]
    assert list(ar.host["zy"][:7]) == [1, 2, 3, 4, 5, 6, 7]
    assert ar.append(np.zeros(0, dtype=TERM_DTYPE), retired) == 7 and ar.size == 7
