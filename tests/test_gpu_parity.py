"""GPU parity: CUDA path (through the C ABI) against the oracle and the
reference's golden vectors.

Tolerances: complex128 amplitudes / energies 1e-12 (spec bar);
complex64 amplitudes 2e-6 * sqrt(gates) and energies 1e-5 relative to the
Hamiltonian's 1-norm (FP32 state, FP64 accumulation).  Bit layout (basis
ordering, bitstrings, sampled indices) is compared exactly.
"""
import math

import numpy as np
import pytest
import torch

from oracle import sv
from tests import golden_data

pytestmark = pytest.mark.gpu

C64, C128 = torch.complex64, torch.complex128


def _engine(dtype, fusion):
    from tyxonq_gb300.engine import GpuStatevectorEngine

    return GpuStatevectorEngine(dtype=dtype, fusion=fusion)


class _C:
    def __init__(self, n, ops, ucache=None):
        self.num_qubits = n
        self.ops = ops
        self._unitary_cache = ucache or {}


@pytest.mark.parametrize("fusion", ["plain", "fused"])
@pytest.mark.parametrize("case", golden_data.circuit_cases(), ids=lambda c: c[0])
def test_golden_states_c128(case, fusion):
    name, n, ops, ucache, ref_state, ref_z = case
    eng = _engine(C128, fusion)
    psi = eng.state(_C(n, ops, ucache)).cpu().numpy()
    np.testing.assert_allclose(psi, ref_state, atol=1e-12, rtol=0)
    out = eng.run(_C(n, list(ops) + [("measure_z", q) for q in range(n)], ucache), shots=0)
    z = [out["expectations"][f"Z{q}"] for q in range(n)]
    np.testing.assert_allclose(z, ref_z, atol=1e-12, rtol=0)


@pytest.mark.parametrize("fusion", ["plain", "fused"])
@pytest.mark.parametrize("case", golden_data.circuit_cases(), ids=lambda c: c[0])
def test_golden_states_c64(case, fusion):
    name, n, ops, ucache, ref_state, ref_z = case
    psi = _engine(C64, fusion).state(_C(n, ops, ucache)).cpu().numpy()
    tol = 2e-6 * math.sqrt(len(ops) + 1)
    np.testing.assert_allclose(psi, ref_state, atol=tol, rtol=0)


@pytest.mark.parametrize("dtype,tol", [(C128, 1e-13), (C64, 2e-6)])
def test_golden_kqubit_unitary(dtype, tol):
    from tyxonq_gb300 import kernels as K

    arrays, meta = golden_data.load()
    for c in meta["kq"]:
        k = c["k"]
        psi = K.from_array(arrays[f"kq{k}_in"], dtype=dtype)
        K.apply_kq(psi, arrays[f"kq{k}_u"], c["qubits"])
        np.testing.assert_allclose(psi.cpu().numpy(), arrays[f"kq{k}_out"], atol=tol, rtol=0)


@pytest.mark.parametrize("dtype", [C128, C64])
def test_golden_pauli_energy_and_hpsi(dtype):
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.hamiltonian import PauliSum

    arrays, meta = golden_data.load()
    for c in meta["pauli"]:
        nm = c["name"]
        H = PauliSum.from_codes(arrays[f"{nm}_codes"], arrays[f"{nm}_w"])
        psi = K.from_array(arrays[f"{nm}_psi"], dtype=dtype)
        e = float(K.pauli_expectation(psi, H).item())
        tol = 1e-12 if dtype == C128 else 1e-5 * H.one_norm()
        assert abs(e - c["energy"]) < tol
        hp = K.apply_pauli_sum(psi, H).cpu().numpy()
        np.testing.assert_allclose(hp, arrays[f"{nm}_hpsi"], atol=1e-12 if dtype == C128 else 1e-5 * H.one_norm())


def _hea12_pgates():
    from tyxonq_gb300.adjoint import ParamGate
    from tyxonq_gb300.ir import Gate, _rot_gate

    pg = []
    for l in range(4):
        for q in range(12):
            pg.append(ParamGate(_rot_gate("ry", (q,), 0.0), l * 12 + q))
        for q in range(11):
            pg.append(ParamGate(Gate("cx", (q, q + 1))))
    return pg


@pytest.mark.parametrize("dtype", [C128, C64])
def test_hea12_energy_and_adjoint_gradient(dtype):
    from tyxonq_gb300.adjoint import AdjointEstimator
    from tyxonq_gb300.hamiltonian import PauliSum

    arrays, meta = golden_data.load()
    H = PauliSum.from_codes(arrays["hea12_codes"], arrays["hea12_w"])
    est = AdjointEstimator(12, _hea12_pgates(), 48, H, dtype=dtype)
    theta = arrays["hea12_theta"].reshape(-1)
    e, g = est.energy_and_grad(theta)
    e_tol = 1e-12 if dtype == C128 else 1e-5
    assert abs(e - 0.1195334104542979) < e_tol
    assert abs(est.energy(theta) - meta["hea12"]["energy_numpy"]) < e_tol
    g_tol = 1e-10 if dtype == C128 else 1e-4
    np.testing.assert_allclose(g, arrays["hea12_grad_autograd"].reshape(-1), atol=g_tol)


def test_adjoint_matches_fd_and_parameter_shift_with_all_rotation_kinds():
    from tyxonq_gb300.adjoint import AdjointEstimator, ParamGate
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.ir import Gate, _rot_gate, pauli_rotation

    rng = np.random.default_rng(7)
    n = 9
    H = random_pauli_sum(n, 40, rng)
    pg, ops_spec = [], []
    p = 0
    for q in range(n):
        for nm in ("rx", "ry", "rz"):
            pg.append(ParamGate(_rot_gate(nm, (q,), 0.0), p))
            ops_spec.append((nm, (q,), p))
            p += 1
    for q in range(n - 1):
        nm = ("rxx", "ryy", "rzz")[q % 3]
        pg.append(ParamGate(_rot_gate(nm, (q, q + 1), 0.0), p))
        ops_spec.append((nm, (q, q + 1), p))
        p += 1
        pg.append(ParamGate(Gate("cx", (q, (q + 2) % n))))
        ops_spec.append(("cx", (q, (q + 2) % n), None))
    pauli = ((0, "X"), (3, "Y"), (5, "Z"), (8, "X"))
    pg.append(ParamGate(pauli_rotation(pauli, 0.0), p, 2.0))
    ops_spec.append(("prot", pauli, p))
    p += 1
    theta = rng.uniform(0, 2 * np.pi, p)
    est = AdjointEstimator(n, pg, p, H, dtype=C128)
    e, g = est.energy_and_grad(theta)

    def ops_fn(th):
        ops = []
        for nm, qs, pi in ops_spec:
            if nm == "prot":
                # evolve_pauli_ops structure of exp(-i a/2 P), a = 2 theta (utils.py:29-59)
                a = 2.0 * th[pi]
                for q, s in qs:
                    if s == "X":
                        ops.append(("h", q))
                    elif s == "Y":
                        ops += [("sdg", q), ("h", q)]
                for i in range(len(qs) - 1):
                    ops.append(("cx", qs[i][0], qs[i + 1][0]))
                ops.append(("rz", qs[-1][0], a))
                for i in reversed(range(len(qs) - 1)):
                    ops.append(("cx", qs[i][0], qs[i + 1][0]))
                for q, s in qs:
                    if s == "X":
                        ops.append(("h", q))
                    elif s == "Y":
                        ops += [("h", q), ("s", q)]
            elif pi is None:
                ops.append((nm, *qs))
            else:
                ops.append((nm, *qs, float(th[pi])))
        return ops

    e_or = sv.energy(n, ops_fn, theta, H.codes, H.coeffs)
    assert abs(e - e_or) < 1e-12
    gfd = sv.grad_central_fd(n, ops_fn, theta, H.codes, H.coeffs, h=1e-4)
    np.testing.assert_allclose(g, gfd, atol=1e-6)
    gps = sv.grad_param_shift(n, ops_fn, theta, H.codes, H.coeffs)
    # the last parameter enters as 2*theta, outside the two-term shift rule
    np.testing.assert_allclose(g[:-1], gps[:-1], atol=1e-10)


@pytest.mark.parametrize("n,depth,dtype", [(16, 12, C128), (20, 20, C64), (22, 10, C64)])
def test_random_circuits_fused_vs_plain_vs_oracle(n, depth, dtype):
    from tyxonq_gb300.workloads import random_circuit

    ops = random_circuit(n, depth, seed=n + depth)
    c = _C(n, ops)
    a = _engine(dtype, "fused").state(c)
    b = _engine(dtype, "plain").state(c)
    ref, _ = sv.run_ops(n, ops, mode="state")
    tol = 1e-12 if dtype == C128 else 2e-6 * math.sqrt(len(ops))
    np.testing.assert_allclose(a.cpu().numpy(), ref, atol=tol, rtol=0)
    np.testing.assert_allclose(b.cpu().numpy(), ref, atol=tol, rtol=0)


def test_probabilities_ordering_and_sampling_chi2():
    from tyxonq_gb300 import kernels as K

    eng = _engine(C128, "fused")
    c = _C(2, [("h", 0)])
    p = eng.probability(c).cpu().numpy()
    assert abs(p[0] + p[2] - 1) < 1e-12  # big-endian (test_statevector_engine_probs.py:15-17)
    assert abs(eng.amplitude(c, "01")) < 1e-12
    bits, prob = eng.perfect_sampling(c, rng=np.random.default_rng(0))
    assert bits in ("00", "10") and abs(prob - 0.5) < 1e-12
    ops = [("h", 0), ("ry", 1, 0.3), ("cx", 0, 2), ("rx", 3, 1.1), ("ry", 4, 2.2), ("cx", 4, 5), ("h", 6)]
    n = 7
    psi_ref, _ = sv.run_ops(n, ops)
    for dtype in (C64, C128):
        out = _engine(dtype, "fused").run(_C(n, ops + [("measure_z", q) for q in range(n)]), shots=200000, seed=123)
        counts = out["result"]
        assert sum(counts.values()) == 200000
        for b in counts:
            assert len(b) == n and psi_ref[int(b, 2)] != 0
        assert sv.chi2_pvalue(counts, sv.probabilities(psi_ref)) > 1e-4
    # seeded sampler is deterministic and indices are sorted
    psi = K.from_array(psi_ref, dtype=C64)
    s1 = K.sample(psi, 5000, 99).cpu().numpy()
    s2 = K.sample(psi, 5000, 99).cpu().numpy()
    assert (s1 == s2).all() and (np.diff(s1) >= 0).all()


def test_expect_z_all_and_projection():
    eng = _engine(C128, "plain")
    out = eng.run(_C(2, [("h", 0), ("project_z", 0, 0), ("reset", 1), ("measure_z", 0), ("measure_z", 1)]))
    assert abs(out["expectations"]["Z0"] - 1) < 1e-12 and abs(out["expectations"]["Z1"] - 1) < 1e-12
    rng = np.random.default_rng(1)
    for n in (1, 3, 9, 14, 17):
        ops = [("ry", q, float(rng.uniform(0, 6))) for q in range(n)] + [("cx", q, q + 1) for q in range(n - 1)]
        out = _engine(C128, "fused").run(_C(n, ops + [("measure_z", q) for q in range(n)]), shots=0)
        ref, _ = sv.run_ops(n, ops)
        for q in range(n):
            assert abs(out["expectations"][f"Z{q}"] - sv.expect_z(ref, q, n)) < 1e-12


def test_28q_fused_circuit_then_inverse_is_identity():
    """Full-size property check (28 qubits, complex64): U then U^dagger returns
    |0...0> and the norm stays 1."""
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward
    from tyxonq_gb300.workloads import random_circuit

    n = 28
    ops = random_circuit(n, 40, seed=1)
    gates, _ = lower_ops(_C(n, ops), mode="run")
    inv = []
    for g in reversed(gates):
        from tyxonq_gb300.ir import Gate

        if g.kind in ("cx", "cz", "swap"):
            inv.append(g)
        else:
            inv.append(Gate(g.kind, g.qubits, np.conj(g.mat).T))
    psi = K.init_statevector(n, dtype=C64)
    compile_forward(gates, n, C64).run(psi)
    nrm = float(K.norm2(psi).item())
    assert abs(nrm - 1) < 1e-5
    compile_forward(inv, n, C64).run(psi)
    a0 = psi[0].item()
    assert abs(abs(a0) - 1) < 1e-4
    assert abs(float(K.norm2(psi).item()) - 1) < 1e-5
    del psi
    torch.cuda.empty_cache()


def test_autograd_state_matches_reference_gradient():
    from tyxonq_gb300.engine import GpuStatevectorEngine

    arrays, meta = golden_data.load()
    theta = torch.tensor(arrays["hea12_theta"], dtype=torch.float64, device="cuda", requires_grad=True)
    ops = []
    for l in range(4):
        for q in range(12):
            ops.append(("ry", q, theta[l, q]))
        for q in range(11):
            ops.append(("cx", q, q + 1))
    eng = GpuStatevectorEngine(dtype=C128)
    psi = eng.state(_C(12, ops))
    Hd = torch.as_tensor(sv.dense_hamiltonian(arrays["hea12_codes"], arrays["hea12_w"]), device="cuda")
    e = torch.real(torch.conj(psi) @ (Hd @ psi))
    e.backward()
    assert abs(e.item() - 0.1195334104542979) < 1e-12
    np.testing.assert_allclose(theta.grad.cpu().numpy(), arrays["hea12_grad_autograd"], atol=1e-10)


@pytest.mark.parametrize("n", [12, 14, 17])
@pytest.mark.parametrize("dtype", [C128, C64])
def test_tiled_pauli_sum_matches_oracle_and_sweep_kernels(n, dtype):
    """tq_sv_pauli_sum_tiled (H psi and <H> of one state through the wave H psi
    kernel, group slices summed in order) against the oracle and against the
    one-amplitude-per-thread kernels: a random Pauli sum (about one term per
    flip group) and a molecular Jordan-Wigner H (many terms per group, class
    sums + Walsh-Hadamard transform), energy only, and no terms."""
    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import chem
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.hamiltonian import PauliSum, random_pauli_sum

    rng = np.random.default_rng(n)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    psi = K.from_array(v, dtype=dtype)
    hs = [random_pauli_sum(n, 300, rng)]
    if n in (12, 14):
        h1, h2 = chem.random_integrals(n // 2, seed=1)
        hs.append(chem.molecular_hamiltonian(h1, h2))
    for H in hs:
        nrm = H.one_norm()
        e_ref = sv.pauli_expectation(v, H.codes, H.coeffs)
        hp_ref = sv.apply_pauli_sum(v, H.codes, H.coeffs)
        tol_e = 1e-11 * max(1.0, nrm) if dtype == C128 else 1e-5 * nrm
        tol_v = 1e-11 * max(1.0, nrm) if dtype == C128 else 1e-5 * nrm
        out = torch.empty_like(psi)
        e_dev = torch.empty(1, dtype=torch.float64, device="cuda")
        K._pauli_sum_tiled(psi, H, n, out, e_dev)
        np.testing.assert_allclose(out.cpu().numpy(), hp_ref, atol=tol_v)
        assert abs(float(e_dev.item()) - e_ref) < tol_e
        e_only = torch.empty(1, dtype=torch.float64, device="cuda")
        K._pauli_sum_tiled(psi, H, n, None, e_only)
        assert float(e_only.item()) == float(e_dev.item())  # same items, same order
        # the sweep kernels (one amplitude per thread / one sweep per group)
        gd, td, ng, nt = H.to_device(psi.device)
        out2 = torch.empty_like(psi)
        nat.call("tq_sv_apply_pauli_sum", K._ptr(psi), K._ptr(out2), n, K.dtype_tag(psi), K._ptr(gd), ng,
                 K._ptr(td), nt, K.stream_ptr())
        np.testing.assert_allclose(out.cpu().numpy(), out2.cpu().numpy(), atol=tol_v)
        # replays are bit-identical
        out3 = torch.empty_like(psi)
        K._pauli_sum_tiled(psi, H, n, out3, None)
        assert torch.equal(out3, out)
    empty = PauliSum.from_codes(np.zeros((0, n), dtype=np.int64), np.zeros(0))
    out = torch.ones_like(psi)
    e_dev = torch.ones(1, dtype=torch.float64, device="cuda")
    K._pauli_sum_tiled(psi, empty, n, out, e_dev)
    assert float(e_dev.item()) == 0.0 and not bool(out.abs().any())


@pytest.mark.parametrize("dtype", [C128, C64])
def test_staged_single_state_reverse_sweep_matches_tile_passes(dtype, monkeypatch):
    """ParametricEstimator from 14 qubits runs its reverse sweep as register-
    staged wave adjoint passes (one-instance plan).  Against the shared-memory
    tile-pass sweep (forced by raising the size threshold) and the oracle's
    central differences, on every rotation kind, fixed gates, a scaled
    multi-qubit Pauli rotation with Z strings and a phase gate."""
    import tyxonq_gb300.adjoint as A
    from tyxonq_gb300.adjoint import ParamGate, ParametricEstimator
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.ir import Gate, _rot_gate, pauli_rotation

    rng = np.random.default_rng(11)
    n = 14
    H = random_pauli_sum(n, 120, rng)
    pg, p = [], 0
    for layer in range(3):
        for q in range(n):
            nm = ("rx", "ry", "rz")[(q + layer) % 3]
            pg.append(ParamGate(_rot_gate(nm, (q,), 0.0), p))
            p += 1
        for q in range(layer % 2, n - 1, 2):
            pg.append(ParamGate(Gate("cx", (q, q + 1))))
        pg.append(ParamGate(_rot_gate("rzz", (0, n - 1), 0.0), p))
        p += 1
        pg.append(ParamGate(Gate("cz", (2, 9))))
        pg.append(ParamGate(pauli_rotation(((1, "X"), (4, "Z"), (7, "Y"), (12, "Z")), 0.0), p, 2.0))
        p += 1
    theta = rng.uniform(0, 2 * np.pi, p)
    staged = ParametricEstimator(n, pg, p, H, dtype=dtype)
    e_only = staged.energy(theta)  # energy alone does not build the staged sweep
    assert staged._staged is None
    e, g = staged.energy_and_grad(theta)
    assert staged._staged is not None
    assert abs(e_only - e) < (1e-12 if dtype == C128 else 1e-5 * H.one_norm())
    monkeypatch.setattr(A, "STAGED_ADJOINT_MIN_N", 99)
    tiles = ParametricEstimator(n, pg, p, H, dtype=dtype)
    e2, g2 = tiles.energy_and_grad(theta)
    assert tiles._staged is None
    nrm = H.one_norm()
    tol = 1e-10 if dtype == C128 else 2e-4 * nrm
    assert abs(e - e2) < (1e-12 if dtype == C128 else 1e-5 * nrm)
    np.testing.assert_allclose(g, g2, atol=tol)
    # repeated calls give identical results (fixed-order reductions)
    e3, g3 = staged.energy_and_grad(theta)
    assert e3 == e and np.array_equal(g3, g)
    if dtype == C128:  # central differences through the same engine's energies
        for k in rng.choice(p, 6, replace=False):
            tp, tm = theta.copy(), theta.copy()
            tp[k] += 1e-4
            tm[k] -= 1e-4
            fd = (staged.energy(tp) - staged.energy(tm)) / 2e-4
            assert abs(fd - g[k]) < 1e-6, (k, fd, g[k])


@pytest.mark.parametrize("dtype", [C128, C64])
def test_tiled_pauli_sum_general_complex_weights(dtype):
    """tq_sv_pauli_sum_tiled with term weights that are neither real nor
    imaginary (the C tables accept any complex weight): groups of one term,
    of a few terms and of many terms (the class-sum path), against
    (H psi)_i = sum_t w_t (-1)^popc((i ^ flip) & zy_t) psi_(i ^ flip) on the host."""
    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.hamiltonian import random_pauli_sum, sort_terms_by_class

    n = 14
    rng = np.random.default_rng(21)
    H = random_pauli_sum(n, 200, rng)
    g, t = H.pack()
    t = sort_terms_by_class(g, t, 12).copy()
    # one group with many terms: the diagonal group (flip 0) gets extra Z strings
    extra = np.zeros(9, dtype=t.dtype)
    extra["zy"] = rng.integers(1, 1 << n, size=9, dtype=np.uint64)
    g0 = g.copy()
    if len(g0) == 0 or g0[0]["flip"] != 0:  # no diagonal group yet: add one in front
        g0 = np.concatenate([np.zeros(1, dtype=g0.dtype), g0])
    t = np.concatenate([t[:g0[0]["n_terms"]], extra, t[g0[0]["n_terms"]:]])
    g0["first_term"][1:] += len(extra)
    g0[0]["n_terms"] += len(extra)
    t = sort_terms_by_class(g0, t, 12).copy()
    phase = np.exp(1j * rng.uniform(0, 2 * np.pi, len(t)))
    w = (np.where(t["w_re"] != 0, t["w_re"], 0.3) + 1j * t["w_im"]) * phase
    t["w_re"], t["w_im"] = w.real, w.imag
    t["f_re"], t["f_im"] = w.real, w.imag
    assert (np.abs(w.real) > 0).all() and (np.abs(w.imag) > 0).all()
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    idx = np.arange(1 << n, dtype=np.uint64)
    ref = np.zeros(1 << n, dtype=np.complex128)
    for gi in range(len(g0)):
        m = np.uint64(g0[gi]["flip"])
        src = idx ^ m
        for k in range(g0[gi]["first_term"], g0[gi]["first_term"] + g0[gi]["n_terms"]):
            x = src & np.uint64(t[k]["zy"])
            for sh in (32, 16, 8, 4, 2, 1):
                x ^= x >> np.uint64(sh)
            par = x & np.uint64(1)
            ref += w[k] * np.where(par == 1, -1.0, 1.0) * v[src.astype(np.int64)]
    psi = K.from_array(v, dtype=dtype)
    out = torch.empty_like(psi)
    e_dev = torch.empty(1, dtype=torch.float64, device="cuda")
    gd = torch.from_numpy(np.frombuffer(g0.tobytes(), dtype=np.uint8).copy()).cuda()
    td = torch.from_numpy(np.frombuffer(t.tobytes(), dtype=np.uint8).copy()).cuda()
    lib = nat.load()
    dt = K.dtype_tag(psi)
    ws = torch.empty(int(lib.tq_sv_pauli_sum_tiled_workspace_bytes(n, dt, len(g0), 1)), dtype=torch.uint8,
                     device="cuda")
    nat.call("tq_sv_pauli_sum_tiled", K._ptr(psi), K._ptr(out), n, dt, K._ptr(gd), len(g0), K._ptr(td), len(t),
             K._ptr(e_dev), K._ptr(ws), ws.numel(), K.stream_ptr(psi.device))
    torch.cuda.synchronize()
    nrm = float(np.abs(w).sum())
    tol = 1e-11 * nrm if dtype == C128 else 1e-5 * nrm
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=tol)
    assert abs(float(e_dev.item()) - float(np.vdot(v, ref).real)) < tol
