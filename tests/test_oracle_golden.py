"""The CPU oracle reproduces the reference's own outputs (golden vectors) and
the known answers of the reference's tests.  CPU only."""
import math

import numpy as np
import pytest

from oracle import sv
from tests import golden_data


@pytest.mark.parametrize("case", golden_data.circuit_cases(), ids=lambda c: c[0])
def test_state_and_run_z(case):
    name, n, ops, ucache, ref_state, ref_z = case
    psi, _ = sv.run_ops(n, ops, mode="state", unitary_cache=ucache)
    np.testing.assert_allclose(psi, ref_state, atol=1e-12, rtol=0)
    psi_run, _ = sv.run_ops(n, ops, mode="run", unitary_cache=ucache)
    z = [sv.expect_z(psi_run, q, n) for q in range(n)]
    np.testing.assert_allclose(z, ref_z, atol=1e-12, rtol=0)


def test_kqubit_unitary():
    arrays, meta = golden_data.load()
    for c in meta["kq"]:
        k = c["k"]
        out = sv.apply_kq(arrays[f"kq{k}_in"], arrays[f"kq{k}_u"], c["qubits"], c["n"])
        np.testing.assert_allclose(out, arrays[f"kq{k}_out"], atol=1e-13, rtol=0)


def test_pauli_energy_and_hpsi():
    arrays, meta = golden_data.load()
    for c in meta["pauli"]:
        nm = c["name"]
        codes, w, psi = arrays[f"{nm}_codes"], arrays[f"{nm}_w"], arrays[f"{nm}_psi"]
        assert abs(sv.pauli_expectation(psi, codes, w) - c["energy"]) < 1e-12
        np.testing.assert_allclose(sv.apply_pauli_sum(psi, codes, w), arrays[f"{nm}_hpsi"], atol=1e-12)


def hea12_ops(theta):
    n, L = 12, 4
    ops = []
    for l in range(L):
        for q in range(n):
            ops.append(("ry", q, float(theta[l * n + q])))
        for q in range(n - 1):
            ops.append(("cx", q, q + 1))
    return ops


def test_hea12_energy_and_autograd_gradient():
    arrays, meta = golden_data.load()
    theta = arrays["hea12_theta"].reshape(-1)
    codes, w = arrays["hea12_codes"], arrays["hea12_w"]
    psi, _ = sv.run_ops(12, hea12_ops(theta))
    np.testing.assert_allclose(psi, arrays["hea12_state"], atol=1e-12, rtol=0)
    e = sv.pauli_expectation(psi, codes, w)
    assert abs(e - 0.1195334104542979) < 1e-12
    assert abs(e - meta["hea12"]["energy_pytorch"]) < 1e-12
    gates = []
    for l in range(4):
        for q in range(12):
            gates.append(("ry", [q], l * 12 + q, 1.0))
        for q in range(11):
            gates.append(("cx", [q, q + 1], None, 1.0))
    e2, g = sv.grad_adjoint(12, gates, theta, codes, w)
    assert abs(e2 - e) < 1e-12
    np.testing.assert_allclose(g, arrays["hea12_grad_autograd"].reshape(-1), atol=1e-10)


def test_reference_known_answers():
    # Bell: <Z>=0, norm 1 (test_devices_simulators_gates.py:17-30)
    psi, _ = sv.run_ops(2, [("h", 0), ("cx", 0, 1)])
    assert abs(np.vdot(psi, psi) - 1) < 1e-12
    assert abs(sv.expect_z(psi, 0, 2)) < 1e-12
    # big-endian: h(0) on 2 qubits -> p[0] + p[2] = 1 (test_statevector_engine_probs.py:15-17)
    p = sv.probabilities(sv.run_ops(2, [("h", 0)])[0])
    assert abs(p[0] + p[2] - 1) < 1e-12
    # <X> on |+> = 1; ZZ, XX on Bell = 1; TFIM |+++> = -3 (test_circuit_expectation.py)
    plus, _ = sv.run_ops(1, [("h", 0)])
    assert abs(sv.pauli_expectation(plus, np.array([[1]]), np.array([1.0])) - 1) < 1e-10
    assert abs(sv.pauli_expectation(psi, np.array([[3, 3]]), np.array([1.0])) - 1) < 1e-10
    assert abs(sv.pauli_expectation(psi, np.array([[1, 1]]), np.array([1.0])) - 1) < 1e-10
    ppp, _ = sv.run_ops(3, [("h", 0), ("h", 1), ("h", 2)])
    codes, w = sv.terms_to_codes(3, [(-1.0, [("X", i)]) for i in range(3)] + [(1.0, [("Z", 0), ("Z", 1)]), (1.0, [("Z", 1), ("Z", 2)])])
    assert abs(sv.pauli_expectation(ppp, codes, w) + 3) < 1e-10
    # <Z> after RX(0.5) = cos 0.5 (test_circuit_state_autograd.py:84-102)
    r, _ = sv.run_ops(1, [("rx", 0, 0.5)])
    assert abs(sv.expect_z(r, 0, 1) - math.cos(0.5)) < 1e-12
    # projection / reset (test_mid_measure_postselect.py:9-16)
    s, m = sv.run_ops(2, [("h", 0), ("project_z", 0, 0), ("reset", 1), ("measure_z", 0), ("measure_z", 1)], mode="run")
    assert abs(sv.expect_z(s, 0, 2) - 1) < 1e-12 and abs(sv.expect_z(s, 1, 2) - 1) < 1e-12


def test_gradient_oracles_agree():
    rng = np.random.default_rng(5)
    n = 5
    theta = rng.uniform(0, 2 * np.pi, 2 * n)
    from tyxonq_gb300.hamiltonian import random_pauli_sum

    H = random_pauli_sum(n, 20, rng)

    def ops_fn(t):
        ops = [("ry", q, float(t[q])) for q in range(n)]
        ops += [("cx", q, q + 1) for q in range(n - 1)]
        ops += [("rz", q, float(t[n + q])) for q in range(n)]
        return ops

    gates = [("ry", [q], q, 1.0) for q in range(n)] + [("cx", [q, q + 1], None, 1.0) for q in range(n - 1)] + [
        ("rz", [q], n + q, 1.0) for q in range(n)]
    e, g = sv.grad_adjoint(n, gates, theta, H.codes, H.coeffs)
    gfd = sv.grad_central_fd(n, ops_fn, theta, H.codes, H.coeffs)
    gps = sv.grad_param_shift(n, ops_fn, theta, H.codes, H.coeffs)
    np.testing.assert_allclose(g, gps, atol=1e-12)
    np.testing.assert_allclose(g, gfd, atol=1e-7)


def test_chi2_sampler_check_is_sensitive():
    rng = np.random.default_rng(3)
    psi, _ = sv.run_ops(4, [("h", 0), ("ry", 1, 0.3), ("cx", 0, 2), ("rx", 3, 1.1)])
    p = sv.probabilities(psi)
    good = sv.sample_counts(psi, 20000, rng)
    assert sv.chi2_pvalue(good, p) > 1e-4
    # a planted mistake in the oracle side: sample from the wrong distribution
    bad = sv.sample_counts(sv.run_ops(4, [("h", 0), ("ry", 1, 0.5), ("cx", 0, 2), ("rx", 3, 1.1)])[0], 20000, rng)
    assert sv.chi2_pvalue(bad, p) < 1e-6


@pytest.mark.parametrize("case", golden_data.noise_cases(), ids=lambda c: c[0])
def test_kraus_and_noise_against_reference(case):
    """Kraus channels with explicit status and use_noise Z attenuation, against
    the reference engine's own outputs."""
    name, n, ops, kc, state, runz, runz_depol = case
    psi, _ = sv.run_ops(n, ops, mode="state", kraus_cache=kc)
    np.testing.assert_allclose(psi, state, atol=1e-12)
    ops_m = list(ops) + [("measure_z", q) for q in range(n)]
    psi_r, meas = sv.run_ops(n, ops_m, mode="run", kraus_cache=kc)
    z = np.array([sv.expect_z(psi_r, q, n) for q in meas])
    np.testing.assert_allclose(z, runz, atol=1e-12)
    att = sv.z_attenuation(n, ops_m, {"type": "depolarizing", "p": 0.05})
    np.testing.assert_allclose(z * att, runz_depol, atol=1e-12)


def test_noisy_probabilities_readout_and_depolarizing():
    rng = np.random.default_rng(3)
    n = 4
    psi = rng.normal(size=16) + 1j * rng.normal(size=16)
    psi /= np.linalg.norm(psi)
    p = np.abs(psi) ** 2
    cals = {0: np.array([[0.9, 0.2], [0.1, 0.8]]), 2: np.array([[0.95, 0.05], [0.05, 0.95]])}
    pr = sv.noisy_probabilities(psi, n, {"type": "readout", "cals": cals})
    A = np.kron(np.kron(np.kron(cals[0], np.eye(2)), cals[2]), np.eye(2))
    np.testing.assert_allclose(pr, A @ p / (A @ p).sum(), atol=1e-14)
    pd = sv.noisy_probabilities(psi, n, {"type": "depolarizing", "p": 0.3})
    np.testing.assert_allclose(pd, 0.6 * p + 0.4 / 16, atol=1e-14)


@pytest.mark.parametrize("case", golden_data.counts_cases(), ids=lambda c: f"n{c[0]}")
def test_counts_expectation_against_reference(case):
    n, counts, items, energy, expvals = case
    ev = [sv.term_expectation_from_counts(counts, [q for q, _ in t]) for t, _ in items]
    np.testing.assert_allclose(ev, expvals, atol=1e-14)
    assert abs(sv.expval_pauli_sum(counts, items, 0.25) - energy) < 1e-12


def test_parity_expectations_match_counts_rule():
    """The device path reduces parities from sampled indices; same numbers as
    the counts rule on the histogram of those indices."""
    from tyxonq_gb300.shots import parity_expectations

    rng = np.random.default_rng(8)
    n = 7
    idx = np.sort(rng.integers(0, 1 << n, size=3000))
    counts = {}
    for i in idx:
        b = format(int(i), f"0{n}b")
        counts[b] = counts.get(b, 0) + 1
    terms = [((0, "Z"), (3, "X")), ((6, "Y"),), ((1, "Z"), (2, "Z"), (5, "Z"))]
    ev = parity_expectations(idx, terms, n)
    ref = [sv.term_expectation_from_counts(counts, [q for q, _ in t]) for t in terms]
    np.testing.assert_allclose(ev, ref, atol=1e-12)


def test_group_by_basis_matches_oracle():
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.shots import group_by_basis

    H = random_pauli_sum(6, 40, np.random.default_rng(2))
    c1, g1 = group_by_basis(H, 6)
    c0, g0 = sv.group_by_basis(H.codes, H.coeffs)
    assert c1 == c0 and g1 == g0
