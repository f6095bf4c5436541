"""Shot-based energies and parameter-shift gradients on the device, checked
statistically against the exact values."""
import math

import numpy as np
import pytest
import torch

from oracle import sv

pytestmark = pytest.mark.gpu


def _tfim(n):
    terms = [(-1.0, [("Z", i), ("Z", i + 1)]) for i in range(n - 1)] + [(-1.0, [("X", i)]) for i in range(n)]
    terms += [(0.3, [("Y", 0), ("Y", 1)]), (0.5, [])]
    return terms


def test_shot_energy_is_unbiased_within_bounds():
    from tyxonq_gb300.vqe import HEA

    n, layers = 8, 2
    hea = HEA(n, layers, _tfim(n), dtype=torch.complex128)
    th = np.random.default_rng(1).uniform(0, 2 * np.pi, hea.n_params)
    exact = hea.energy(th)
    shots = 20000
    est = hea.energy(th, shots=shots, seed=3)
    # each term's estimate has variance <= 1/shots; 2n+1 weighted terms
    sigma = math.sqrt(sum(c * c for c, t in _tfim(n) if t) / shots)
    assert abs(est - exact) < 5 * sigma
    again = hea.energy(th, shots=shots, seed=3)
    assert again == est  # same seed, same shots


def test_parameter_shift_gradient_with_shots():
    from tyxonq_gb300.vqe import HEA

    n, layers = 5, 1
    hea = HEA(n, layers, _tfim(n), dtype=torch.complex128)
    th = np.random.default_rng(2).uniform(0, 2 * np.pi, hea.n_params)
    e, g = hea.energy_and_grad(th)
    shots = 40000
    es, gs = hea.energy_and_grad(th, runtime="device", shots=shots, seed=5)
    sigma = math.sqrt(sum(c * c for c, t in _tfim(n) if t) / shots)
    assert abs(es - e) < 5 * sigma
    assert np.max(np.abs(gs - g)) < 5 * sigma  # each shifted difference has std <= sigma / sqrt(2)


def test_basis_change_restores_state():
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.hamiltonian import as_pauli_sum
    from tyxonq_gb300.shots import shot_energy

    n = 6
    rng = np.random.default_rng(4)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    psi = K.from_array(v, dtype=torch.complex128)
    H = as_pauli_sum(_tfim(n), n)
    shot_energy(psi, H, 1000, 1)
    np.testing.assert_allclose(psi.cpu().numpy(), v, atol=1e-13)


def test_reference_basis_mapping_matches_its_exact_observable():
    """basis_map='reference' rotates circuit qubit n-1-q for Hamiltonian index q
    and reads parities at q (hea_device_runtime.py:282-284): the estimate
    converges to the exact value of that measured observable."""
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.shots import group_by_basis, shot_energy

    n = 6
    rng = np.random.default_rng(9)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    terms = [(0.7, [("X", 0), ("Z", 2)]), (-0.4, [("Y", 1)]), (0.9, [("Z", 3), ("Z", 5)]), (0.5, [("X", 4)])]
    psi = K.from_array(v, dtype=torch.complex128)
    shots = 40000
    est = shot_energy(psi, terms, shots, seed=2, basis_map="reference")
    h = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
    to_z = {"X": h, "Y": h @ np.diag([1.0, -1j])}
    const, groups = group_by_basis(terms, n)
    exact = const
    for bases, items in groups.items():
        w = v.copy()
        for q, p in enumerate(bases):
            if p in to_z:
                w = sv.apply_1q(w, to_z[p], n - 1 - q, n)
        prob = np.abs(w) ** 2
        idx = np.arange(1 << n)
        for term, c in items:
            mask = 0
            for q, _ in term:
                mask |= 1 << (n - 1 - q)
            par = np.array([bin(i & mask).count("1") & 1 for i in idx])
            exact += c * float(np.sum(prob * (1 - 2 * par)))
    sigma = math.sqrt(sum(c * c for c, t in terms) / shots)
    assert abs(est - exact) < 5 * sigma
    same = shot_energy(psi, terms, shots, seed=2)
    exact_same = float(np.real(np.vdot(v, sv.apply_pauli_sum(v, *sv.terms_to_codes(n, terms)))))
    assert abs(same - exact_same) < 5 * sigma
