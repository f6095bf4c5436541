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
