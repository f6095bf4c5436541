"""CI-space UCC on the GPU against the oracle and the statevector engine."""
import numpy as np
import pytest
import torch

from oracle import ci
from tyxonq_gb300 import chem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_orb,n_elec", [(4, 4), (6, 4), (8, 4)])
def test_civector_energy_and_grad(n_orb, n_elec):
    from tyxonq_gb300.vqe import UCCSD

    no = n_elec // 2
    n = 2 * n_orb
    h1, h2 = chem.random_integrals(n_orb, seed=11)
    u_ci = UCCSD(h1, h2, n_elec, engine="civector")
    params = np.random.default_rng(2).uniform(-0.3, 0.3, u_ci.n_params)
    e, g = u_ci.energy_and_grad(params)
    ex = u_ci.ex_ops
    pid = list(range(len(ex)))
    H = u_ci.hamiltonian
    strings, fperm, fphase, f2phase = ci.operator_tensors(n, (no, no), ex)
    e_ref, g_ref = ci.energy_and_grad(params, pid, strings, fperm, fphase, f2phase,
                                      ci.h_apply_via_full_space(H.codes, H.coeffs, strings, n))
    assert abs(e - e_ref) < 1e-10
    np.testing.assert_allclose(g, g_ref, atol=1e-10)
    assert abs(u_ci.energy(params) - e) < 1e-12
    # the statevector engine (complex128 Pauli rotations, adjoint gradient) agrees
    u_sv = UCCSD(h1, h2, n_elec, dtype=torch.complex128)
    e_sv, g_sv = u_sv.energy_and_grad(params)
    assert abs(e_sv - e) < 1e-9
    np.testing.assert_allclose(g_sv, g, atol=1e-8)
