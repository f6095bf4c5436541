"""CI-space UCC restatement: consistency with the statevector UCC oracle (the
reference's two numeric engines describe the same state), and the product's
host-side tensor builder against the oracle's."""
import numpy as np
import pytest

from oracle import ci, ucc
from tyxonq_gb300 import chem


@pytest.mark.parametrize("n_orb,n_elec", [(3, 2), (4, 4), (4, 2)])
def test_ci_space_equals_statevector_ucc(n_orb, n_elec):
    no = n_elec // 2
    n = 2 * n_orb
    ex, pid = chem.uccsd_excitations(no, n_orb - no)
    h1, h2 = chem.random_integrals(n_orb, seed=3)
    H = chem.molecular_hamiltonian(h1, h2)
    params = np.random.default_rng(5).uniform(-0.5, 0.5, max(pid) + 1)
    strings, fperm, fphase, f2phase = ci.operator_tensors(n, (no, no), ex)
    e_ci, g_ci = ci.energy_and_grad(params, pid, strings, fperm, fphase, f2phase,
                                    ci.h_apply_via_full_space(H.codes, H.coeffs, strings, n))
    e_sv, g_th = ucc.uccsd_energy_and_autograd(n, chem.hf_basis(n, no), ex, params[pid], H.codes, H.coeffs)
    g_sv = np.zeros_like(params)
    np.add.at(g_sv, pid, g_th)
    assert abs(e_ci - e_sv) < 1e-12
    np.testing.assert_allclose(g_ci, g_sv, atol=1e-12)


def test_host_tensors_match_oracle():
    from tyxonq_gb300.ci import operator_tensors

    n_orb, no = 5, 2
    ex, _ = chem.uccsd_excitations(no, n_orb - no)
    a = operator_tensors(2 * n_orb, (no, no), ex)
    b = ci.operator_tensors(2 * n_orb, (no, no), ex)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(np.asarray(x).astype(np.int64), np.asarray(y).astype(np.int64))
