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


def _csr_apply(strings, H):
    import scipy.sparse as sp

    from tyxonq_gb300.ci import ci_hamiltonian_csr

    rp, col, val = ci_hamiltonian_csr(strings, H)
    m = sp.csr_matrix((val, col, rp), shape=(len(strings), len(strings)))
    return lambda x: m @ x


@pytest.mark.parametrize("n_orb,n_elec,fused", [(4, 4, True), (4, 4, False), (7, 6, True), (7, 6, False),
                                                (8, 6, True), (8, 8, True)])
def test_civector_one_cta_and_stepwise_paths(n_orb, n_elec, fused):
    """Both GPU paths (one single-CTA launch for D up to the shared-memory
    limit; one launch per excitation step) against the oracle's reverse sweep
    with H as the CI-space CSR (checked against the full-space H on the CPU).
    Sweep CTAs: (4, 4) 256 threads, one pair each; (7, 6) 256 threads, up to
    two; (8, 6) 1024 threads, one; (8, 8) D = 4900, 1024 threads, up to two."""
    from tyxonq_gb300.ci import CIVectorUCC

    no = n_elec // 2
    n = 2 * n_orb
    h1, h2 = chem.random_integrals(n_orb, seed=5)
    H = chem.molecular_hamiltonian(h1, h2)
    ex, pid = chem.uccsd_excitations(no, n_orb - no)
    m = CIVectorUCC(n, (no, no), ex, pid, H, fused=fused)
    assert m.fused == fused
    params = np.random.default_rng(3).uniform(-0.4, 0.4, max(pid) + 1)
    e, g = m.energy_and_grad(params)
    strings, fperm, fphase, f2phase = ci.operator_tensors(n, (no, no), ex)
    e_ref, g_ref = ci.energy_and_grad(params, pid, strings, fperm, fphase, f2phase, _csr_apply(strings, H))
    assert abs(e - e_ref) < 1e-10
    np.testing.assert_allclose(g, g_ref, atol=1e-10)
    assert abs(m.energy(params) - e) < 1e-12
    ket = m.civector(params).cpu().numpy()
    np.testing.assert_allclose(ket, ci.evolve(np.eye(len(strings))[0], fperm, fphase, f2phase,
                                              np.asarray(params)[pid]), atol=1e-12)


def test_civector_repeated_calls_and_zero_excitations():
    from tyxonq_gb300.ci import CIVectorUCC

    h1, h2 = chem.random_integrals(4, seed=6)
    H = chem.molecular_hamiltonian(h1, h2)
    ex, pid = chem.uccsd_excitations(2, 2)
    m = CIVectorUCC(8, (2, 2), ex, pid, H)
    rng = np.random.default_rng(0)
    ps = [rng.uniform(-0.5, 0.5, max(pid) + 1) for _ in range(4)]
    first = [m.energy_and_grad(p) for p in ps]
    again = [m.energy_and_grad(p) for p in ps]
    for (e1, g1), (e2, g2) in zip(first, again):
        assert e1 == e2 and np.array_equal(g1, g2)  # fixed-order sums: bit-identical
    # no excitations: the energy of the first determinant, an empty gradient
    m0 = CIVectorUCC(8, (2, 2), [], [], H)
    strings, _ = ci.ci_strings(8, (2, 2))
    e0, g0 = m0.energy_and_grad(np.zeros(0))
    assert abs(e0 - _csr_apply(strings, H)(np.eye(len(strings))[0])[0]) < 1e-12 and g0.shape == (0,)
