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


@pytest.mark.parametrize("n_orb,n_elec", [(3, 2), (4, 4), (5, 4)])
def test_ci_hamiltonian_csr_matches_full_space_apply(n_orb, n_elec):
    """The product's CI-space CSR of H against the oracle's H applied in the
    full statevector and gathered back."""
    from tyxonq_gb300.ci import ci_hamiltonian_csr

    no = n_elec // 2
    n = 2 * n_orb
    h1, h2 = chem.random_integrals(n_orb, seed=4)
    H = chem.molecular_hamiltonian(h1, h2)
    strings, _ = ci.ci_strings(n, (no, no))
    rp, col, val = ci_hamiltonian_csr(strings, H)
    D = len(strings)
    assert rp.shape == (D + 1,) and rp[0] == 0 and rp[-1] == len(col) == len(val)
    assert col.min() >= 0 and col.max() < D
    dense = np.zeros((D, D))
    for i in range(D):
        dense[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    np.testing.assert_allclose(dense, dense.T, atol=1e-12)
    apply = ci.h_apply_via_full_space(H.codes, H.coeffs, strings, n)
    x = np.random.default_rng(1).normal(size=(D, 3))
    for k in range(3):
        np.testing.assert_allclose(dense @ x[:, k], apply(x[:, k]), atol=1e-12)


def test_excitation_pairs_cover_the_dense_update():
    """The pair lists the GPU sweeps use reproduce the oracle's dense
    per-excitation update c + omc f2 c + sin f c[perm] exactly."""
    from tyxonq_gb300.ci import CI_SWEEP_THREADS, excitation_pairs, operator_tensors, partial_starts

    n_orb, no = 5, 2
    ex, _ = chem.uccsd_excitations(no, n_orb - no)
    _, fperm, fphase, f2phase = operator_tensors(2 * n_orb, (no, no), ex)
    pairs, starts = excitation_pairs(fperm, fphase, f2phase)
    assert pairs.dtype == np.int32 and starts[0] == 0 and starts[-1] == len(pairs)
    D = fperm.shape[1]
    rng = np.random.default_rng(0)
    for j in range(len(ex)):
        c = rng.normal(size=D)
        s, omc = np.sin(0.3 + j), 1 - np.cos(0.3 + j)
        dense = c + omc * f2phase[j] * c + s * fphase[j] * c[fperm[j]]
        sparse = c.copy()
        for i, y in pairs[starts[j]:starts[j + 1]]:
            p, phi = y >> 1, (-1.0 if y & 1 else 1.0)
            sparse[i] = c[i] - omc * c[i] + s * phi * c[p]
            sparse[p] = c[p] - omc * c[p] - s * phi * c[i]
        np.testing.assert_allclose(sparse, dense, atol=1e-14)
    ps = partial_starts(D, starts)
    assert ps[0] == 0 and ps[1] == min(D, CI_SWEEP_THREADS) and len(ps) == len(ex) + 2
    np.testing.assert_array_equal(np.diff(ps)[1:], np.minimum(np.diff(starts), CI_SWEEP_THREADS))
    bad = fphase.copy()
    bad[0, np.flatnonzero(bad[0])[0]] *= -1
    with pytest.raises(ValueError):
        excitation_pairs(fperm, bad, f2phase)
