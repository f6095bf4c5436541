"""UCCSD (16 qubits: 8 spatial orbitals, 4 electrons, Jordan-Wigner; 198
excitations, one parameter each, 1440 Pauli rotations) from the Hartree-Fock
bitstring, with the excitations applied exactly (pair rotations) and as
Pauli-string exponentials through the fused-pass engine.  The adjoint gradient is checked against central finite
differences (h = 1e-4), the per-rotation parameter-shift rule, and the torch
autograd gradient of the reference's excitation-evolution formula (oracle).
Tolerances: complex128 energies 1e-10; gradients 1e-9 vs parameter shift and
autograd, 1e-6 vs central differences (O(h^2) truncation)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[False, True], ids=["excitations", "pauli_rotations"])
def ucc(request):
    from tyxonq_gb300 import chem
    from tyxonq_gb300.vqe import UCCSD

    h, g = chem.random_integrals(8, seed=7)
    m = UCCSD(h, g, n_elec=4, dtype=torch.complex128, trotter=request.param)
    theta = np.random.default_rng(2).uniform(-0.3, 0.3, m.n_params)
    return m, theta


def test_uccsd_shapes_and_hf_energy(ucc):
    m, _ = ucc
    assert m.n_qubits == 16 and len(m.ex_ops) == 198 and m.n_params == 198 and len(m.param_gates) == 1440
    # HF energy from the integrals directly: sum_i h_ii + 1/2 sum_ij [(ii|jj) - delta_spin (ij|ji)]
    h, g = m.int1e, m.int2e
    occ = [0, 1]
    e_hf = 2 * sum(h[i, i] for i in occ)
    for i in occ:
        for j in occ:
            e_hf += 2 * g[i, i, j, j] - g[i, j, j, i]
    assert abs(m.energy(np.zeros(m.n_params)) - e_hf) < 1e-10


def test_uccsd_adjoint_vs_autograd_fd_and_parameter_shift(ucc):
    from oracle import ucc as oucc
    from tyxonq_gb300.adjoint import ParamGate, ParametricEstimator
    from tyxonq_gb300.chem import hf_basis

    m, theta = ucc
    e, g = m.energy_and_grad(theta)
    # reference formula (statevector_ops.evolve_excitation) with torch autograd
    e_ref, g_ref = oucc.uccsd_energy_and_autograd(16, hf_basis(16, 2), m.ex_ops, theta, m.hamiltonian.codes,
                                                  m.hamiltonian.coeffs)
    assert abs(e - e_ref) < 1e-10
    np.testing.assert_allclose(g, g_ref, atol=1e-9)
    # central finite differences on a parameter subset
    rng = np.random.default_rng(0)
    sub = rng.choice(m.n_params, 12, replace=False)
    for p in sub:
        tp, tm = theta.copy(), theta.copy()
        tp[p] += 1e-4
        tm[p] -= 1e-4
        fd = (m.energy(tp) - m.energy(tm)) / 2e-4
        assert abs(fd - g[p]) < 1e-6, (p, fd, g[p])
    # parameter shift per rotation: a_r = s_r theta_p, dE/dtheta_p = sum_r s_r (E(a_r+pi/2) - E(a_r-pi/2)) / 2
    rot = [ParamGate(pg.gate, r, 1.0) for r, pg in enumerate(m.param_gates)]
    est = ParametricEstimator(16, rot, len(rot), m.hamiltonian, dtype=torch.complex128,
                              init_basis=hf_basis(16, 2))
    a = np.array([pg.scale * theta[pg.param] for pg in m.param_gates])
    for p in sub[:4]:
        acc = 0.0
        for r, pg in enumerate(m.param_gates):
            if pg.param != p:
                continue
            ap, am = a.copy(), a.copy()
            ap[r] += np.pi / 2
            am[r] -= np.pi / 2
            acc += pg.scale * 0.5 * (est.energy(ap) - est.energy(am))
        assert abs(acc - g[p]) < 1e-9, (p, acc, g[p])


def test_uccsd_complex64_within_tolerance(ucc):
    from tyxonq_gb300 import chem
    from tyxonq_gb300.vqe import UCCSD

    m, theta = ucc
    h, gint = m.int1e, m.int2e
    m64 = UCCSD(h, gint, n_elec=4, dtype=torch.complex64, trotter=m.trotter)
    e64, g64 = m64.energy_and_grad(theta)
    e, g = m.energy_and_grad(theta)
    nrm = m.hamiltonian.one_norm()
    assert abs(e64 - e) < 1e-5 * nrm
    np.testing.assert_allclose(g64, g, atol=1e-4 * nrm)
    _ = chem


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-12), (torch.complex64, 2e-6)])
def test_excitations_on_a_random_state_match_the_oracle(dtype, tol):
    """tq_sv_apply_excitations on an arbitrary state (not only the particle
    sector of the Hartree-Fock state) against the oracle's F built from ladder
    operators, then the inverse sweep back to the start."""
    import ctypes

    from oracle import ucc as oucc
    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import chem
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.excitation import excitation_records

    n = 10
    ex, _ = chem.uccsd_excitations(2, 3)
    rng = np.random.default_rng(4)
    theta = rng.uniform(-1.0, 1.0, len(ex))
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    ref = torch.from_numpy(v.copy())
    for f, t in zip(ex, theta):
        ref = oucc.evolve_excitation(ref, oucc.excitation_generator(tuple(f), n), torch.tensor(t))
    psi = torch.from_numpy(v).to(dtype).cuda()
    rec = torch.from_numpy(excitation_records(n, ex).view(np.uint8).copy()).cuda()
    sc = torch.from_numpy(np.stack([np.sin(theta), np.cos(theta)], 1).reshape(-1).copy()).cuda()
    P = ctypes.c_void_p
    nat.call("tq_sv_apply_excitations", P(psi.data_ptr()), n, K.dtype_tag(psi), P(rec.data_ptr()), len(ex),
             P(sc.data_ptr()), 0, K.stream_ptr())
    np.testing.assert_allclose(psi.cpu().numpy(), ref.numpy(), atol=tol)
    nat.call("tq_sv_apply_excitations", P(psi.data_ptr()), n, K.dtype_tag(psi), P(rec.data_ptr()), len(ex),
             P(sc.data_ptr()), 1, K.stream_ptr())
    np.testing.assert_allclose(psi.cpu().numpy(), v, atol=tol)
