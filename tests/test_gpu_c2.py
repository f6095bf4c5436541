"""The 28-qubit depth-40 random circuit (complex64 on the device) against the
C complex128 oracle (oracle/sv_ref.c), with full probabilities and 8192 shots.

Every device path is checked: the fused register-staged tile passes (the
interpreting kernel and the circuit-specialised kernels) and the
one-launch-per-gate engine.  Tolerances (unit-norm state, about 760 gates):
  * ||psi_gpu - psi_ref||_2 <= 2e-5, max |psi_gpu - psi_ref| <= 2e-7
    (amplitudes are about 2^-14 = 6e-5 in magnitude);
  * probabilities (float32): sum |p_gpu - p_ref| <= 2e-5;
  * 8192 device shots: chi^2 tests (p > 1e-3) against the oracle's
    probabilities, in 16 bins of equal probability mass ordered by the
    outcome's own probability (Porter-Thomas shape) and in the 16 bins of the
    four leading qubits.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NQ = 28
SHOTS = 8192
CHUNK = 1 << 24


@pytest.fixture(scope="module")
def c2():
    from oracle import csv
    from tyxonq_gb300.workloads import random_circuit

    ops = random_circuit(NQ, 40, seed=1)
    ref = csv.run_ops(NQ, ops)
    return ops, ref


def _gates(ops):
    from tyxonq_gb300.ir import lower_ops

    class _C:
        def __init__(self, n, o):
            self.num_qubits, self.ops = n, o

    gates, _ = lower_ops(_C(NQ, ops), mode="run")
    return gates


def _state_errors(psi, ref):
    sq, mx = 0.0, 0.0
    for o in range(0, ref.size, CHUNK):
        a = psi[o:o + CHUNK].cpu().numpy().astype(np.complex128)
        d = np.abs(a - ref[o:o + CHUNK])
        sq += float(np.dot(d, d))
        mx = max(mx, float(d.max()))
    return np.sqrt(sq), mx


def _chi2_p(observed, expected):
    from scipy.stats import chi2

    stat = float(((observed - expected) ** 2 / expected).sum())
    return float(chi2.sf(stat, observed.size - 1))


def test_c2_fused_and_plain_states_match_c128_oracle(c2):
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.engine import execute_plain
    from tyxonq_gb300.program import compile_forward

    ops, ref = c2
    gates = _gates(ops)
    assert 700 <= len(gates) <= 800
    prog = compile_forward(gates, NQ, torch.complex64)
    psi = K.init_statevector(NQ, dtype=torch.complex64)
    prog.run(psi)
    torch.cuda.synchronize()
    l2, mx = _state_errors(psi, ref)
    print(f"\nfused ({prog.n_passes} passes): ||d||_2 = {l2:.3e}, max |d| = {mx:.3e}")
    assert l2 <= 2e-5 and mx <= 2e-7
    assert prog.specialise(torch.complex64) == prog.n_passes
    psi = K.init_statevector(NQ, dtype=torch.complex64)
    prog.run(psi)
    torch.cuda.synchronize()
    l2, mx = _state_errors(psi, ref)
    print(f"fused, specialised kernels: ||d||_2 = {l2:.3e}, max |d| = {mx:.3e}")
    assert l2 <= 2e-5 and mx <= 2e-7
    del psi
    psi = K.init_statevector(NQ, dtype=torch.complex64)
    execute_plain(psi, gates)
    torch.cuda.synchronize()
    l2, mx = _state_errors(psi, ref)
    print(f"plain ({len(gates)} launches): ||d||_2 = {l2:.3e}, max |d| = {mx:.3e}")
    assert l2 <= 2e-5 and mx <= 2e-7
    del psi
    torch.cuda.empty_cache()


def test_c2_probabilities_and_shots_match_c128_oracle(c2):
    from oracle import csv
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.program import compile_forward

    ops, ref = c2
    prog = compile_forward(_gates(ops), NQ, torch.complex64)
    prog.specialise(torch.complex64)
    psi = K.init_statevector(NQ, dtype=torch.complex64)
    prog.run(psi)
    probs = K.probabilities(psi)
    idx = K.sample(psi, SHOTS, seed=11)
    torch.cuda.synchronize()
    p_ref = csv.probabilities(ref)
    l1 = 0.0
    for o in range(0, p_ref.size, CHUNK):
        l1 += float(np.abs(probs[o:o + CHUNK].cpu().numpy().astype(np.float64) - p_ref[o:o + CHUNK]).sum())
    print(f"\nprobabilities: sum |dp| = {l1:.3e}")
    assert l1 <= 2e-5
    idx = idx.cpu().numpy()
    assert idx.size == SHOTS and (np.diff(idx) >= 0).all() and idx.min() >= 0 and idx.max() < (1 << NQ)
    assert (p_ref[idx] > 0).all()
    # equal-mass bins of the outcome's own probability
    x = p_ref * float(1 << NQ)
    qs = np.linspace(0, 1, 17)[1:-1]
    # edges from the mass-weighted distribution: sort a uniform subsample by x, weight by x
    sub = np.sort(x[np.random.default_rng(0).integers(0, x.size, 1 << 22)])
    cum = np.cumsum(sub)
    cum /= cum[-1]
    edges = sub[np.searchsorted(cum, qs)]
    bins = np.concatenate([[-np.inf], edges, [np.inf]])
    mass, _ = np.histogram(x, bins=bins, weights=p_ref)
    obs, _ = np.histogram(x[idx], bins=bins)
    exp = SHOTS * mass / mass.sum()
    assert exp.min() > 50
    p1 = _chi2_p(obs.astype(np.float64), exp)
    # leading four qubits
    lead = p_ref.reshape(16, -1).sum(axis=1)
    obs2 = np.bincount(idx >> (NQ - 4), minlength=16).astype(np.float64)
    p2 = _chi2_p(obs2, SHOTS * lead / lead.sum())
    print(f"chi^2 p-values: probability-mass bins {p1:.3f}, leading-qubit bins {p2:.3f}")
    assert p1 > 1e-3 and p2 > 1e-3
    del psi, probs
    torch.cuda.empty_cache()
