"""The C complex128 restatement (oracle/sv_ref.c) pinned like the NumPy one:
golden states, energies and the 12-qubit HEA energy produced by the reference
itself, and agreement with the NumPy restatement on random circuits (1e-12)."""
import numpy as np
import pytest

from oracle import csv, sv
from tests import golden_data as gd


def test_c_oracle_golden_states():
    checked = 0
    for name, n, ops, ucache, state, _runz in gd.circuit_cases():
        if any(o[0] in ("project_z", "reset", "kraus") for o in ops):
            continue
        psi = csv.run_ops(n, ops, allowed=sv.STATE_OPS, unitary_cache=ucache)
        np.testing.assert_allclose(psi, state, atol=1e-12, err_msg=name)
        checked += 1
    assert checked >= 3


def test_c_oracle_golden_energies():
    arrays, meta = gd.load()
    for case in meta["pauli"]:
        nm = case["name"]
        e = csv.pauli_expectation(arrays[f"{nm}_psi"].astype(np.complex128), arrays[f"{nm}_codes"], arrays[f"{nm}_w"])
        assert abs(e - case["energy"]) < 1e-12, nm


def test_c_oracle_hea12_energy():
    from tyxonq_gb300.hamiltonian import PauliSum, tfim_terms
    from tyxonq_gb300.workloads import hea_tfim

    _, meta = gd.load()
    ops, H, _theta = hea_tfim(12, 4, seed=0)
    psi = csv.run_ops(12, ops)
    e = csv.pauli_expectation(psi, H.codes, H.coeffs)
    assert abs(e - meta["hea12"]["energy_numpy"]) < 1e-12


@pytest.mark.parametrize("seed", [0, 1])
def test_c_oracle_matches_numpy_oracle(seed):
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.workloads import random_circuit

    n = 11
    ops = random_circuit(n, 12, seed=seed)
    rng = np.random.default_rng(seed)
    extra = [("rxx", 0, 5, 0.3), ("ryy", 2, 9, 1.1), ("rzz", 4, 3, 2.2), ("swap", 1, 8), ("iswap", 7, 2),
             ("s", 3), ("sdg", 6), ("x", 10), ("cx", 4, 4)]
    ops = ops + extra
    a = csv.run_ops(n, ops)
    b, _ = sv.run_ops(n, ops)
    np.testing.assert_allclose(a, b, atol=1e-12)
    H = random_pauli_sum(n, 120, rng)
    assert abs(csv.pauli_expectation(a, H.codes, H.coeffs) - sv.pauli_expectation(b, H.codes, H.coeffs)) < 1e-12
    np.testing.assert_allclose(csv.probabilities(a), np.abs(b) ** 2, atol=1e-15)
