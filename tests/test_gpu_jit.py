"""Circuit-specialised (runtime-compiled) staged passes against the oracle and
the interpreting kernel.

Tolerances: complex128 1e-12 absolute per amplitude; complex64
2e-6 * sqrt(gates) absolute per amplitude (as the other state tests).
"""
import math

import numpy as np
import pytest
import torch

from oracle import csv, sv

pytestmark = pytest.mark.gpu

C64, C128 = torch.complex64, torch.complex128


class _C:
    def __init__(self, n, ops):
        self.num_qubits, self.ops = n, ops


def _extended_ops(n, depth, seed):
    from tyxonq_gb300.workloads import random_circuit

    rng = np.random.default_rng(seed)
    ops = random_circuit(n, depth, seed=seed)
    extra = []
    for _ in range(4 * n):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        kind = ["rxx", "ryy", "rzz", "swap", "iswap", "s", "sdg", "x"][int(rng.integers(8))]
        if kind in ("rxx", "ryy", "rzz"):
            extra.append((kind, a, b, float(rng.uniform(0, 2 * np.pi))))
        elif kind in ("swap", "iswap"):
            extra.append((kind, a, b))
        else:
            extra.append((kind, a))
    ops = ops[: len(ops) // 2] + extra + ops[len(ops) // 2:]
    return ops


@pytest.mark.parametrize("n,dtype", [(14, C128), (18, C128), (20, C64), (24, C64)])
def test_specialised_passes_match_oracle_and_interpreter(n, dtype):
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward

    ops = _extended_ops(n, 16, seed=n)
    gates, _ = lower_ops(_C(n, ops), mode="state")
    ref = csv.run_ops(n, ops, allowed=sv.STATE_OPS)
    tol = 1e-12 if dtype == C128 else 2e-6 * math.sqrt(len(ops))
    prog = compile_forward(gates, n, dtype)
    a = prog.run(K.init_statevector(n, dtype=dtype)).cpu().numpy()
    np.testing.assert_allclose(a, ref, atol=tol, rtol=0)
    for bits in (4, 5):  # 4-bit stages (the library kernel's layout) and 5-bit stages
        prog = compile_forward(gates, n, dtype)
        assert prog.specialise(dtype, stage_bits=bits) == prog.n_passes > 0
        assert {obj.rb for kind, obj in prog.segments if kind == "staged"} == {bits}
        b = prog.run(K.init_statevector(n, dtype=dtype)).cpu().numpy()
        np.testing.assert_allclose(b, ref, atol=tol, rtol=0, err_msg=f"{bits}-bit stages")
        np.testing.assert_allclose(b, a, atol=tol, rtol=0)


def _prot_oracle(psi, n, pauli, a):
    """exp(-i a/2 P) psi = cos(a/2) psi - i sin(a/2) P psi (evolve_pauli_ops,
    circuits_library/utils.py:29-59, as one unitary)."""
    codes = [0] * n
    for q, p in pauli:
        codes[q] = {"X": 1, "Y": 2, "Z": 3}[p]
    return math.cos(a / 2) * psi - 1j * math.sin(a / 2) * sv.apply_pauli_term(psi, codes, n)


@pytest.mark.parametrize("dtype", [C128, C64])
def test_specialised_device_angle_pauli_rotations(dtype):
    """Device-side angles (theta read on the GPU), Pauli strings with Z factors
    outside the register stage and outside the tile (Jordan-Wigner-like), and
    multi-qubit X/Y rotations (general rotation code)."""
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.ir import Gate, _rot_gate, pauli_rotation
    from tyxonq_gb300.program import compile_forward

    n = 16
    rng = np.random.default_rng(3)
    gates, params, specs = [], {}, []
    for q in range(n):
        gates.append(_rot_gate("ry", (q,), 0.0))
        params[len(gates) - 1] = (q, 1.0)
        specs.append(("ry", q, q))
    p = n
    for k in range(40):
        i, j = sorted(int(x) for x in rng.choice(n, 2, replace=False))
        mid = [(q, "Z") for q in range(i + 1, j)]
        if k % 3 == 0:
            pauli = ((i, "X"),) + tuple(mid) + ((j, "Y"),)
        elif k % 3 == 1:
            pauli = ((i, "Y"),) + tuple(mid) + ((j, "Z"),)
        else:
            pauli = ((i, "X"), (j, "X"))
        gates.append(pauli_rotation(pauli, 0.0))
        params[len(gates) - 1] = (p, 2.0)
        specs.append(("prot", pauli, p))
        p += 1
        gates.append(Gate("cx", (j, i)))
        specs.append(("cx", (j, i), None))
    theta = rng.uniform(0, 2 * np.pi, p)
    th = torch.tensor(theta, dtype=torch.float64, device="cuda")
    prog = compile_forward(gates, n, dtype, params=params)
    a = prog.run(K.init_statevector(n, dtype=dtype), th).cpu().numpy()
    assert prog.specialise(dtype) > 0
    b = prog.run(K.init_statevector(n, dtype=dtype), th).cpu().numpy()
    ref = sv.init_state(n)
    for nm, x, pi in specs:
        if nm == "ry":
            ref = sv.apply_1q(ref, sv.gate_matrix("ry", theta[pi]), x, n)
        elif nm == "prot":
            ref = _prot_oracle(ref, n, x, 2.0 * theta[pi])
        else:
            ref = sv.apply_2q(ref, sv.gate_matrix("cx"), x[0], x[1], n)
    tol = 1e-12 if dtype == C128 else 2e-6 * math.sqrt(len(gates))
    np.testing.assert_allclose(a, ref, atol=tol, rtol=0)
    np.testing.assert_allclose(b, ref, atol=tol, rtol=0)
    # a new angle vector reuses the compiled kernels
    theta2 = rng.uniform(0, 2 * np.pi, p)
    c = prog.run(K.init_statevector(n, dtype=dtype), torch.tensor(theta2, dtype=torch.float64, device="cuda"))
    d = compile_forward(gates, n, dtype, params=params).run(
        K.init_statevector(n, dtype=dtype), torch.tensor(theta2, dtype=torch.float64, device="cuda"))
    np.testing.assert_allclose(c.cpu().numpy(), d.cpu().numpy(), atol=tol, rtol=0)
