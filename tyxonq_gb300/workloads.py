"""Seeded synthetic workloads (the benchmark configurations).

* ``hea_tfim_ops``      12-qubit hardware-efficient ansatz [RY on every qubit;
                        CX ladder i->i+1] x layers with the open-chain TFIM
                        H = -sum Z_i Z_{i+1} - sum X_i (the reference's
                        CPU-runnable case).
* ``random_circuit``    depth-d random circuit: per layer the qubits are
                        shuffled, ~half of the gates are CX/CZ on random pairs,
                        the rest 1q gates uniform in {H, RX, RY, RZ}, angles
                        U[0, 2pi) (the 28-qubit memory-bound case).
* ``batched_vqe``       instances with n ~ U{8..20}, depth ~ U{2..8} of
                        [RY layer; RZ layer; CX ladder], theta ~ U[0, 2pi), and
                        an own random Pauli sum of 50-500 terms (weight 1-4,
                        Paulis uniform in X/Y/Z, coefficients N(0,1)).
No public dataset is involved; every generator takes an explicit seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .hamiltonian import PauliSum, random_pauli_sum, tfim_terms


def hea_ry_cx_ops(n: int, layers: int, theta) -> list:
    """Op tuples of [RY(theta) on all qubits; CX(i, i+1) ladder] x layers."""
    th = np.asarray(theta, dtype=np.float64).reshape(layers, n)
    ops = []
    for l in range(layers):
        for q in range(n):
            ops.append(("ry", q, float(th[l, q])))
        for q in range(n - 1):
            ops.append(("cx", q, q + 1))
    return ops


def hea_tfim(n: int = 12, layers: int = 4, seed: int = 0):
    theta = np.random.default_rng(seed).uniform(0, 2 * math.pi, (layers, n))
    return hea_ry_cx_ops(n, layers, theta), PauliSum.from_terms(n, tfim_terms(n)), theta


def random_circuit(n: int = 28, depth: int = 40, seed: int = 1, pairs_per_layer: int | None = None) -> list:
    rng = np.random.default_rng(seed)
    if pairs_per_layer is None:
        pairs_per_layer = n // 3  # 2q gates cover 2/3 of the qubits -> ~50% of gates are 2q
    ops = []
    for _ in range(depth):
        perm = rng.permutation(n)
        k = 2 * pairs_per_layer
        for j in range(0, k, 2):
            a, b = int(perm[j]), int(perm[j + 1])
            ops.append(("cx" if rng.random() < 0.5 else "cz", a, b))
        for q in perm[k:]:
            kind = ["h", "rx", "ry", "rz"][int(rng.integers(4))]
            if kind == "h":
                ops.append(("h", int(q)))
            else:
                ops.append((kind, int(q), float(rng.uniform(0, 2 * math.pi))))
    return ops


def hea_rz_ops_params(n: int, depth: int) -> list:
    """[(name, qubits, param index or None)] of [RY layer; RZ layer; CX ladder] x depth."""
    out = []
    p = 0
    for _ in range(depth):
        for q in range(n):
            out.append(("ry", (q,), p))
            p += 1
        for q in range(n):
            out.append(("rz", (q,), p))
            p += 1
        for q in range(n - 1):
            out.append(("cx", (q, q + 1), None))
    return out


@dataclass
class VqeInstance:
    n: int
    depth: int
    theta: np.ndarray
    H: PauliSum

    @property
    def n_params(self) -> int:
        return 2 * self.n * self.depth

    def structure(self) -> list:
        return hea_rz_ops_params(self.n, self.depth)

    def ops(self, theta=None) -> list:
        th = self.theta if theta is None else np.asarray(theta)
        ops = []
        for name, qs, p in self.structure():
            ops.append((name, *qs) if p is None else (name, *qs, float(th[p])))
        return ops


def batched_vqe(count: int = 4096, seed: int = 3, n_range=(8, 20), depth_range=(2, 8), terms_range=(50, 500)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        d = int(rng.integers(depth_range[0], depth_range[1] + 1))
        K = int(rng.integers(terms_range[0], terms_range[1] + 1))
        theta = rng.uniform(0, 2 * math.pi, 2 * n * d)
        out.append(VqeInstance(n, d, theta, random_pauli_sum(n, K, rng)))
    return out
