"""Shot-based Pauli-sum energies on the device (the "device" runtime path).

The reference estimates <H> from measurement counts: terms are grouped by
their product basis (tyxonq/libs/hamiltonian_encoding/hamiltonian_grouping.py:
120-138, identical bases share one circuit), each group's circuit gets the
basis change H (X) or S^dagger H (Y) before measuring every qubit in Z
(applications/chem/runtimes/hea_device_runtime.py:_prefix_ops_for_bases),
and a term's expectation is the mean parity of its qubits over the shots
(postprocessing/counts_expval.py:7-20, expval_pauli_sum :96-130).  Gradients
in that runtime are parameter-shift differences E(theta + pi/2) - E(theta -
pi/2) over the same estimator (hea_device_runtime.py:energy_and_grad).

Here the state is prepared once per parameter vector on the GPU, each group's
basis change is applied in place with the 1q kernel, shots are drawn with the
device sampler (sorted basis indices, counter-based RNG), the change is undone,
and the parities are reduced from the sampled indices.  A term's qubit q is
the circuit's qubit q (bit n-1-q of the basis index); basis_map="reference"
reproduces the reference runtime's mapping instead (rotation on circuit qubit
n-1-q for Hamiltonian index q).
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np
import torch

from . import kernels as K
from .hamiltonian import PauliSum, as_pauli_sum

_H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2)
_SDG = np.diag([1.0, -1j])
_TO_Z = {"X": _H, "Y": _H @ _SDG}  # applied as the matrix product (S^dagger first, then H)
_FROM_Z = {p: m.conj().T for p, m in _TO_Z.items()}


def group_by_basis(H, n: int) -> tuple[float, dict]:
    """(identity constant, {bases: [(term, coeff)]}) with bases a length-n tuple
    over 'IXYZ' and term = ((q, P), ...): the grouping rule of
    group_hamiltonian_pauli_terms (hamiltonian_grouping.py:120-138)."""
    ps = as_pauli_sum(H, n)
    inv = "IXYZ"
    const = 0.0
    groups: dict = {}
    for codes, c in zip(ps.codes, ps.coeffs):
        term = tuple((q, inv[int(x)]) for q, x in enumerate(codes) if x)
        if not term:
            const += float(c)
            continue
        bases = tuple(inv[int(x)] for x in codes)
        groups.setdefault(bases, []).append((term, float(c)))
    return const, groups


def parity_expectations(indices: np.ndarray, terms: Sequence, n: int) -> np.ndarray:
    """<Z_{q1} Z_{q2} ...> per term from sampled basis indices (mean of
    (-1)^{parity of the term's bits}), as term_expectation_from_counts."""
    idx = np.asarray(indices, dtype=np.uint64)
    out = np.empty(len(terms))
    for k, term in enumerate(terms):
        mask = np.uint64(0)
        for q, _p in term:
            mask |= np.uint64(1) << np.uint64(n - 1 - int(q))
        par = np.bitwise_count(idx & mask) & 1
        out[k] = 1.0 - 2.0 * float(par.mean()) if idx.size else 0.0
    return out


def shot_energy(psi: torch.Tensor, H, shots: int, seed: int, grouping: tuple | None = None,
                basis_map: str = "same") -> float:
    """Estimate <psi|H|psi> from `shots` samples per basis group.  psi is
    restored (up to rounding) on return.

    basis_map: "same" rotates circuit qubit q for the term's qubit q (the
    estimate of <H>); "reference" reproduces hea_device_runtime.py:
    _prefix_ops_for_bases (:282-284), which rotates circuit qubit n-1-q for
    Hamiltonian index q while the parities are read at position q, so that
    results equal that runtime's on the same counts."""
    n = K._check_state(psi)
    if basis_map not in ("same", "reference"):
        raise ValueError("basis_map must be 'same' or 'reference'")
    const, groups = grouping if grouping is not None else group_by_basis(H, n)
    e = const
    for gi, (bases, items) in enumerate(groups.items()):
        rot = [((n - 1 - q) if basis_map == "reference" else q, p) for q, p in enumerate(bases) if p in _TO_Z]
        for q, p in rot:
            K.apply_1q(psi, _TO_Z[p], q)
        idx = K.sample(psi, shots, (int(seed) * 1000003 + gi) & ((1 << 63) - 1)).cpu().numpy()
        for q, p in rot:
            K.apply_1q(psi, _FROM_Z[p], q)
        ev = parity_expectations(idx, [t for t, _ in items], n)
        e += float(np.dot(ev, [c for _, c in items]))
    return float(e)


class ShotEstimator:
    """Shot-based energy and parameter-shift gradient of a parametrised circuit
    whose angles are read on the device (ParametricEstimator's forward
    program): every shifted parameter vector is one forward run plus one
    sampling round per basis group."""

    def __init__(self, est, H, shots: int = 1024, seed: int = 0, basis_map: str = "same"):
        self.est = est
        self.n = est.n
        self.shots = int(shots)
        self.seed = int(seed)
        self.grouping = group_by_basis(H, self.n)
        self.basis_map = basis_map
        self._calls = 0

    def energy(self, theta) -> float:
        psi = self.est._forward(np.asarray(theta, dtype=np.float64))
        self._calls += 1
        return shot_energy(psi, None, self.shots, self.seed + self._calls, self.grouping, self.basis_map)

    def energy_and_grad(self, theta) -> tuple[float, np.ndarray]:
        th = np.asarray(theta, dtype=np.float64)
        e0 = self.energy(th)
        g = np.zeros_like(th)
        s = 0.5 * math.pi
        for i in range(th.size):
            tp, tm = th.copy(), th.copy()
            tp[i] += s
            tm[i] -= s
            g[i] = 0.5 * (self.energy(tp) - self.energy(tm))
        return e0, g
