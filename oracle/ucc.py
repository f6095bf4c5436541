"""Oracle for the UCCSD statevector path (test infrastructure only).

Restates the reference's numeric UCC evolution -- per excitation
psi <- psi + (1 - cos t) F^2 psi + sin t F psi with F = T - T^dagger
(chem_libs/quantum_chem_library/statevector_ops.py:140-168) -- with F built
directly from its second-quantised definition on basis states: ladder
operators with the Jordan-Wigner sign (-1)^{number of occupied lower modes}
(the operator statevector_ops.py:25-63 forms from ad_a_hc / adad_aa_hc and a
JW parity phase), mode m = basis bit m (TyxonQ's reversed qubit order).
Runs in PyTorch (CPU, float64/complex128) so autograd gives the reference's
gradient (numerics/backends/pytorch_backend.py:446-564).  The Pauli-sum
energy follows pauli_string_to_matrix semantics without forming 4^n.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _apply_ladder(x: np.ndarray, ops) -> tuple[np.ndarray, np.ndarray]:
    """Apply ladder operators (rightmost first) to all basis states x (int64).
    Returns (x', sign) with sign 0 where the product annihilates the state."""
    x = x.copy()
    sign = np.ones(x.shape, dtype=np.float64)
    for m, creation in reversed(ops):
        bit = (x >> m) & 1
        ok = (bit == 0) if creation else (bit == 1)
        below = x & ((1 << m) - 1)
        par = np.array([bin(int(v)).count("1") & 1 for v in below]) if x.size < 4096 else _popcount_parity(below)
        sign = np.where(ok, sign * np.where(par == 1, -1.0, 1.0), 0.0)
        x = np.where(ok, x ^ (1 << m), x)
    return x, sign


def _popcount_parity(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64)
    p = np.zeros(v.shape, dtype=np.uint64)
    while np.any(v):
        p ^= v & np.uint64(1)
        v >>= np.uint64(1)
    return p.astype(np.int64)


def excitation_generator(f_idx: tuple, n: int) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """F = T - T^dagger as (dest, src, value) triplets over the 2^n basis."""
    x = np.arange(1 << n, dtype=np.int64)
    if len(f_idx) == 2:
        p, q = f_idx
        T = [(p, True), (q, False)]
        Td = [(q, True), (p, False)]
    else:
        p, q, r, s = f_idx
        T = [(p, True), (q, True), (r, False), (s, False)]
        Td = [(s, True), (r, True), (q, False), (p, False)]
    d1, s1 = _apply_ladder(x, T)
    d2, s2 = _apply_ladder(x, Td)
    dest = np.concatenate([d1[s1 != 0], d2[s2 != 0]])
    src = np.concatenate([x[s1 != 0], x[s2 != 0]])
    val = np.concatenate([s1[s1 != 0], -s2[s2 != 0]])
    return torch.from_numpy(dest), torch.from_numpy(src), torch.from_numpy(val).to(torch.complex128)


def apply_F(psi: torch.Tensor, F) -> torch.Tensor:
    dest, src, val = F
    return torch.zeros_like(psi).index_add(0, dest, val * psi[src])


def evolve_excitation(psi: torch.Tensor, F, theta: torch.Tensor) -> torch.Tensor:
    """statevector_ops.py:140-168: psi + (1 - cos t) F^2 psi + sin t F psi."""
    f1 = apply_F(psi, F)
    f2 = apply_F(f1, F)
    return psi + (1.0 - torch.cos(theta)) * f2 + torch.sin(theta) * f1


def pauli_energy(psi: torch.Tensor, codes: np.ndarray, coeffs: np.ndarray) -> torch.Tensor:
    """Re <psi|H|psi>, term by term: P|i> = i^{ny} (-1)^{popc(i & zy)} |i ^ flip>."""
    n = codes.shape[1]
    idx = torch.arange(1 << n, dtype=torch.int64)
    e = torch.zeros((), dtype=torch.float64)
    for row, c in zip(codes, coeffs):
        flip = zy = 0
        ny = 0
        for q, code in enumerate(row):
            b = 1 << (n - 1 - q)
            if code in (1, 2):
                flip |= b
            if code in (2, 3):
                zy |= b
            ny += code == 2
        src = idx ^ flip
        par = torch.zeros(1 << n, dtype=torch.int64)
        v = src & zy
        while bool((v != 0).any()):
            par ^= v & 1
            v = v >> 1
        sgn = (1 - 2 * par).to(torch.complex128) * (1j ** ny)
        hp = sgn * psi[src]  # (P psi)_i
        e = e + float(c) * torch.real(torch.sum(torch.conj(psi) * hp))
    return e


def uccsd_energy_and_autograd(n: int, hf_basis: int, ex_ops, theta: np.ndarray, codes: np.ndarray,
                              coeffs: np.ndarray) -> tuple[float, np.ndarray]:
    """Energy and torch-autograd gradient of the UCC statevector path."""
    th = torch.tensor(np.asarray(theta, dtype=np.float64), requires_grad=True)
    psi = torch.zeros(1 << n, dtype=torch.complex128)
    psi[hf_basis] = 1.0
    for k, f in enumerate(ex_ops):
        psi = evolve_excitation(psi, excitation_generator(tuple(f), n), th[k])
    e = pauli_energy(psi, codes, coeffs)
    e.backward()
    return float(e.item()), th.grad.numpy().copy()


_ = math
