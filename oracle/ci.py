"""CPU restatement of TyxonQ's CI-space UCC (test infrastructure only).

Follows tyxonq/applications/chem/chem_libs/quantum_chem_library/:
  * ci_state_mapping.py:38-115  get_ci_strings / get_addr (alpha strings in the
    high half of the bitstring, alpha-major order);
  * civector_ops.py:436-483     get_operators, get_fket_permutation, get_fket_phase;
  * libs/hamiltonian_encoding/pauli_io.py:169-206  get_fermion_phase (Z mask and
    sign of the first Jordan-Wigner Pauli word of the excitation operator);
  * civector_ops.py:334-350     evolve_civector_by_tensor;
  * civector_ops.py:141-200     energy_and_grad_civector (reverse sweep).
The reference builds the per-spin strings with pyscf's cistring.make_strings
(pyscf is not installed here); for a contiguous orbital range that is the
ascending order of the bit patterns, which this restatement uses.  Energies
and gradients do not depend on the order.
"""
from __future__ import annotations

from itertools import combinations

import numpy as np


def make_strings(norb: int, nelec: int) -> np.ndarray:
    """All norb-bit patterns with nelec bits set, ascending."""
    out = [sum(1 << i for i in occ) for occ in combinations(range(norb), nelec)]
    return np.array(sorted(out), dtype=np.uint64)


def ci_strings(n_qubits: int, n_elec_s: tuple[int, int]) -> tuple[np.ndarray, dict]:
    """(strings, per-spin address tables) of get_ci_strings(strs2addr=True)."""
    na, nb = n_elec_s
    h = n_qubits // 2
    beta = make_strings(h, nb)
    alpha = make_strings(h, na)
    strings = ((alpha << np.uint64(h)).reshape(-1, 1) + beta.reshape(1, -1)).ravel()
    a2 = np.zeros(1 << h, dtype=np.int64)
    b2 = np.zeros(1 << h, dtype=np.int64)
    a2[alpha.astype(np.int64)] = np.arange(len(alpha))
    b2[beta.astype(np.int64)] = np.arange(len(beta))
    return strings, {"alpha": a2, "beta": b2, "nbeta": len(beta), "half": h}


def _ladder(m: int, creation: bool) -> dict:
    # a^dagger_m / a_m = (X_m -/+ i Y_m)/2 Z_{<m}; in X^x Z^z words: (X + s X Z)/2 Z_{<m}
    low = (1 << m) - 1
    return {(1 << m, low): 0.5, (1 << m, low | (1 << m)): 0.5 if creation else -0.5}


def _mul(A: dict, B: dict) -> dict:
    out: dict = {}
    for (x1, z1), c1 in A.items():
        for (x2, z2), c2 in B.items():
            s = -1.0 if bin(z1 & x2).count("1") & 1 else 1.0
            k = (x1 ^ x2, z1 ^ z2)
            out[k] = out.get(k, 0) + s * c1 * c2
    return out


def fermion_phase_mask_sign(f_idx: tuple, n_qubits: int) -> tuple[int, int]:
    """(Z mask, sign) of get_fermion_phase: the JW image of a^dagger_f0 a_f1
    (or a^dagger a^dagger a a) is sorted as openfermion sorts its terms
    (tuples of (qubit, 'X'|'Y'|'Z') by qubit); the first word's Z qubits give
    the mask and sign = -1 if its coefficient's real part is positive."""
    ops = [(f_idx[0], True), (f_idx[1], False)] if len(f_idx) == 2 else \
        [(f_idx[0], True), (f_idx[1], True), (f_idx[2], False), (f_idx[3], False)]
    acc = {(0, 0): 1.0 + 0j}
    for m, cr in ops:
        acc = _mul(acc, _ladder(m, cr))
    words = []
    for (x, z), c in acc.items():
        if abs(c) < 1e-12:
            continue
        ny = bin(x & z).count("1")
        w = c * (-1j) ** ny  # coefficient of the word with Y where x and z overlap
        key = []
        for q in range(n_qubits):
            xb, zb = (x >> q) & 1, (z >> q) & 1
            if xb or zb:
                key.append((q, "Y" if xb and zb else ("X" if xb else "Z")))
        words.append((tuple(key), w))
    words.sort(key=lambda kv: kv[0])
    key, w = words[0]
    mask = 0
    for q, p in key:
        if p == "Z":
            mask |= 1 << q
    return mask, (-1 if w.real > 0 else 1)


def operator_tensors(n_qubits: int, n_elec_s: tuple[int, int], ex_ops) -> tuple:
    """(strings, fperm, fphase, f2phase) of get_operator_tensors (mode 'fermion')."""
    strings, tab = ci_strings(n_qubits, n_elec_s)
    s = strings.astype(np.int64)
    h = tab["half"]
    fperm, fphase, f2phase = [], [], []
    for f in ex_ops:
        if len(set(f)) != len(f):
            raise ValueError(f"Excitation {f} not supported")
        mask = sum(1 << i for i in f)
        exc = s ^ mask
        perm = tab["alpha"][exc >> h] * tab["nbeta"] + tab["beta"][exc & ((1 << h) - 1)]
        if len(f) == 2:
            m1, m2 = 1 << f[0], 1 << f[1]
        else:
            m1, m2 = (1 << f[0]) + (1 << f[1]), (1 << f[2]) + (1 << f[3])
        masked = (s ^ m1) & (m1 | m2)
        pos = masked == (m1 | m2)
        neg = masked == 0
        zmask, sign = fermion_phase_mask_sign(tuple(f), n_qubits)
        par = np.array([bin(int(v) & zmask).count("1") & 1 for v in s])
        ph = sign * np.where(par == 1, 1, -1)
        fperm.append(perm)
        fphase.append((neg.astype(np.int64) - pos.astype(np.int64)) * ph)
        f2phase.append(-(pos.astype(np.int64) + neg.astype(np.int64)))
    return strings, np.array(fperm), np.array(fphase), np.array(f2phase)


def evolve(civ: np.ndarray, fperm, fphase, f2phase, theta: np.ndarray) -> np.ndarray:
    """evolve_civector_by_tensor: civ += (1 - cos t) f2phase civ + sin t civ[fperm] fphase."""
    c = np.asarray(civ, dtype=np.float64).copy()
    for j in range(len(fperm)):
        c = c + (1 - np.cos(theta[j])) * (f2phase[j] * c) + np.sin(theta[j]) * (c[fperm[j]] * fphase[j])
    return c


def energy_and_grad(params, param_ids, strings, fperm, fphase, f2phase, apply_h) -> tuple[float, np.ndarray]:
    """energy_and_grad_civector with apply_h(ket) = H ket in CI space."""
    params = np.asarray(params, dtype=np.float64)
    theta = np.array([params[i] for i in param_ids])
    ket = np.zeros(len(strings))
    ket[0] = 1.0
    ket = evolve(ket, fperm, fphase, f2phase, theta)
    bra = apply_h(ket)
    e = float(np.dot(bra, ket))
    k, b = ket.copy(), bra.copy()
    gj = np.zeros(len(fperm))
    for j in range(len(fperm) - 1, -1, -1):
        s, omc = np.sin(theta[j]), 1 - np.cos(theta[j])
        k = k + omc * (k * f2phase[j]) - s * (k[fperm[j]] * fphase[j])
        b = b + omc * (b * f2phase[j]) - s * (b[fperm[j]] * fphase[j])
        gj[j] = float(np.dot(b, k[fperm[j]] * fphase[j]))
    g = np.zeros_like(params)
    for v, pid in zip(gj, param_ids):
        g[pid] += v
    return e, 2.0 * g


def h_apply_via_full_space(codes: np.ndarray, coeffs: np.ndarray, strings: np.ndarray, n: int):
    """H restricted to the CI space through the full statevector (H conserves
    the particle number, so the restriction is exact): basis index = string
    value (fermion mode m = basis bit m)."""
    from .sv import apply_pauli_sum

    idx = strings.astype(np.int64)

    def apply(ket):
        psi = np.zeros(1 << n, dtype=np.complex128)
        psi[idx] = ket
        out = apply_pauli_sum(psi, codes, coeffs)
        return np.real(out[idx])

    return apply
