"""UCCSD energy / gradient workload on the GPU engine.

Restates the parts of TyxonQ's chemistry stack the UCCSD statevector path
needs (TyxonQ takes them from openfermion / pyscf, which are not used here):

* integrals -> second-quantised H, following ``get_hop_from_integral``
  (chem_libs/hamiltonians_chem_library/hamiltonian_builders.py:71-108) and
  ``symmetrize_int2e`` (:270-277);
* Jordan-Wigner with a Z string on lower modes (openfermion's convention), and
  TyxonQ's index reversal: fermion mode m acts on qubit n-1-m
  (``reverse_qop_idx``, libs/hamiltonian_encoding/pauli_io.py:87-93), which is
  basis-index bit m;
* UCCSD excitation lists in TyxonQ's order (``UCC.get_ex1_ops`` /
  ``get_ex2_ops``, applications/chem/algorithms/ucc.py:680-832);
* the trotterised ansatz: each excitation's anti-Hermitian JW generator
  i*sum_k v_k P_k becomes one Pauli rotation per string with angle
  -2 v_k theta (circuits_library/ucc.py:111-117), all strings of one
  excitation commute, so the product is exp(theta (T - T^dagger)) exactly;
* the Hartree-Fock start bitstring of ``get_init_circuit``
  (chem_libs/quantum_chem_library/statevector_ops.py:172-199).
Pauli algebra runs on (x, z) bit masks: X^x Z^z, with
(X^x1 Z^z1)(X^x2 Z^z2) = (-1)^{popc(z1 & x2)} X^{x1^x2} Z^{z1^z2}.
"""
from __future__ import annotations

from collections import defaultdict
from itertools import product

import numpy as np

from .hamiltonian import PauliSum


# ---------------------------------------------------------------- integrals
def symmetrize_int2e(int2e: np.ndarray) -> np.ndarray:
    g = 0.25 * (int2e + int2e.transpose((0, 1, 3, 2)) + int2e.transpose((1, 0, 2, 3)) + int2e.transpose((2, 3, 0, 1)))
    return 0.5 * (g + g.transpose(3, 2, 1, 0))


def random_integrals(n_orb: int, seed: int = 7, sigma1: float = 1.0, sigma2: float = 0.1):
    """h_pq ~ N(0, sigma1^2) symmetric, g_pqrs ~ N(0, sigma2^2) with 8-fold symmetry."""
    rng = np.random.default_rng(seed)
    h = rng.normal(0, sigma1, (n_orb, n_orb))
    h = 0.5 * (h + h.T)
    g = symmetrize_int2e(rng.normal(0, sigma2, (n_orb,) * 4))
    return h, g


def fermion_terms(int1e: np.ndarray, int2e: np.ndarray) -> list:
    """[(coeff, ((mode, is_creation), ...))] as get_hop_from_integral builds them."""
    n_orb = int1e.shape[0]
    ns = 2 * n_orb
    h1e = np.zeros((ns, ns))
    h2e = np.zeros((ns, ns, ns, ns))
    h1e[:n_orb, :n_orb] = h1e[n_orb:, n_orb:] = int1e
    for p, q, r, s in product(range(ns), repeat=4):
        if ((p < n_orb) == (s < n_orb)) and ((q < n_orb) == (r < n_orb)):
            h2e[p, q, r, s] = int2e[p % n_orb, s % n_orb, q % n_orb, r % n_orb]
    out = []
    for p, q in product(range(ns), repeat=2):
        v = h1e[p, q]
        if abs(v) >= 1e-12:
            out.append((v, ((p, True), (q, False))))
    for q, s in product(range(ns), repeat=2):
        for p, r in product(range(q), range(s)):
            v = h2e[p, q, r, s] - h2e[q, p, r, s]
            if abs(v) >= 1e-12:
                out.append((v, ((p, True), (q, True), (r, False), (s, False))))
    return out


# ---------------------------------------------------------------- Jordan-Wigner
def _ladder(m: int, creation: bool) -> dict:
    """a^dagger_m = (X_m + X_m Z_m)/2 Z_{<m};  a_m = (X_m - X_m Z_m)/2 Z_{<m}."""
    low = (1 << m) - 1
    x = 1 << m
    s = 0.5 if creation else -0.5
    return {(x, low): 0.5, (x, low | x): s}


def _mul(A: dict, B: dict) -> dict:
    out: dict = defaultdict(complex)
    for (x1, z1), c1 in A.items():
        for (x2, z2), c2 in B.items():
            sign = -1.0 if bin(z1 & x2).count("1") & 1 else 1.0
            out[(x1 ^ x2, z1 ^ z2)] += sign * c1 * c2
    return out


def jordan_wigner(terms: list) -> dict:
    """sum of fermion products -> {(x, z): coeff} in the X^x Z^z basis."""
    total: dict = defaultdict(complex)
    for c, ops in terms:
        acc = {(0, 0): complex(c)}
        for m, cr in ops:
            acc = _mul(acc, _ladder(m, cr))
        for k, v in acc.items():
            total[k] += v
    return {k: v for k, v in total.items() if abs(v) > 1e-12}


def _word_coeff(x: int, z: int, c: complex) -> complex:
    """Coefficient of the Pauli word (Y where x and z overlap) for c * X^x Z^z."""
    ny = bin(x & z).count("1")
    return c * (-1j) ** ny


def to_pauli_sum(xz: dict, n: int, tol: float = 1e-10) -> PauliSum:
    codes, coeffs = [], []
    for (x, z), c in sorted(xz.items()):
        w = _word_coeff(x, z, c)
        if abs(w.imag) > tol:
            raise ValueError("Hamiltonian is not Hermitian in the Pauli basis")
        if abs(w.real) < 1e-12:
            continue
        row = np.zeros(n, dtype=np.int8)
        for m in range(n):
            xb, zb = (x >> m) & 1, (z >> m) & 1
            row[n - 1 - m] = 0 if not (xb or zb) else (1 if xb and not zb else (2 if xb and zb else 3))
        codes.append(row)
        coeffs.append(w.real)
    return PauliSum(n, np.array(codes, dtype=np.int8).reshape(-1, n), np.array(coeffs))


def molecular_hamiltonian(int1e: np.ndarray, int2e: np.ndarray) -> PauliSum:
    n = 2 * int1e.shape[0]
    return to_pauli_sum(jordan_wigner(fermion_terms(int1e, int2e)), n)


# ---------------------------------------------------------------- UCCSD
def uccsd_excitations(no: int, nv: int) -> tuple[list, list]:
    """(excitation tuples, parameter ids) in the order of get_ex1_ops + get_ex2_ops."""
    ex, pid = [], []
    nxt = 0
    for i in range(no):
        for a in range(nv):
            ex += [(2 * no + nv + a, no + nv + i), (no + a, i)]
            pid += [nxt, nxt]
            nxt += 1
    av = lambda k: 2 * no + nv + k  # noqa: E731
    ao = lambda k: no + nv + k  # noqa: E731
    bo = lambda k: k  # noqa: E731
    bv = lambda k: no + k  # noqa: E731
    for i in range(no):
        for j in range(i):
            for a in range(nv):
                for b in range(a):
                    ex += [(av(b), av(a), ao(i), ao(j)), (bv(b), bv(a), bo(i), bo(j))]
                    pid += [nxt, nxt]
                    nxt += 1
    for i in range(no):
        for j in range(i + 1):
            for a in range(nv):
                for b in range(a + 1):
                    if i == j and a == b:
                        ex.append((bv(a), av(a), ao(i), bo(i)))
                        pid.append(nxt)
                        nxt += 1
                        continue
                    ex += [(bv(b), av(a), ao(i), bo(j)), (av(b), bv(a), bo(i), ao(j))]
                    pid += [nxt, nxt]
                    nxt += 1
                    if i != j and a != b:
                        ex += [(bv(a), av(b), ao(i), bo(j)), (av(a), bv(b), bo(i), ao(j))]
                        pid += [nxt, nxt]
                        nxt += 1
    return ex, pid


def excitation_generator(ex_op: tuple) -> dict:
    """JW of T - T^dagger for 'p^ q' or 'p^ q^ r s' (ex_op_to_fop with conjugation)."""
    if len(ex_op) == 2:
        p, q = ex_op
        T = [(1.0, ((p, True), (q, False)))]
        Td = [(-1.0, ((q, True), (p, False)))]
    else:
        p, q, r, s = ex_op
        T = [(1.0, ((p, True), (q, True), (r, False), (s, False)))]
        Td = [(-1.0, ((s, True), (r, True), (q, False), (p, False)))]
    return jordan_wigner(T + Td)


def excitation_rotations(ex_op: tuple, n: int) -> list[tuple[tuple, float]]:
    """[(pauli [(qubit, 'X'|'Y'|'Z')...], scale)] with each rotation angle = scale * theta."""
    out = []
    for (x, z), c in sorted(excitation_generator(ex_op).items()):
        w = _word_coeff(x, z, c)
        if abs(w.real) > 1e-10:
            raise ValueError("excitation generator is not anti-Hermitian")
        if abs(w.imag) < 1e-12:
            continue
        pauli = []
        for m in range(n):
            xb, zb = (x >> m) & 1, (z >> m) & 1
            if xb or zb:
                pauli.append((n - 1 - m, "X" if xb and not zb else ("Y" if xb and zb else "Z")))
        out.append((tuple(sorted(pauli)), -2.0 * w.imag))
    return out


def hf_basis(n_qubits: int, no: int) -> int:
    """Basis index of the HF state: occupied beta modes 0..no-1 and alpha modes
    n/2..n/2+no-1 (mode m = basis bit m)."""
    b = 0
    for i in range(no):
        b |= 1 << i
        b |= 1 << (n_qubits // 2 + i)
    return b


def uccsd_param_gates(n_orb: int, n_elec: int, one_param_per_excitation: bool = True):
    """(ParamGate list, number of parameters, excitations) of the trotterised UCCSD ansatz."""
    from .adjoint import ParamGate
    from .ir import pauli_rotation

    no = n_elec // 2
    nv = n_orb - no
    n = 2 * n_orb
    ex, pid = uccsd_excitations(no, nv)
    if one_param_per_excitation:
        pid = list(range(len(ex)))
    pg = []
    for e, p in zip(ex, pid):
        for pauli, sc in excitation_rotations(e, n):
            pg.append(ParamGate(pauli_rotation(pauli, 0.0), p, sc))
    return pg, max(pid) + 1, ex
