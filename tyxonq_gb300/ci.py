"""CI-space UCC energies and gradients on the GPU.

The UCC state restricted to determinants with fixed alpha / beta electron
counts, as TyxonQ's civector engine keeps it
(applications/chem/chem_libs/quantum_chem_library/civector_ops.py, used by
``UCC.energy_and_grad(numeric_engine="civector")``): a real vector over the
CI strings, one signed permutation per excitation.  Host side here:

* CI strings (ci_state_mapping.py:38-115): per-spin bit patterns in
  ascending order (pyscf's cistring order for a contiguous orbital range),
  alpha in the high half, alpha-major;
* per-excitation tensors (civector_ops.py:436-483): determinant map
  ``fperm``, sign ``fphase`` including the fermion phase of
  pauli_io.py:169-206 (Z mask and sign of the first Jordan-Wigner word), and
  ``f2phase``.
The evolution, the reverse-sweep gradient and the dot products run in
``csrc/ci.cu``; the Hamiltonian is applied in the full statevector with the
Pauli-sum kernel and gathered back (H conserves the particle numbers).
"""
from __future__ import annotations

import ctypes
from itertools import combinations
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .chem import _ladder, _mul
from .hamiltonian import as_pauli_sum


def ci_strings(n_qubits: int, n_elec_s: tuple[int, int]) -> tuple[np.ndarray, np.ndarray, np.ndarray, int]:
    """(strings, alpha address table, beta address table, number of beta strings)."""
    na, nb = n_elec_s
    h = n_qubits // 2

    def make(ne):
        return np.array(sorted(sum(1 << i for i in occ) for occ in combinations(range(h), ne)), dtype=np.uint64)

    alpha, beta = make(na), make(nb)
    strings = ((alpha << np.uint64(h)).reshape(-1, 1) + beta.reshape(1, -1)).ravel()
    a2 = np.zeros(1 << h, dtype=np.int64)
    b2 = np.zeros(1 << h, dtype=np.int64)
    a2[alpha.astype(np.int64)] = np.arange(len(alpha))
    b2[beta.astype(np.int64)] = np.arange(len(beta))
    return strings, a2, b2, len(beta)


def _fermion_phase_mask_sign(f_idx: tuple, n_qubits: int) -> tuple[int, int]:
    """Z mask and sign of the first (openfermion-sorted) Jordan-Wigner word of
    a^dagger_f0 a_f1 or a^dagger_f0 a^dagger_f1 a_f2 a_f3 (pauli_io.py:169-191)."""
    ops = [(f_idx[0], True), (f_idx[1], False)] if len(f_idx) == 2 else \
        [(f_idx[0], True), (f_idx[1], True), (f_idx[2], False), (f_idx[3], False)]
    acc = {(0, 0): 1.0 + 0j}
    for m, cr in ops:
        acc = _mul(acc, _ladder(m, cr))
    words = []
    for (x, z), c in acc.items():
        if abs(c) < 1e-12:
            continue
        w = c * (-1j) ** bin(x & z).count("1")
        key = tuple((q, "Y" if (x >> q) & (z >> q) & 1 else ("X" if (x >> q) & 1 else "Z"))
                    for q in range(n_qubits) if ((x | z) >> q) & 1)
        words.append((key, w))
    key, w = min(words, key=lambda kv: kv[0])
    mask = sum(1 << q for q, p in key if p == "Z")
    return mask, (-1 if w.real > 0 else 1)


def operator_tensors(n_qubits: int, n_elec_s: tuple[int, int], ex_ops: Sequence[tuple]):
    """(strings, fperm int32 [n_ex, D], fphase int8, f2phase int8)."""
    strings, a2, b2, nbeta = ci_strings(n_qubits, n_elec_s)
    s = strings.astype(np.int64)
    h = n_qubits // 2
    n_ex, D = len(ex_ops), len(s)
    fperm = np.zeros((n_ex, D), dtype=np.int32)
    fphase = np.zeros((n_ex, D), dtype=np.int8)
    f2phase = np.zeros((n_ex, D), dtype=np.int8)
    for j, f in enumerate(ex_ops):
        f = tuple(int(x) for x in f)
        if len(set(f)) != len(f) or len(f) not in (2, 4):
            raise ValueError(f"Excitation {f} not supported")
        exc = s ^ sum(1 << i for i in f)
        fperm[j] = a2[exc >> h] * nbeta + b2[exc & ((1 << h) - 1)]
        m1, m2 = ((1 << f[0]), (1 << f[1])) if len(f) == 2 else ((1 << f[0]) + (1 << f[1]), (1 << f[2]) + (1 << f[3]))
        masked = (s ^ m1) & (m1 | m2)
        pos, neg = masked == (m1 | m2), masked == 0
        zmask, sign = _fermion_phase_mask_sign(f, n_qubits)
        par = np.bitwise_count((s & zmask).astype(np.uint64)) & 1
        ph = sign * np.where(par == 1, 1, -1)
        fphase[j] = (neg.astype(np.int64) - pos.astype(np.int64)) * ph
        f2phase[j] = -(pos.astype(np.int64) + neg.astype(np.int64))
    if fperm.size and (fperm.min() < 0 or fperm.max() >= D):
        raise ValueError("CI excitation map leaves the CI space")
    return strings, fperm, fphase, f2phase


class CIVectorUCC:
    """Energy and gradient of a UCC ansatz in CI space (real FP64 CI vector on
    the device; H applied through an n-qubit complex128 statevector)."""

    def __init__(self, n_qubits: int, n_elec_s: tuple[int, int], ex_ops: Sequence[tuple], param_ids: Sequence[int],
                 hamiltonian, device="cuda"):
        self.n = int(n_qubits)
        self.n_elec_s = (int(n_elec_s[0]), int(n_elec_s[1]))
        self.ex_ops = [tuple(int(x) for x in f) for f in ex_ops]
        self.param_ids = np.asarray(param_ids, dtype=np.int64)
        self.H = as_pauli_sum(hamiltonian, self.n)
        self.device = torch.device(device)
        strings, fperm, fphase, f2phase = operator_tensors(self.n, self.n_elec_s, self.ex_ops)
        self.D = len(strings)
        dev = self.device
        self.strings = torch.from_numpy(strings.astype(np.int64)).to(dev)
        self.fperm = torch.from_numpy(fperm).to(dev)
        self.fphase = torch.from_numpy(fphase).to(dev)
        self.f2phase = torch.from_numpy(f2phase).to(dev)
        self.ket = torch.zeros(self.D, dtype=torch.float64, device=dev)
        self.bra = torch.zeros_like(self.ket)
        self.tmp = torch.zeros_like(self.ket)
        self.psi = torch.zeros(1 << self.n, dtype=torch.complex128, device=dev)
        self.lam = torch.zeros_like(self.psi)

    def _angles(self, params):
        th = np.asarray(params, dtype=np.float64)[self.param_ids]
        s = np.ascontiguousarray(np.sin(th))
        omc = np.ascontiguousarray(1.0 - np.cos(th))
        return s, omc

    def civector(self, params) -> torch.Tensor:
        """The evolved CI vector (device FP64), from the first determinant."""
        P = ctypes.c_void_p
        st = K.stream_ptr(self.device)
        s, omc = self._angles(params)
        self.ket.zero_()
        self.ket[0] = 1.0
        nat.call("tq_ci_apply_excitations", P(self.ket.data_ptr()), P(self.tmp.data_ptr()), self.D,
                 P(self.fperm.data_ptr()), P(self.fphase.data_ptr()), P(self.f2phase.data_ptr()),
                 s.ctypes.data_as(P), omc.ctypes.data_as(P), len(self.ex_ops), 0, st)
        return self.ket

    def _apply_h(self, ket: torch.Tensor, out: torch.Tensor) -> None:
        P = ctypes.c_void_p
        st = K.stream_ptr(self.device)
        nat.call("tq_ci_embed", P(ket.data_ptr()), P(self.strings.data_ptr()), self.D, P(self.psi.data_ptr()),
                 self.n, 1, st)
        K.apply_pauli_sum(self.psi, self.H, out=self.lam)
        nat.call("tq_ci_gather", P(self.lam.data_ptr()), P(self.strings.data_ptr()), self.D, 1, P(out.data_ptr()), st)

    def energy(self, params) -> float:
        ket = self.civector(params)
        self._apply_h(ket, self.bra)
        return float(self._dot(self.bra, ket).item())

    def _dot(self, a, b) -> torch.Tensor:
        P = ctypes.c_void_p
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        lib = nat.load()
        ws, cap = K._ws(lib.tq_ci_dot_workspace_bytes(self.D), self.device)
        nat.call("tq_ci_dot", P(a.data_ptr()), P(b.data_ptr()), self.D, P(out.data_ptr()), ws, cap,
                 K.stream_ptr(self.device))
        return out

    def energy_and_grad(self, params) -> tuple[float, np.ndarray]:
        P = ctypes.c_void_p
        params = np.asarray(params, dtype=np.float64)
        ket = self.civector(params)
        self._apply_h(ket, self.bra)
        e = self._dot(self.bra, ket)
        s, omc = self._angles(params)
        n_ex = len(self.ex_ops)
        gj = torch.empty(max(n_ex, 1), dtype=torch.float64, device=self.device)
        lib = nat.load()
        ws, cap = K._ws(lib.tq_ci_adjoint_workspace_bytes(self.D, n_ex), self.device)
        nat.call("tq_ci_adjoint", P(ket.data_ptr()), P(self.bra.data_ptr()), self.D, P(self.fperm.data_ptr()),
                 P(self.fphase.data_ptr()), P(self.f2phase.data_ptr()), s.ctypes.data_as(P),
                 omc.ctypes.data_as(P), n_ex, P(gj.data_ptr()), ws, cap, K.stream_ptr(self.device))
        g = np.zeros_like(params)
        np.add.at(g, self.param_ids, gj[:n_ex].cpu().numpy())
        return float(e.item()), 2.0 * g
