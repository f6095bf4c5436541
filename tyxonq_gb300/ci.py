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
* H restricted to the CI space as a CSR matrix built from the Pauli sum
  (the operator the reference applies with apply_op).
* per-excitation pair lists: an excitation changes only the determinants
  with fphase != 0, which pair up as (i, fperm[i]) with opposite signs.
The evolution, H ket, the energy and the reverse-sweep gradient run in
``csrc/ci.cu``: when the vectors fit in one CTA's shared memory, a forward
and a reverse sweep over the pairs (one CTA each), H ket on many CTAs and an
ordered sum of the partials; else one launch per excitation step over the
whole vector.
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


def ci_hamiltonian_csr(strings: np.ndarray, H) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """H restricted to the CI space as CSR (row_ptr int64 [D+1], col int32,
    val float64): the operator TyxonQ's civector engine applies with
    ``apply_op`` (hamiltonian_builders.py:283-318; its CI-space form is the
    pyscf contraction of hamiltonian_builders.py:165-178).  Built from the
    Pauli sum: term c P with flip mask f and Z/Y mask zy maps determinant j =
    i ^ f to i with c i^ny (-1)^popcount(j & zy) (fermion mode m = basis bit
    m); H conserves the particle numbers, so every nonzero lands in the CI
    space.  Raises if an element is not real (the CI vector is real)."""
    s = np.asarray(strings, dtype=np.uint64)
    D = len(s)
    flip, zy, ny = H.masks()
    coef = np.asarray(H.coeffs, dtype=np.float64) * (1j ** (ny % 4))
    order = np.argsort(flip, kind="stable")
    fs = flip[order]
    starts = np.flatnonzero(np.r_[True, fs[1:] != fs[:-1]]) if len(fs) else np.zeros(0, np.int64)
    ends = np.r_[starts[1:], len(fs)]
    rows, cols, vals = [], [], []
    for a, b in zip(starts, ends):
        ids = order[a:b]
        src = s ^ fs[a]
        j = np.minimum(np.searchsorted(s, src), D - 1)
        ok = np.flatnonzero(s[j] == src)
        if not len(ok):
            continue
        par = np.bitwise_count(src[ok, None] & zy[None, ids]) & 1
        v = ((1 - 2 * par.astype(np.int64)) * coef[None, ids]).sum(axis=1)
        if np.abs(v.imag).max() > 1e-10 * max(1.0, np.abs(v.real).max()):
            raise ValueError("Hamiltonian is not real in the CI space")
        keep = v.real != 0.0
        rows.append(ok[keep])
        cols.append(j[ok[keep]])
        vals.append(v.real[keep])
    r = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    c = np.concatenate(cols) if cols else np.zeros(0, np.int64)
    v = np.concatenate(vals) if vals else np.zeros(0, np.float64)
    o = np.lexsort((c, r))
    row_ptr = np.zeros(D + 1, dtype=np.int64)
    np.add.at(row_ptr, r + 1, 1)
    return np.cumsum(row_ptr), c[o].astype(np.int32), v[o]


CI_SWEEP_THREADS = 1024  # largest CTA of the one-CTA sweeps in csrc/ci.cu


def sweep_threads(max_pairs: int) -> int:
    """CTA size of the sweeps: 256 (a shorter per-excitation barrier) when no
    excitation has more than 512 pairs, else 1024."""
    return 256 if max_pairs <= 512 else CI_SWEEP_THREADS


def excitation_pairs(fperm: np.ndarray, fphase: np.ndarray, f2phase: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(pairs int32 [total, 2], pair_start int64 [n_ex + 1]): for each
    excitation the determinants it changes, as pairs {i, (p << 1) | (fphase[i]
    < 0)} with p = fperm[i] > i (the layout tq_ci_energy_grad reads).  Checks
    the structure the pair form relies on: the changed determinants are
    exactly those with fphase != 0, fperm swaps each pair, fphase[p] =
    -fphase[i] and f2phase = -1 on both."""
    n_ex = fperm.shape[0]
    recs, starts = [], [0]
    for j in range(n_ex):
        i = np.flatnonzero(fphase[j] != 0)
        p = fperm[j, i].astype(np.int64)
        ok = (np.array_equal(fperm[j, p], i) and np.array_equal(fphase[j, p], -fphase[j, i])
              and np.all(f2phase[j, i] == -1) and np.all(f2phase[j][fphase[j] == 0] == 0))
        if not ok:
            raise ValueError(f"excitation {j}: changed determinants do not form sign-reversing pairs")
        keep = i < p
        rec = np.empty((int(keep.sum()), 2), dtype=np.int32)
        rec[:, 0] = i[keep]
        rec[:, 1] = (p[keep] << 1) | (fphase[j, i[keep]] < 0)
        recs.append(rec)
        starts.append(starts[-1] + len(rec))
    pairs = np.concatenate(recs) if recs else np.zeros((0, 2), dtype=np.int32)
    return pairs, np.asarray(starts, dtype=np.int64)


def partial_starts(D: int, pair_start: np.ndarray, threads: int = CI_SWEEP_THREADS) -> np.ndarray:
    """part_start of tq_ci_energy_grad: the energy's partial sums, then each
    excitation's gradient partials (one per sweep thread that holds a pair)."""
    cnt = np.r_[min(D, threads), np.minimum(np.diff(pair_start), threads)]
    return np.r_[0, np.cumsum(cnt)].astype(np.int64)


class CIVectorUCC:
    """Energy and gradient of a UCC ansatz in CI space: real FP64 CI vector,
    H as a CSR matrix over the CI strings.  Up to tq_ci_pairs_max_dim
    determinants the sweeps run in one CTA each with the vectors in shared
    memory and touch only the determinant pairs each excitation changes
    (tq_ci_energy_grad, four launches per evaluation); above it, one launch
    per excitation step over the whole vector."""

    def __init__(self, n_qubits: int, n_elec_s: tuple[int, int], ex_ops: Sequence[tuple], param_ids: Sequence[int],
                 hamiltonian, device="cuda", fused: bool | None = None):
        self.n = int(n_qubits)
        self.n_elec_s = (int(n_elec_s[0]), int(n_elec_s[1]))
        self.ex_ops = [tuple(int(x) for x in f) for f in ex_ops]
        self.param_ids = np.asarray(param_ids, dtype=np.int64)
        self.H = as_pauli_sum(hamiltonian, self.n)
        self.device = torch.device(device)
        strings, fperm, fphase, f2phase = operator_tensors(self.n, self.n_elec_s, self.ex_ops)
        self.D = len(strings)
        self.n_ex = len(self.ex_ops)
        dev = self.device
        lib = nat.load()
        pairs, pair_start = excitation_pairs(fperm, fphase, f2phase)
        self.max_pairs = int(np.diff(pair_start).max()) if self.n_ex else 0
        limit = lib.tq_ci_pairs_max_dim(self.n_ex)
        can_fuse = self.D <= limit and self.max_pairs <= 2 * CI_SWEEP_THREADS
        if fused and not can_fuse:
            raise ValueError(f"{self.D} determinants exceed the one-CTA limit {limit}")
        self.fused = can_fuse if fused is None else bool(fused)
        rp, col, val = ci_hamiltonian_csr(strings, self.H)
        self.row_ptr = torch.from_numpy(rp).to(dev)
        self.col = torch.from_numpy(col).to(dev)
        self.val = torch.from_numpy(val).to(dev)
        self.strings = torch.from_numpy(strings.astype(np.int64)).to(dev)
        if self.fused:
            self.threads = sweep_threads(self.max_pairs)
            part_start = partial_starts(self.D, pair_start, self.threads)
            self.n_partials = int(part_start[-1])
            self.pairs = torch.from_numpy(pairs).to(dev)
            self.pair_start = torch.from_numpy(pair_start).to(dev)
            self.part_start = torch.from_numpy(part_start).to(dev)
        else:
            self.fperm = torch.from_numpy(fperm).to(dev)
            self.fphase = torch.from_numpy(fphase).to(dev)
            self.f2phase = torch.from_numpy(f2phase).to(dev)
            self.tmp = torch.zeros(self.D, dtype=torch.float64, device=dev)
        self.sin_omc = torch.zeros(max(2 * self.n_ex, 2), dtype=torch.float64, device=dev)
        self._sin_omc_host = torch.zeros(self.sin_omc.shape, dtype=torch.float64, pin_memory=dev.type == "cuda")
        self._copied = None  # event after the last host -> device angle copy
        self.ket = torch.zeros(self.D, dtype=torch.float64, device=dev)
        self.bra = torch.zeros_like(self.ket)
        self.out = torch.zeros(1 + max(self.n_ex, 1), dtype=torch.float64, device=dev)  # energy, grads

    def _angles(self, params):
        th = np.asarray(params, dtype=np.float64)[self.param_ids]
        s = np.ascontiguousarray(np.sin(th))
        omc = np.ascontiguousarray(1.0 - np.cos(th))
        return s, omc

    def _upload_angles(self, params):
        s, omc = self._angles(params)
        if self._copied is not None:
            self._copied.synchronize()  # the staging buffer is free again
        h = self._sin_omc_host.numpy()
        h[0:2 * self.n_ex:2] = s
        h[1:2 * self.n_ex:2] = omc
        self.sin_omc.copy_(self._sin_omc_host, non_blocking=True)
        self._copied = torch.cuda.Event()
        self._copied.record()
        return s, omc

    def _fused(self, params, grad: bool) -> None:
        P = ctypes.c_void_p
        self._upload_angles(params)
        lib = nat.load()
        ws, cap = K._ws(lib.tq_ci_energy_grad_workspace_bytes(self.D, self.n_partials), self.device)
        nat.call("tq_ci_energy_grad", self.D, 0, self.n_ex, P(self.pairs.data_ptr()), P(self.pair_start.data_ptr()),
                 self.max_pairs, P(self.part_start.data_ptr()), self.n_partials, P(self.sin_omc.data_ptr()),
                 P(self.row_ptr.data_ptr()), P(self.col.data_ptr()), P(self.val.data_ptr()), int(grad), self.threads,
                 P(self.ket.data_ptr()), P(self.out.data_ptr()), ws, cap, K.stream_ptr(self.device))

    def _evolve(self, params) -> None:
        P = ctypes.c_void_p
        s, omc = self._angles(params)
        self.ket.zero_()
        self.ket[0] = 1.0
        nat.call("tq_ci_apply_excitations", P(self.ket.data_ptr()), P(self.tmp.data_ptr()), self.D,
                 P(self.fperm.data_ptr()), P(self.fphase.data_ptr()), P(self.f2phase.data_ptr()),
                 s.ctypes.data_as(P), omc.ctypes.data_as(P), self.n_ex, 0, K.stream_ptr(self.device))

    def _apply_h(self, ket: torch.Tensor, out: torch.Tensor) -> None:
        P = ctypes.c_void_p
        nat.call("tq_ci_spmv", P(self.row_ptr.data_ptr()), P(self.col.data_ptr()), P(self.val.data_ptr()), self.D,
                 P(ket.data_ptr()), P(out.data_ptr()), K.stream_ptr(self.device))

    def _dot(self, a, b, out: torch.Tensor) -> None:
        P = ctypes.c_void_p
        lib = nat.load()
        ws, cap = K._ws(lib.tq_ci_dot_workspace_bytes(self.D), self.device)
        nat.call("tq_ci_dot", P(a.data_ptr()), P(b.data_ptr()), self.D, P(out.data_ptr()), ws, cap,
                 K.stream_ptr(self.device))

    def civector(self, params) -> torch.Tensor:
        """The evolved CI vector (device FP64), from the first determinant."""
        if self.fused:
            self._fused(params, grad=False)
        else:
            self._evolve(params)
        return self.ket

    def energy(self, params) -> float:
        if self.fused:
            self._fused(params, grad=False)
        else:
            self._evolve(params)
            self._apply_h(self.ket, self.bra)
            self._dot(self.bra, self.ket, self.out)
        return float(self.out[0].item())

    def energy_and_grad(self, params) -> tuple[float, np.ndarray]:
        P = ctypes.c_void_p
        params = np.asarray(params, dtype=np.float64)
        if self.fused:
            self._fused(params, grad=True)
        else:
            self._evolve(params)
            self._apply_h(self.ket, self.bra)
            self._dot(self.bra, self.ket, self.out)
            s, omc = self._angles(params)
            if self.n_ex:
                lib = nat.load()
                ws, cap = K._ws(lib.tq_ci_adjoint_workspace_bytes(self.D, self.n_ex), self.device)
                nat.call("tq_ci_adjoint", P(self.ket.data_ptr()), P(self.bra.data_ptr()), self.D,
                         P(self.fperm.data_ptr()), P(self.fphase.data_ptr()), P(self.f2phase.data_ptr()),
                         s.ctypes.data_as(P), omc.ctypes.data_as(P), self.n_ex, P(self.out.data_ptr() + 8), ws, cap,
                         K.stream_ptr(self.device))
        res = self.out.cpu().numpy()
        g = np.zeros_like(params)
        np.add.at(g, self.param_ids, res[1:1 + self.n_ex])
        return float(res[0]), 2.0 * g
