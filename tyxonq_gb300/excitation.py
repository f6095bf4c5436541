"""UCC excitations applied exactly on the statevector.

TyxonQ's numeric UCC statevector engine (chem_libs/quantum_chem_library/
statevector_ops.py:66-168, ``get_statevector`` / ``evolve_excitation``)
evolves psi <- psi + (1 - cos t) F^2 psi + sin t F psi per excitation with
F = T - T^dagger, and differentiates with autograd.  F changes only the basis
states whose excitation bits match one of two patterns; those pair up and
exp(t F) rotates each pair (``tq_excitation`` in include/tq_sv.h).  The GPU
path here applies one such pair rotation per excitation over 2^(n-k) pairs
(k = 2 or 4 excitation bits) and differentiates with a reverse sweep
(``tq_sv_excitation_adjoint``), instead of 2 or 8 Pauli rotations over all
amplitudes per excitation.  Fermion mode m is basis bit m (qubit n-1-m), as in
the reference's reversed wires.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .hamiltonian import as_pauli_sum

EXCITATION_DTYPE = np.dtype([("m_neg", "<u8"), ("m_pos", "<u8"), ("zmask", "<u8"), ("sign", "<i4"), ("k", "<i4"),
                             ("bits", "<i4", (4,))])


def excitation_records(n_qubits: int, ex_ops: Sequence[tuple]) -> np.ndarray:
    """tq_excitation records of the excitations 'p^ q' (2 indices) or
    'p^ q^ r s' (4): m_neg = the bits of the annihilated-side pattern
    (f0 | f1 for doubles, f0 for singles) the civector tensors call m1, m_pos
    the other bits, and the Jordan-Wigner Z mask and sign of
    pauli_io.py:169-206."""
    from .ci import _fermion_phase_mask_sign

    out = np.zeros(len(ex_ops), dtype=EXCITATION_DTYPE)
    for j, f in enumerate(ex_ops):
        f = tuple(int(x) for x in f)
        if len(f) not in (2, 4) or len(set(f)) != len(f) or min(f) < 0 or max(f) >= n_qubits:
            raise ValueError(f"Excitation {f} not supported on {n_qubits} qubits")
        if len(f) == 2:
            m1, m2 = 1 << f[0], 1 << f[1]
        else:
            m1, m2 = (1 << f[0]) | (1 << f[1]), (1 << f[2]) | (1 << f[3])
        zmask, sign = _fermion_phase_mask_sign(f, n_qubits)
        if zmask & (m1 | m2):
            raise ValueError(f"Excitation {f}: Z string overlaps the excitation bits")
        bits = sorted(f)
        out[j]["m_neg"], out[j]["m_pos"], out[j]["zmask"] = m1, m2, zmask
        out[j]["sign"], out[j]["k"] = sign, len(f)
        out[j]["bits"][:len(f)] = bits
    return out


class ExcitationEstimator:
    """Energy and adjoint gradient of a UCC ansatz given as excitations
    (one angle theta[param_ids[j]] each), from a basis state, on an n-qubit
    complex64 / complex128 statevector."""

    def __init__(self, n: int, ex_ops: Sequence[tuple], param_ids: Sequence[int], n_params: int, hamiltonian,
                 dtype=torch.complex64, device="cuda", init_basis: int = 0):
        self.n = int(n)
        self.ex_ops = [tuple(int(x) for x in f) for f in ex_ops]
        self.param_ids = np.asarray(param_ids, dtype=np.int64)
        if len(self.param_ids) != len(self.ex_ops):
            raise ValueError("one parameter index per excitation")
        self.n_params = int(n_params)
        self.n_ex = len(self.ex_ops)
        self.H = as_pauli_sum(hamiltonian, self.n)
        self.dtype = dtype
        self.device = torch.device(device)
        self.init_basis = int(init_basis)
        rec = excitation_records(self.n, self.ex_ops)
        self.records = torch.from_numpy(rec.view(np.uint8).copy()).to(self.device)
        self.sincos = torch.zeros(max(2 * self.n_ex, 2), dtype=torch.float64, device=self.device)
        self._sincos_host = torch.zeros(self.sincos.shape, dtype=torch.float64,
                                        pin_memory=self.device.type == "cuda")
        self._copied = None
        self.psi = torch.empty(1 << self.n, dtype=dtype, device=self.device)
        self.lam = torch.empty_like(self.psi)
        self.grads = torch.zeros(max(self.n_ex, 1), dtype=torch.float64, device=self.device)
        self._graphs: dict = {}

    def _upload(self, params) -> None:
        th = np.asarray(params, dtype=np.float64)[self.param_ids]
        if self._copied is not None:
            self._copied.synchronize()  # the staging buffer is free again
        h = self._sincos_host.numpy()
        h[0:2 * self.n_ex:2] = np.sin(th)
        h[1:2 * self.n_ex:2] = np.cos(th)
        self.sincos.copy_(self._sincos_host, non_blocking=True)
        self._copied = torch.cuda.Event()
        self._copied.record()

    def _evolve(self) -> None:
        P = ctypes.c_void_p
        st = K.stream_ptr(self.device)
        nat.call("tq_sv_init_basis", P(self.psi.data_ptr()), self.n, K.dtype_tag(self.psi), self.init_basis, st)
        nat.call("tq_sv_apply_excitations", P(self.psi.data_ptr()), self.n, K.dtype_tag(self.psi),
                 P(self.records.data_ptr()), self.n_ex, P(self.sincos.data_ptr()), 0, st)

    def _launch(self, grad: bool) -> torch.Tensor:
        """Forward, <H> (and H psi + reverse sweep); angles from self.sincos."""
        P = ctypes.c_void_p
        self._evolve()
        if not grad:
            return K.pauli_expectation(self.psi, self.H)
        K.apply_pauli_sum(self.psi, self.H, out=self.lam)
        e = K.inner_re(self.psi, self.lam)
        if self.n_ex:
            lib = nat.load()
            ws, cap = K._ws(lib.tq_sv_excitation_adjoint_workspace_bytes(self.n, self.n_ex), self.device)
            nat.call("tq_sv_excitation_adjoint", P(self.psi.data_ptr()), P(self.lam.data_ptr()), self.n,
                     K.dtype_tag(self.psi), P(self.records.data_ptr()), self.n_ex, P(self.sincos.data_ptr()),
                     P(self.grads.data_ptr()), ws, cap, K.stream_ptr(self.device))
        return e

    def _replay(self, grad: bool) -> torch.Tensor:
        """Run _launch as a CUDA graph (captured on first use: some 400 small
        launches per evaluation, one per excitation and sweep)."""
        if self.device.type != "cuda":
            return self._launch(grad)
        key = bool(grad)
        hit = self._graphs.get(key)
        if hit is None:
            self._launch(grad)  # warm-up outside capture: workspaces, shared-memory attributes
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                out = self._launch(grad)
            hit = self._graphs[key] = (g, out)
        hit[0].replay()
        return hit[1]

    def state(self, params) -> torch.Tensor:
        """The evolved statevector (device tensor, reused across calls)."""
        self._upload(params)
        self._evolve()
        return self.psi

    def energy(self, params) -> float:
        self._upload(params)
        return float(self._replay(False).item())

    def energy_and_grad(self, params) -> tuple[float, np.ndarray]:
        params = np.asarray(params, dtype=np.float64)
        self._upload(params)
        e = self._replay(True)
        gj = self.grads[:self.n_ex].cpu().numpy()
        g = np.zeros(self.n_params)
        np.add.at(g, self.param_ids, gj)
        return float(e.item()), 2.0 * g
