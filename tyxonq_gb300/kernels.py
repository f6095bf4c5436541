"""Statevector kernels on CUDA torch tensors (GPU counterpart of
tyxonq/libs/quantum_library/kernels/statevector.py).

Each function validates its arguments, picks the tensor's device and the
current torch stream, and calls the C ABI of libtyxonq_gb300.so.  Unlike the
reference (which returns a fresh array per gate), gates update the state in
place and return the same tensor.  States are 1-D contiguous complex64 or
complex128 CUDA tensors of length 2^n.
"""
from __future__ import annotations

import ctypes
import math
import threading
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from .hamiltonian import PauliSum, as_pauli_sum

_DT = {torch.complex64: nat.TQ_C64, torch.complex128: nat.TQ_C128}


def dtype_tag(t: torch.Tensor) -> int:
    try:
        return _DT[t.dtype]
    except KeyError:
        raise TypeError(f"state dtype must be complex64 or complex128, got {t.dtype}") from None


def _check_state(psi: torch.Tensor, n: int | None = None) -> int:
    if not isinstance(psi, torch.Tensor) or not psi.is_cuda:
        raise TypeError("state must be a CUDA torch tensor")
    if psi.dim() != 1 or not psi.is_contiguous():
        raise ValueError("state must be a contiguous 1-D tensor")
    N = psi.numel()
    nn = N.bit_length() - 1
    if N != (1 << nn):
        raise ValueError(f"state length {N} is not a power of two")
    if n is not None and int(n) != nn:
        raise ValueError(f"state has {nn} qubits, caller said {n}")
    return nn


def stream_ptr(device=None) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


# ---------------------------------------------------------------- workspace
class _Workspace:
    """Grow-only scratch buffer per (device, stream); callers on one stream
    reuse one allocation, so stream order makes reuse safe."""

    def __init__(self):
        self._bufs: dict = {}
        self._lock = threading.Lock()

    def get(self, nbytes: int, device) -> torch.Tensor:
        dev = torch.device(device)
        key = (dev.index, torch.cuda.current_stream(dev).cuda_stream)
        with self._lock:
            buf = self._bufs.get(key)
            if buf is None or buf.numel() < nbytes:
                buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
                self._bufs[key] = buf
            return buf


workspace = _Workspace()


def _ws(nbytes: int, device) -> tuple[ctypes.c_void_p, int]:
    buf = workspace.get(nbytes, device)
    return _ptr(buf), buf.numel()


# ---------------------------------------------------------------- state prep
def init_statevector(num_qubits: int, dtype=torch.complex64, device="cuda", basis_index: int = 0) -> torch.Tensor:
    """|basis_index> (init_statevector, statevector.py:19-25)."""
    n = int(num_qubits)
    if n < 0 or n > nat.TQ_MAX_QUBITS:
        raise ValueError(f"num_qubits {n} outside [0, {nat.TQ_MAX_QUBITS}]")
    psi = torch.empty(1 << n, dtype=dtype, device=device)
    nat.call("tq_sv_init_basis", _ptr(psi), n, dtype_tag(psi), int(basis_index), stream_ptr(psi.device))
    return psi


def from_array(state, dtype=torch.complex64, device="cuda") -> torch.Tensor:
    """Copy a host/numpy/torch state vector onto the device (custom initial state)."""
    t = torch.as_tensor(np.asarray(state) if not isinstance(state, torch.Tensor) else state)
    t = t.reshape(-1).to(device=device, dtype=dtype).contiguous()
    _check_state(t)
    return t


# ---------------------------------------------------------------- gates
def _mat(u, size: int) -> ctypes.Array:
    a = np.asarray(u, dtype=np.complex128).reshape(size, size)
    return nat.dbl_array(np.stack([a.real, a.imag], axis=-1).reshape(-1))


def apply_1q(psi: torch.Tensor, u, qubit: int) -> torch.Tensor:
    """Dense 2x2 on `qubit` (apply_1q_statevector, statevector.py:28-42)."""
    n = _check_state(psi)
    nat.call("tq_sv_apply_1q", _ptr(psi), n, dtype_tag(psi), int(qubit), _mat(u, 2), stream_ptr(psi.device))
    return psi


def apply_diag1(psi: torch.Tensor, d0: complex, d1: complex, qubit: int) -> torch.Tensor:
    n = _check_state(psi)
    d = nat.dbl_array([complex(d0).real, complex(d0).imag, complex(d1).real, complex(d1).imag])
    nat.call("tq_sv_apply_diag1", _ptr(psi), n, dtype_tag(psi), int(qubit), d, stream_ptr(psi.device))
    return psi


def apply_2q(psi: torch.Tensor, u, q0: int, q1: int) -> torch.Tensor:
    """Dense 4x4, q0 = high index bit (apply_2q_statevector, statevector.py:45-59)."""
    n = _check_state(psi)
    nat.call("tq_sv_apply_2q", _ptr(psi), n, dtype_tag(psi), int(q0), int(q1), _mat(u, 4), stream_ptr(psi.device))
    return psi


def apply_cx(psi: torch.Tensor, c: int, t: int) -> torch.Tensor:
    n = _check_state(psi)
    nat.call("tq_sv_apply_cx", _ptr(psi), n, dtype_tag(psi), int(c), int(t), stream_ptr(psi.device))
    return psi


def apply_cz(psi: torch.Tensor, a: int, b: int) -> torch.Tensor:
    n = _check_state(psi)
    nat.call("tq_sv_apply_cz", _ptr(psi), n, dtype_tag(psi), int(a), int(b), stream_ptr(psi.device))
    return psi


def apply_swap(psi: torch.Tensor, a: int, b: int) -> torch.Tensor:
    n = _check_state(psi)
    nat.call("tq_sv_apply_swap", _ptr(psi), n, dtype_tag(psi), int(a), int(b), stream_ptr(psi.device))
    return psi


def apply_kq(psi: torch.Tensor, u, qubits: Sequence[int]) -> torch.Tensor:
    """Dense 2^k unitary, qubits[0] = high index bit (apply_kqubit_unitary,
    statevector.py:71-129)."""
    n = _check_state(psi)
    qs = [int(q) for q in qubits]
    k = len(qs)
    if k == 0:
        return psi
    nat.call("tq_sv_apply_kq", _ptr(psi), n, dtype_tag(psi), nat.int_array(qs), k, _mat(u, 1 << k),
             stream_ptr(psi.device))
    return psi


def pauli_masks(n: int, pauli: Sequence[tuple[int, str]]) -> tuple[int, int]:
    """(x_mask, z_mask) of a Pauli string [(qubit, 'X'|'Y'|'Z'), ...]."""
    xm = zm = 0
    for q, p in pauli:
        b = 1 << (n - 1 - int(q))
        p = str(p).upper()
        if p in ("X", "Y"):
            xm |= b
        if p in ("Y", "Z"):
            zm |= b
    return xm, zm


def apply_pauli_rotation(psi: torch.Tensor, pauli: Sequence[tuple[int, str]], theta: float) -> torch.Tensor:
    """exp(-i theta/2 P): the unitary of evolve_pauli_ops (circuits_library/utils.py:29-59)."""
    n = _check_state(psi)
    xm, zm = pauli_masks(n, pauli)
    nat.call("tq_sv_apply_pauli_rotation", _ptr(psi), n, dtype_tag(psi), xm, zm, float(theta), stream_ptr(psi.device))
    return psi


def scale(psi: torch.Tensor, factor: complex) -> torch.Tensor:
    n = _check_state(psi)
    f = complex(factor)
    nat.call("tq_sv_scale", _ptr(psi), n, dtype_tag(psi), f.real, f.imag, stream_ptr(psi.device))
    return psi


def project_z(psi: torch.Tensor, qubit: int, keep: int) -> torch.Tensor:
    """Zero the amplitudes with qubit != keep and renormalise (engine.py:1075-1086)."""
    apply_diag1(psi, 1.0 if int(keep) == 0 else 0.0, 0.0 if int(keep) == 0 else 1.0, qubit)
    nrm = float(norm2(psi).item())
    if nrm > 0:
        scale(psi, 1.0 / np.sqrt(nrm))
    return psi


# ---------------------------------------------------------------- measurement
def expect_z_all(psi: torch.Tensor) -> torch.Tensor:
    """<Z_q> for all q (float64 device tensor of length n)."""
    n = _check_state(psi)
    out = torch.empty(max(n, 1), dtype=torch.float64, device=psi.device)
    if n == 0:
        return out[:0]
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_expect_z_workspace_bytes(n), psi.device)
    nat.call("tq_sv_expect_z_all", _ptr(psi), n, dtype_tag(psi), _ptr(out), p, cap, stream_ptr(psi.device))
    return out


def expect_z(psi: torch.Tensor, qubit: int) -> float:
    """expect_z_statevector (statevector.py:62-68)."""
    n = _check_state(psi)
    if qubit < 0 or qubit >= n:
        raise ValueError("qubit out of range")
    return float(expect_z_all(psi)[qubit].item())


def probabilities(psi: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """|psi|^2 (float32 for complex64 states, float64 for complex128), into
    `out` when given."""
    n = _check_state(psi)
    dt = torch.float32 if psi.dtype == torch.complex64 else torch.float64
    if out is None:
        out = torch.empty(psi.numel(), dtype=dt, device=psi.device)
    elif out.dtype != dt or out.numel() != psi.numel() or not out.is_contiguous() or out.device != psi.device:
        raise ValueError("probabilities: `out` must be a contiguous tensor of the state's size and real dtype")
    nat.call("tq_sv_probabilities", _ptr(psi), n, dtype_tag(psi), _ptr(out), stream_ptr(psi.device))
    return out


def norm2(psi: torch.Tensor) -> torch.Tensor:
    n = _check_state(psi)
    out = torch.empty(1, dtype=torch.float64, device=psi.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_norm_workspace_bytes(n), psi.device)
    nat.call("tq_sv_norm2", _ptr(psi), n, dtype_tag(psi), _ptr(out), p, cap, stream_ptr(psi.device))
    return out


def qubit_rdm(psi: torch.Tensor, qubit: int) -> np.ndarray:
    """Unnormalised 2x2 reduced density matrix of `qubit` (host complex128)."""
    n = _check_state(psi)
    out = torch.empty(4, dtype=torch.float64, device=psi.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_qubit_rdm_workspace_bytes(n), psi.device)
    nat.call("tq_sv_qubit_rdm", _ptr(psi), n, dtype_tag(psi), int(qubit), _ptr(out), p, cap, stream_ptr(psi.device))
    r = out.cpu().numpy()
    return np.array([[r[0], r[2] + 1j * r[3]], [r[2] - 1j * r[3], r[1]]], dtype=np.complex128)


def apply_kraus(psi: torch.Tensor, ops, qubit: int, status: float) -> int:
    """One stochastic Kraus step (apply_kraus_statevector,
    tyxonq/libs/quantum_library/kernels/statevector.py:132-218): Born weights
    p_i = ||K_i psi||^2 from the qubit's reduced density matrix, the first i
    whose cumulative normalised weight reaches `status` (0 if none does), then
    psi <- K_i psi / sqrt(p_i).  Returns the chosen index."""
    rho = qubit_rdm(psi, qubit)
    mats = [np.asarray(k.detach().cpu().numpy() if hasattr(k, "detach") else k, dtype=np.complex128).reshape(2, 2)
            for k in ops]
    p = np.array([float(np.real(np.trace(m @ rho @ m.conj().T))) for m in mats])
    cum = np.cumsum(p / p.sum())
    sel = 0
    for i, c in enumerate(cum):
        if status <= float(c) and p[i] > 0:  # a zero-weight operator would leave a zero state
            sel = i
            break
    apply_1q(psi, mats[sel] / math.sqrt(p[sel]), qubit)
    return sel


def kraus_trajectories(psi: torch.Tensor, n: int, n_traj: int, ops, qubit: int, status: torch.Tensor) -> torch.Tensor:
    """One Kraus channel on every trajectory of a batch (psi: n_traj states of
    2^n amplitudes, back to back): each trajectory picks its operator from its
    own status on the device (tq_traj_kraus).  Returns the chosen operator
    index per trajectory (int32 device tensor)."""
    mats = np.stack([np.asarray(k.detach().cpu().numpy() if hasattr(k, "detach") else k,
                                dtype=np.complex128).reshape(2, 2) for k in ops])
    kd = torch.from_numpy(np.stack([mats.real, mats.imag], axis=-1).reshape(len(ops), 8).copy()).to(psi.device)
    st = status.to(device=psi.device, dtype=torch.float64).contiguous()
    chosen = torch.empty(n_traj, dtype=torch.int32, device=psi.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_traj_kraus_workspace_bytes(int(n), int(n_traj)), psi.device)
    nat.call("tq_traj_kraus", _ptr(psi), int(n), int(n_traj), dtype_tag(psi), int(qubit), _ptr(kd), len(ops), _ptr(st),
             _ptr(chosen), p, cap, stream_ptr(psi.device))
    return chosen


def inner_re(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    n = _check_state(a)
    _check_state(b, n)
    if a.dtype != b.dtype:
        raise TypeError("inner_re: dtype mismatch")
    out = torch.empty(1, dtype=torch.float64, device=a.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_inner_workspace_bytes(n), a.device)
    nat.call("tq_sv_inner_re", _ptr(a), _ptr(b), n, dtype_tag(a), _ptr(out), p, cap, stream_ptr(a.device))
    return out


def sample(psi: torch.Tensor, shots: int, seed: int) -> torch.Tensor:
    """`shots` basis indices drawn from |psi|^2 (ascending int64 device tensor)."""
    n = _check_state(psi)
    shots = int(shots)
    out = torch.empty(max(shots, 1), dtype=torch.int64, device=psi.device)
    if shots == 0:
        return out[:0]
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_sample_workspace_bytes(n, shots), psi.device)
    nat.call("tq_sv_sample", _ptr(psi), n, dtype_tag(psi), shots, int(seed) & 0xFFFFFFFFFFFFFFFF, _ptr(out), p, cap,
             stream_ptr(psi.device))
    return out


TILED_MIN_N = 12  # H psi and <H> through the tiled kernel (tq_sv_pauli_sum_tiled) from this size up


def _pauli_sum_tiled(psi: torch.Tensor, H, nn: int, out: torch.Tensor | None, energy: torch.Tensor | None) -> None:
    gd, td, ng, nt = H.to_device_classed(psi.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_pauli_sum_tiled_workspace_bytes(nn, dtype_tag(psi), ng, int(out is not None)), psi.device)
    nat.call("tq_sv_pauli_sum_tiled", _ptr(psi), _ptr(out) if out is not None else None, nn, dtype_tag(psi),
             _ptr(gd), ng, _ptr(td), nt, _ptr(energy) if energy is not None else None, p, cap,
             stream_ptr(psi.device))


def pauli_expectation(psi: torch.Tensor, H, n: int | None = None) -> torch.Tensor:
    """Re <psi|H|psi> for a Pauli sum (float64 device tensor of shape (1,))."""
    nn = _check_state(psi, n)
    H = as_pauli_sum(H, nn)
    if H.n != nn:
        raise ValueError(f"Hamiltonian has {H.n} qubits, state {nn}")
    out = torch.empty(1, dtype=torch.float64, device=psi.device)
    if nn >= TILED_MIN_N:
        _pauli_sum_tiled(psi, H, nn, None, out)
        return out
    gd, td, ng, nt = H.to_device(psi.device)
    lib = nat.load()
    p, cap = _ws(lib.tq_sv_pauli_expectation_workspace_bytes(nn, ng), psi.device)
    nat.call("tq_sv_pauli_expectation", _ptr(psi), nn, dtype_tag(psi), _ptr(gd), ng, _ptr(td), nt, _ptr(out), p, cap,
             stream_ptr(psi.device))
    return out


def apply_pauli_sum(psi: torch.Tensor, H, out: torch.Tensor | None = None) -> torch.Tensor:
    """H psi into a new (or given) tensor."""
    nn = _check_state(psi)
    H = as_pauli_sum(H, nn)
    if out is None:
        out = torch.empty_like(psi)
    _check_state(out, nn)
    if nn >= TILED_MIN_N:
        _pauli_sum_tiled(psi, H, nn, out, None)
        return out
    gd, td, ng, nt = H.to_device(psi.device)
    nat.call("tq_sv_apply_pauli_sum", _ptr(psi), _ptr(out), nn, dtype_tag(psi), _ptr(gd), ng, _ptr(td), nt,
             stream_ptr(psi.device))
    return out


def bitstring(index: int, n: int) -> str:
    """Big-endian bitstring of a basis index (engine.py:460-463)."""
    return format(int(index), f"0{n}b") if n > 0 else ""


def counts_from_indices(idx: np.ndarray, n: int) -> dict[str, int]:
    vals, cnt = np.unique(np.asarray(idx, dtype=np.int64), return_counts=True)
    return {bitstring(v, n): int(c) for v, c in zip(vals, cnt)}
