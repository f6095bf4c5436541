"""Gate matrices (complex128, host) with the reference's conventions.

Same definitions and index order as tyxonq/libs/quantum_library/kernels/gates.py:
rotations are cos(t/2) I - i sin(t/2) P (gates.py:19-65, 203-249), 2q
matrices take the first qubit as the high bit of the 4x4 index
(gates.py:82-161, 265-284).  Angles are plain floats here: differentiation is
done by the adjoint kernels, not by autograd through the matrices.
"""
from __future__ import annotations

import math

import numpy as np

_I2 = np.eye(2, dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
PAULI = {"I": _I2, "X": _X, "Y": _Y, "Z": _Z}


def gate_h() -> np.ndarray:
    return np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2.0)


def gate_x() -> np.ndarray:
    return _X.copy()


def gate_y() -> np.ndarray:
    return _Y.copy()


def gate_z() -> np.ndarray:
    return _Z.copy()


def gate_phase(theta: float) -> np.ndarray:
    return np.array([[1, 0], [0, np.exp(1j * float(theta))]], dtype=np.complex128)


def gate_s() -> np.ndarray:
    return gate_phase(math.pi / 2.0)


def gate_sd() -> np.ndarray:
    return gate_phase(-math.pi / 2.0)


def gate_t() -> np.ndarray:
    return gate_phase(math.pi / 4.0)


def gate_td() -> np.ndarray:
    return gate_phase(-math.pi / 4.0)


def _rot(theta: float, P: np.ndarray) -> np.ndarray:
    c, s = math.cos(0.5 * float(theta)), math.sin(0.5 * float(theta))
    return c * np.eye(P.shape[0], dtype=np.complex128) + (-1j * s) * P


def gate_rx(theta: float) -> np.ndarray:
    return _rot(theta, _X)


def gate_ry(theta: float) -> np.ndarray:
    c, s = math.cos(0.5 * float(theta)), math.sin(0.5 * float(theta))
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def gate_rz(theta: float) -> np.ndarray:
    return _rot(theta, _Z)


def gate_rxx(theta: float) -> np.ndarray:
    return _rot(theta, np.kron(_X, _X))


def gate_ryy(theta: float) -> np.ndarray:
    return _rot(theta, np.kron(_Y, _Y))


def gate_rzz(theta: float) -> np.ndarray:
    return _rot(theta, np.kron(_Z, _Z))


def gate_cx_4x4() -> np.ndarray:
    return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)


def gate_cy_4x4() -> np.ndarray:
    U = np.eye(4, dtype=np.complex128)
    U[2:, 2:] = _Y
    return U


def gate_cz_4x4() -> np.ndarray:
    return np.diag([1, 1, 1, -1]).astype(np.complex128)


def gate_swap_4x4() -> np.ndarray:
    return np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def gate_iswap_4x4() -> np.ndarray:
    return np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def gate_cry_4x4(theta: float) -> np.ndarray:
    U = np.eye(4, dtype=np.complex128)
    U[2:, 2:] = gate_ry(theta)
    return U


def pauli_string_matrix(paulis: str) -> np.ndarray:
    """kron of single-qubit Paulis, first character = qubit 0 (pauli.py:65-71)."""
    out = np.array([[1.0 + 0j]])
    for ch in paulis:
        out = np.kron(out, PAULI[ch])
    return out
