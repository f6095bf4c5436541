"""ctypes front end of the C complex128 restatement (oracle/sv_ref.c).

TEST INFRASTRUCTURE ONLY: the oracle for states too large for the NumPy
restatement (the 28-qubit random circuit, 22-26-qubit serving requests).
Gate matrices come from ``oracle.sv.gate_matrix`` (kernels/gates.py:11-287);
the op loop follows StatevectorEngine.state's dispatch (engine.py:914-1039)
for the gates these workloads use.
"""
from __future__ import annotations

import ctypes
from typing import Any, Sequence

import numpy as np

from . import build as _build
from .sv import gate_matrix

_LIB = None
_P = ctypes.c_void_p


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(str(_build.build()))
        L.orc_init.argtypes = [_P, ctypes.c_int, ctypes.c_int64]
        L.orc_apply_1q.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P]
        L.orc_apply_2q.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
        L.orc_probs.argtypes = [_P, ctypes.c_int, _P]
        L.orc_pauli_expectation.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int]
        L.orc_pauli_expectation.restype = ctypes.c_double
        L.orc_max_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


ONE_Q = ("h", "x", "y", "z", "s", "sdg", "t", "tdg")
ONE_Q_ROT = ("rx", "ry", "rz", "phase")
TWO_Q = ("cx", "cnot", "cz", "cy", "swap", "iswap")
TWO_Q_ROT = ("rxx", "ryy", "rzz", "cry")


def run_ops(n: int, ops: Sequence[Any], basis: int = 0, allowed=None, unitary_cache: dict | None = None) -> np.ndarray:
    """Final complex128 state of an op-tuple list ((name, q..., angle)).

    ``allowed``: op names applied (others are skipped, as StatevectorEngine
    skips ops outside its dispatch, engine.py:372-374); None applies every op
    this oracle knows and raises on the rest.  ``unitary_cache``: matrices of
    ('unitary', q[, q1], key) ops (engine.py:127-144)."""
    L = lib()
    psi = np.empty(1 << n, dtype=np.complex128)
    L.orc_init(_ptr(psi), n, int(basis))
    for op in ops:
        name = op[0]
        if allowed is not None and name not in allowed:
            continue
        if name in ONE_Q:
            U = np.ascontiguousarray(gate_matrix(name), dtype=np.complex128)
            L.orc_apply_1q(_ptr(psi), n, int(op[1]), _ptr(U))
        elif name in ONE_Q_ROT:
            U = np.ascontiguousarray(gate_matrix(name, float(op[2])), dtype=np.complex128)
            L.orc_apply_1q(_ptr(psi), n, int(op[1]), _ptr(U))
        elif name in TWO_Q:
            U = np.ascontiguousarray(gate_matrix(name), dtype=np.complex128)
            L.orc_apply_2q(_ptr(psi), n, int(op[1]), int(op[2]), _ptr(U))
        elif name in TWO_Q_ROT:
            U = np.ascontiguousarray(gate_matrix(name, float(op[3])), dtype=np.complex128)
            L.orc_apply_2q(_ptr(psi), n, int(op[1]), int(op[2]), _ptr(U))
        elif name == "unitary" and unitary_cache is not None:
            U = np.ascontiguousarray(unitary_cache[str(op[-1])], dtype=np.complex128)
            if len(op) == 3:
                L.orc_apply_1q(_ptr(psi), n, int(op[1]), _ptr(U))
            else:
                L.orc_apply_2q(_ptr(psi), n, int(op[1]), int(op[2]), _ptr(U))
        else:
            raise KeyError(f"C oracle: unsupported op {name!r}")
    return psi


def probabilities(psi: np.ndarray) -> np.ndarray:
    n = int(psi.size).bit_length() - 1
    p = np.empty(psi.size, dtype=np.float64)
    lib().orc_probs(_ptr(psi), n, _ptr(p))
    return p


def pauli_expectation(psi: np.ndarray, codes: np.ndarray, coeffs: np.ndarray) -> float:
    """Re <psi|H|psi>, H = sum_k coeffs[k] P(codes[k]) (codes 0..3 = I, X, Y, Z)."""
    L = lib()
    n = int(psi.size).bit_length() - 1
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    assert codes.shape == (coeffs.size, n)
    nt = L.orc_max_threads()
    part = np.zeros(nt, dtype=np.float64)
    return float(L.orc_pauli_expectation(_ptr(psi), n, int(coeffs.size), _ptr(codes), _ptr(coeffs), _ptr(part), nt))
