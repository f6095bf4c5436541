"""Lowering of reference op tuples to device gate records.

The reference engine interprets ``circuit.ops`` tuples with an if-chain
(tyxonq/devices/simulators/statevector/engine.py:52-374 for ``run``,
:914-1039 for ``state``).  ``lower_ops`` performs the same dispatch once, on
the host, producing ``Gate`` records the GPU executors consume.  The two gate
sets differ exactly as in the reference: ``state()`` has no ``cry`` branch;
neither method has ``y``/``z``/``t``/``tdg``/``cy``, which are ignored like any
unknown op (engine.py:372-374).  ``extended=True`` opts into applying them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Sequence

import numpy as np

from . import gates as G

RUN_GATES = {"h", "rz", "rx", "ry", "cx", "cry", "cz", "iswap", "swap", "rxx", "ryy", "rzz", "x", "s", "sdg",
             "measure_z", "barrier", "project_z", "reset", "unitary", "kraus"}
STATE_GATES = RUN_GATES - {"cry", "measure_z", "barrier"}
EXTENDED_GATES = {"y", "z", "t", "tdg", "cy", "phase", "cnot"}
UNSUPPORTED = {"pulse", "pulse_inline"}
# ops that feed the reference's use_noise Z attenuation (engine.py:56-140, _attenuate :488-494)
ATTENUATED = {"h", "rz", "rx", "ry", "cx", "cry", "cz", "iswap", "swap", "rxx", "ryy", "rzz", "x", "s", "sdg",
              "unitary"}

# Pauli generator of each rotation: U(a) = exp(-i a/2 P)
ROTATION_GENERATORS = {"rx": "X", "ry": "Y", "rz": "Z", "rxx": "XX", "ryy": "YY", "rzz": "ZZ"}


@dataclass
class Gate:
    """One device gate.

    kind: 'u1' dense 2x2 | 'd1' diagonal 2x2 | 'u2' dense 4x4 | 'cx' | 'cz' |
          'swap' | 'uk' dense 2^k | 'prot' Pauli rotation | 'proj' Z projection |
          'kraus' one-qubit channel (kraus: operator list, status: float or None)
    qubits: target qubits, first = most significant matrix index bit.
    mat: complex128 matrix (u1/d1/u2/uk; d1 stores the 2x2 diagonal matrix).
    rot: (name, angle, source) for parametrised rotations, else None; `source`
         is the op's original angle object (float or tensor).
    """

    kind: str
    qubits: tuple
    mat: np.ndarray | None = None
    rot: tuple | None = None
    keep: int = 0
    pauli: tuple | None = None  # ((q, 'X'|'Y'|'Z'), ...) for kind 'prot'
    kraus: tuple | None = None  # 2x2 operators of kind 'kraus'
    status: float | None = None


def _angle(x: Any) -> float:
    try:
        import torch

        if isinstance(x, torch.Tensor):
            return float(x.detach().reshape(-1)[0].item())
    except ImportError:  # pragma: no cover
        pass
    return float(np.asarray(x).reshape(-1)[0]) if not isinstance(x, (int, float)) else float(x)


def _rot_gate(name: str, qubits: tuple, a_src: Any) -> Gate:
    a = _angle(a_src)
    if name == "rz":
        return Gate("d1", qubits, np.diag([np.exp(-0.5j * a), np.exp(0.5j * a)]), rot=(name, a, a_src))
    mat = {"rx": G.gate_rx, "ry": G.gate_ry, "rxx": G.gate_rxx, "ryy": G.gate_ryy, "rzz": G.gate_rzz,
           "cry": G.gate_cry_4x4}[name](a)
    return Gate("u1" if len(qubits) == 1 else "u2", qubits, mat, rot=(name, a, a_src))


def lower_ops(circuit: Any, mode: str = "state", extended: bool = False) -> tuple[list[Gate], list[int]]:
    """circuit.ops -> (gates, measured qubits) following the reference dispatch."""
    n = int(getattr(circuit, "num_qubits", 0))
    allowed = set(RUN_GATES if mode == "run" else STATE_GATES)
    if extended:
        allowed |= EXTENDED_GATES | {"cry"}
    ucache = getattr(circuit, "_unitary_cache", {}) or {}
    out: list[Gate] = []
    measures: list[int] = []
    for op in getattr(circuit, "ops", []):
        if not isinstance(op, (list, tuple)) or not op:
            continue
        name = op[0]
        if name in UNSUPPORTED:
            raise NotImplementedError(
                f"op '{name}' (noise / pulse simulation) is not part of the GPU statevector engine; "
                "use the reference engine for it")
        if name not in allowed:
            continue
        if name == "cnot":
            name = "cx"
        if name in ("h", "x", "y", "z"):
            q = int(op[1])
            out.append(Gate("u1", (q,), {"h": G.gate_h, "x": G.gate_x, "y": G.gate_y, "z": G.gate_z}[name]()))
        elif name in ("s", "sdg", "t", "tdg"):
            q = int(op[1])
            ph = {"s": math.pi / 2, "sdg": -math.pi / 2, "t": math.pi / 4, "tdg": -math.pi / 4}[name]
            out.append(Gate("d1", (q,), np.diag([1.0, np.exp(1j * ph)])))
        elif name == "phase":
            q = int(op[1])
            a = _angle(op[2])
            out.append(Gate("d1", (q,), np.diag([1.0, np.exp(1j * a)]), rot=("phase", a, op[2])))
        elif name in ("rx", "ry", "rz"):
            out.append(_rot_gate(name, (int(op[1]),), op[2]))
        elif name in ("rxx", "ryy", "rzz", "cry"):
            a, b = int(op[1]), int(op[2])
            if a == b:
                continue  # apply_2q_statevector returns psi for q0 == q1
            out.append(_rot_gate(name, (a, b), op[3]))
        elif name in ("cx", "cz", "swap"):
            a, b = int(op[1]), int(op[2])
            if a != b:
                out.append(Gate(name, (a, b)))
        elif name in ("iswap", "cy"):
            a, b = int(op[1]), int(op[2])
            if a != b:
                out.append(Gate("u2", (a, b), G.gate_iswap_4x4() if name == "iswap" else G.gate_cy_4x4()))
        elif name == "kraus":
            # ("kraus", qubit, key[, status]) with operators in circuit._kraus_cache
            # (engine.py:145-155); an unknown key is skipped as there
            ops_k = (getattr(circuit, "_kraus_cache", {}) or {}).get(str(op[2]))
            if ops_k is None:
                continue
            mats = tuple(np.asarray(k.detach().cpu().numpy() if hasattr(k, "detach") else k,
                                    dtype=np.complex128).reshape(2, 2) for k in ops_k)
            out.append(Gate("kraus", (int(op[1]),), kraus=mats, status=float(op[3]) if len(op) > 3 else None))
        elif name == "measure_z":
            measures.append(int(op[1]))
        elif name == "barrier":
            continue
        elif name == "project_z":
            out.append(Gate("proj", (int(op[1]),), keep=int(op[2])))
        elif name == "reset":
            out.append(Gate("proj", (int(op[1]),), keep=0))
        elif name == "unitary":
            if len(op) == 3:
                qs, key = (int(op[1]),), str(op[2])
            elif len(op) == 4:
                qs, key = (int(op[1]), int(op[2])), str(op[3])
            else:
                continue
            U = ucache.get(key)
            if U is None:
                continue
            U = np.asarray(U.detach().cpu().numpy() if hasattr(U, "detach") else U, dtype=np.complex128)
            out.append(Gate("uk", qs, U.reshape(1 << len(qs), 1 << len(qs))))
    for g in out:
        for q in g.qubits:
            if q < 0 or q >= n:
                raise ValueError("qubit index out of range in op")
    return out, measures


def pauli_rotation(pauli: Sequence[tuple[int, str]], angle: Any) -> Gate:
    """exp(-i angle/2 P) as one device gate (the unitary evolve_pauli_ops builds
    from basis changes, a CX ladder and RZ: circuits_library/utils.py:29-59)."""
    ps = tuple((int(q), str(p).upper()) for q, p in pauli)
    return Gate("prot", tuple(q for q, _ in ps), rot=("prot", _angle(angle), angle), pauli=ps)
