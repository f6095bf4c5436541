"""A minimal Circuit with TyxonQ's chain API, for use where TyxonQ itself is
not installed.

Mirrors tyxonq/core/ir/circuit.py: op tuples (name, qubits..., angle) in
``ops`` (:49-182), gate builders (:1042-1633), ``compile()`` / ``device()`` /
``run()`` / ``state()`` (:191-214, :427-583, :828-981), ``expectation`` of
gate products (:1634-1787).  ``run`` applies the
native compile pipeline's two rewrites that change results (auto
``measure_z`` on every qubit when none is present, auto_measure.py:23-35, and
``x`` -> ``rx(pi)``, gates_transform.py:31-32), honours the reference quirk
that ``run``'s own ``shots=1024`` default wins over ``.device(shots=...)``
(circuit.py:873,890), and returns the simulator driver's result layout
(simulators/driver.py:108-131).  With TyxonQ installed, use TyxonQ's Circuit
together with ``tyxonq_gb300.install()`` instead.
"""
from __future__ import annotations

import math
from typing import Any

import numpy as np


class Circuit:
    def __init__(self, num_qubits: int, ops: list | None = None, inputs: Any = None):
        if num_qubits < 0:
            raise ValueError("num_qubits must be non-negative")
        self.num_qubits = int(num_qubits)
        self.ops: list = list(ops) if ops is not None else []
        self._initial_state = inputs
        self._unitary_cache: dict = {}
        self.metadata: dict = {}
        self._device_opts: dict = {"provider": "simulator", "device": "statevector", "shots": 1024}
        for op in self.ops:
            self._validate(op)

    # ------------------------------------------------------------ building
    def _validate(self, op):
        if not isinstance(op, (tuple, list)) or not op:
            raise TypeError("op must be a non-empty tuple or list")
        for a in op[1:]:
            if isinstance(a, int) and (a < 0 or a >= self.num_qubits):
                raise ValueError("qubit index out of range in op")

    def _add(self, *op):
        self._validate(op)
        self.ops.append(tuple(op))
        return self

    def h(self, q):
        return self._add("h", q)

    def x(self, q):
        return self._add("x", q)

    def y(self, q):
        return self._add("y", q)

    def z(self, q):
        return self._add("z", q)

    def s(self, q):
        return self._add("s", q)

    def sdg(self, q):
        return self._add("sdg", q)

    def t(self, q):
        return self._add("t", q)

    def tdg(self, q):
        return self._add("tdg", q)

    def rx(self, q, theta):
        return self._add("rx", q, theta)

    def ry(self, q, theta):
        return self._add("ry", q, theta)

    def rz(self, q, theta):
        return self._add("rz", q, theta)

    def cx(self, c, t):
        return self._add("cx", c, t)

    cnot = cx

    def cz(self, c, t):
        return self._add("cz", c, t)

    def cy(self, c, t):
        return self._add("cy", c, t)

    def cry(self, c, t, theta):
        return self._add("cry", c, t, theta)

    def rxx(self, c, t, theta):
        return self._add("rxx", c, t, theta)

    def ryy(self, c, t, theta):
        return self._add("ryy", c, t, theta)

    def rzz(self, c, t, theta):
        return self._add("rzz", c, t, theta)

    def swap(self, a, b):
        return self._add("swap", a, b)

    def iswap(self, a, b):
        return self._add("iswap", a, b)

    def measure_z(self, q):
        return self._add("measure_z", q)

    def reset(self, q):
        return self._add("reset", q)

    def barrier(self, *qs):
        return self._add("barrier", *qs)

    def unitary(self, *qubits: int, matrix):
        if len(qubits) not in (1, 2):
            raise ValueError("unitary supports 1 or 2 qubits")
        key = f"u{len(self._unitary_cache)}"
        self._unitary_cache[key] = np.asarray(matrix, dtype=np.complex128)
        return self._add("unitary", *qubits, key)

    # ------------------------------------------------------------ chain stages
    def compile(self, **_: Any) -> "Circuit":
        return self

    def device(self, **options: Any) -> "Circuit":
        self._device_opts.update(options)
        return self

    def _compiled(self) -> "Circuit":
        ops = []
        for op in self.ops:
            ops.append(("rx", op[1], math.pi) if op[0] == "x" else op)
        if not any(o[0] == "measure_z" for o in ops):
            ops += [("measure_z", q) for q in range(self.num_qubits)]
        c = Circuit(self.num_qubits, ops, inputs=self._initial_state)
        c._unitary_cache = dict(self._unitary_cache)
        return c

    def _engine(self, **kw):
        from .engine import GpuStatevectorEngine

        return GpuStatevectorEngine(**kw)

    def run(self, *, shots: int = 1024, **opts: Any):
        dev = {**self._device_opts, **opts}
        eng_kw = {k: dev.pop(k) for k in ("dtype", "fusion", "seed") if k in dev}
        if "seed" in eng_kw:
            dev["seed"] = eng_kw["seed"]
        for k in ("provider", "device", "shots"):
            dev.pop(k, None)
        shots = int(shots)
        eng = self._engine(**eng_kw)
        c = self._compiled()
        out = eng.run(c, shots=shots, **dev)
        meta = dict(out.get("metadata", {}))
        prob = statevec = None
        if shots == 0:
            psi = eng.state(c)
            statevec = psi.detach().cpu().numpy() if hasattr(psi, "detach") else np.asarray(psi)
            prob = np.abs(statevec) ** 2
            meta.setdefault("num_qubits", self.num_qubits)
        inner = {"result": out.get("result") or {}, "expectations": out.get("expectations") or {},
                 "probabilities": prob, "statevector": statevec, "result_meta": meta, "uni_status": "completed",
                 "error": ""}
        return [{"result": inner["result"], "result_meta": inner, "uni_status": "completed", "error": "",
                 "metadata": inner, "expectations": {}, "probabilities": None,
                 "postprocessing": {"method": None, "result": None}}]

    def state(self, engine: str | None = None, backend: Any = None, form: str | None = None, **kw):
        eng = self._engine(**kw)
        psi = eng.state(self)
        if form == "numpy":
            return psi.detach().cpu().numpy() if hasattr(psi, "detach") else np.asarray(psi)
        return psi

    def probability(self, **kw):
        return self._engine(**kw).probability(self)

    def amplitude(self, bitstring: str, **kw):
        return self._engine(**kw).amplitude(self, bitstring)

    def expectation_ps(self, hamiltonian, **kw) -> float:
        return self._engine(**kw).expval(self, hamiltonian)

    def expectation(self, *pauli_ops: Any) -> float:
        """<psi|O|psi> for a product of (gate, qubits) factors (circuit.py:1634-1737)."""
        return self._engine().expectation_product(self, pauli_ops)

    def expval(self, *pauli_ops: Any) -> float:
        """Alias of expectation (circuit.py:1720-1737)."""
        return self.expectation(*pauli_ops)
