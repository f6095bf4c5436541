"""VQE entry points with the reference's names, evaluated on the GPU engine.

``HEA`` mirrors tyxonq/applications/chem/algorithms/hea.py for explicit
(n_qubits, layers, hamiltonian) construction (hea.py:125-207): the RY ansatz
of ``build_hwe_ry_ops`` (libs/circuits_library/blocks.py:60-85 -- an initial
RY layer, then per layer a CNOT ladder and an RY layer), (layers+1)*n
parameters, ``energy(params)`` and ``energy_and_grad(params)`` returning
(float, float64 ndarray) like hea.py:231-266.  Gradients come from the adjoint
kernels instead of autograd / finite differences.

``UCCSD`` mirrors the numeric paths of applications/chem/algorithms/
ucc.py:416-510 for integrals given explicitly: UCCSD from the Hartree-Fock
bitstring (tyxonq_gb300.chem) with exact excitations on the statevector, as
Pauli-string exponentials (trotter=True), or in CI space (engine="civector").
Molecule construction through pyscf is outside this package.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from .adjoint import ParamGate, ParametricEstimator
from .hamiltonian import PauliSum, as_pauli_sum
from .ir import Gate, _rot_gate


def hwe_ry_param_gates(n: int, layers: int) -> list[ParamGate]:
    pg = []
    for q in range(n):
        pg.append(ParamGate(_rot_gate("ry", (q,), 0.0), q))
    for l in range(layers):
        for q in range(n - 1):
            pg.append(ParamGate(Gate("cx", (q, q + 1))))
        for q in range(n):
            pg.append(ParamGate(_rot_gate("ry", (q,), 0.0), (l + 1) * n + q))
    return pg


class HEA:
    def __init__(self, n_qubits: int, layers: int, hamiltonian, runtime: str = "numeric", dtype=torch.complex64,
                 device="cuda"):
        self.n_qubits = int(n_qubits)
        self.layers = int(layers)
        self.hamiltonian = as_pauli_sum(hamiltonian, self.n_qubits)
        self.runtime = runtime
        self.n_params = (self.layers + 1) * self.n_qubits
        self.init_guess = np.random.default_rng(7).random(self.n_params, dtype=np.float64)  # hea.py:205-207
        self._est = ParametricEstimator(self.n_qubits, hwe_ry_param_gates(self.n_qubits, self.layers), self.n_params,
                                        self.hamiltonian, dtype=dtype, device=device)

    def _shots(self, runtime, shots):
        rt = runtime or self.runtime
        return int(shots or 0) if rt == "device" or shots else 0

    def energy(self, params: Sequence[float] | None = None, *, runtime: str | None = None, shots: int = 0,
               seed: int = 0) -> float:
        """Exact energy (numeric runtime), or a shot estimate from basis-group
        sampling when shots > 0 (device runtime, tyxonq_gb300.shots)."""
        p = self.init_guess if params is None else np.asarray(params, dtype=np.float64)
        nshots = self._shots(runtime, shots)
        if nshots:
            from .shots import ShotEstimator

            return ShotEstimator(self._est, self.hamiltonian, nshots, seed).energy(p)
        return self._est.energy(p)

    def energy_and_grad(self, params: Sequence[float] | None = None, *, runtime: str | None = None,
                        shots: int = 0, seed: int = 0) -> tuple[float, np.ndarray]:
        """Exact energy and adjoint gradient, or with shots > 0 the shot
        estimate and parameter-shift gradient of the device runtime."""
        p = self.init_guess if params is None else np.asarray(params, dtype=np.float64)
        nshots = self._shots(runtime, shots)
        if nshots:
            from .shots import ShotEstimator

            return ShotEstimator(self._est, self.hamiltonian, nshots, seed).energy_and_grad(p)
        return self._est.energy_and_grad(p)

    def kernel(self, method: str = "L-BFGS-B", maxiter: int = 200) -> float:
        """Minimise the energy with SciPy (hea.py:294-337 uses SciPy the same way)."""
        from scipy.optimize import minimize

        res = minimize(lambda x: self.energy_and_grad(x), self.init_guess, jac=True, method=method,
                       options={"maxiter": maxiter})
        self.opt_res = res
        self.params = res.x
        return float(res.fun)


class UCCSD:
    """engine="statevector" (default): the excitations applied exactly on the
    n-qubit state (statevector_ops.py evolve_excitation; tyxonq_gb300.excitation)
    with a reverse-sweep gradient, or with trotter=True the same ansatz as
    products of Pauli-string exponentials (the circuit form of ucc.py with
    trotter=True; exact too, as the Pauli words of one excitation commute)
    through the fused-pass adjoint engine; engine="civector": the CI-space
    evolution of civector_ops.py on the determinants with n_elec / 2 electrons
    per spin (tyxonq_gb300.ci), FP64.  One parameter per excitation."""

    def __init__(self, int1e: np.ndarray, int2e: np.ndarray, n_elec: int, e_core: float = 0.0,
                 dtype=torch.complex64, device="cuda", engine: str = "statevector", trotter: bool = False):
        from .chem import hf_basis, molecular_hamiltonian, uccsd_param_gates

        self.int1e, self.int2e = np.asarray(int1e), np.asarray(int2e)
        self.n_orb = self.int1e.shape[0]
        self.n_qubits = 2 * self.n_orb
        self.n_elec = int(n_elec)
        self.e_core = float(e_core)
        self.hamiltonian: PauliSum = molecular_hamiltonian(self.int1e, self.int2e)
        pg, self.n_params, self.ex_ops = uccsd_param_gates(self.n_orb, self.n_elec)
        self.param_gates = pg
        self.init_guess = np.zeros(self.n_params)
        self.engine = engine
        self.trotter = bool(trotter)
        if engine == "civector":
            from .ci import CIVectorUCC

            no = self.n_elec // 2
            # same parametrisation as the statevector engine: one angle per excitation
            self._est = CIVectorUCC(self.n_qubits, (no, no), self.ex_ops, list(range(len(self.ex_ops))),
                                    self.hamiltonian, device=device)
        elif engine == "statevector" and trotter:
            self._est = ParametricEstimator(self.n_qubits, pg, self.n_params, self.hamiltonian, dtype=dtype,
                                            device=device, init_basis=hf_basis(self.n_qubits, self.n_elec // 2))
        elif engine == "statevector":
            from .excitation import ExcitationEstimator

            self._est = ExcitationEstimator(self.n_qubits, self.ex_ops, list(range(len(self.ex_ops))),
                                            self.n_params, self.hamiltonian, dtype=dtype, device=device,
                                            init_basis=hf_basis(self.n_qubits, self.n_elec // 2))
        else:
            raise ValueError(f"unknown UCC engine {engine!r} (statevector | civector)")

    def energy(self, params: Sequence[float] | None = None) -> float:
        p = self.init_guess if params is None else np.asarray(params, dtype=np.float64)
        return self._est.energy(p) + self.e_core

    def energy_and_grad(self, params: Sequence[float] | None = None) -> tuple[float, np.ndarray]:
        p = self.init_guess if params is None else np.asarray(params, dtype=np.float64)
        e, g = self._est.energy_and_grad(p)
        return e + self.e_core, g
