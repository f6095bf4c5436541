"""Registration of the GPU engine into an installed TyxonQ.

TyxonQ picks simulator engines in ``devices/simulators/driver.py:_select_engine``
(:20-30), called as ``Engine()`` (driver.py:97,164), and ``Circuit.state()``
imports ``StatevectorEngine`` from ``devices/simulators/statevector/engine``
at call time (core/ir/circuit.py:491-494).  ``install`` wraps the former so
``device="statevector_gpu"`` (and, with ``replace_statevector``, plain
``"statevector"``) returns GpuStatevectorEngine, and rebinds the latter so
``Circuit.state()`` runs on the GPU; ``Circuit.expectation`` of gate products
on a statevector device (circuit.py:1739-1787) runs on the GPU too, and so does
the HEA numeric runtime's energy (no dense Hamiltonian).  The chain API
``c.compile().device(provider="simulator", device="statevector").run()`` then
reaches the GPU engine unchanged.  ``uninstall`` restores both.
"""
from __future__ import annotations

_saved: dict = {}


def install(replace_statevector: bool = True, alias: str = "statevector_gpu"):
    import tyxonq.devices.simulators.driver as drv  # type: ignore
    import tyxonq.devices.simulators.statevector.engine as sv_mod  # type: ignore

    from .engine import GpuStatevectorEngine

    if "select" not in _saved:
        _saved["select"] = drv._select_engine
        _saved["sv_cls"] = sv_mod.StatevectorEngine
    orig = _saved["select"]
    names = {alias, f"simulator:{alias}"}
    if replace_statevector:
        names |= {"statevector", "simulator:statevector"}

    def _select_engine(device: str):
        name = device.split("::")[-1] if "::" in device else device
        if name in names:
            return GpuStatevectorEngine
        return orig(device)

    drv._select_engine = _select_engine
    if replace_statevector:
        sv_mod.StatevectorEngine = GpuStatevectorEngine
        _route_expectation(GpuStatevectorEngine)
        _route_numeric_energy()
    return GpuStatevectorEngine


def _route_numeric_energy() -> bool:
    """HEANumericRuntime.energy (applications/chem/runtimes/hea_numeric_runtime.py:
    71-85) builds a dense 2^n x 2^n Hamiltonian with pauli_string_sum_dense
    (:31-54) and contracts it with the state (dynamics.expectation).  When that
    module is importable (it needs openfermion), its energy is rebound to the
    device Pauli sum: the same circuit state (Circuit.state, on the GPU after
    install) and <psi|H|psi> from the Pauli terms, differentiable through the
    adjoint autograd path, so energy_and_grad's value_and_grad works unchanged
    and no matrix is formed.  Returns whether the runtime was found."""
    try:
        import tyxonq.applications.chem.runtimes.hea_numeric_runtime as hnr  # type: ignore
    except Exception:
        return False
    route_hea_numeric(hnr.HEANumericRuntime)
    return True


def route_hea_numeric(cls) -> None:
    """Rebind cls.energy (the HEANumericRuntime contract: attributes n and
    hamiltonian = [(coeff, [(P, q), ...])], method _build(params, get_circuit))
    to the device Pauli-sum energy."""
    from .adjoint import pauli_energy
    from .hamiltonian import PauliSum

    key = f"hea_energy:{cls.__module__}.{cls.__qualname__}"
    if key not in _saved:
        _saved[key] = (cls, cls.energy)

    def energy(self, params, get_circuit):
        c = self._build(params, get_circuit)
        psi = c.state()
        cache = self.__dict__.setdefault("_gb300_pauli_sum", {})
        hk = (int(self.n), tuple((float(cf), tuple((str(P).upper(), int(q)) for P, q in ops))
                                 for cf, ops in self.hamiltonian))
        H = cache.get(hk)
        if H is None:
            H = cache[hk] = PauliSum.from_terms(int(self.n), self.hamiltonian)
        return pauli_energy(psi, H)

    cls.energy = energy


def _route_expectation(engine_cls) -> None:
    """Circuit.expectation on a statevector device (core/ir/circuit.py:1739-1787)
    runs the state and the operator product on the GPU."""
    from tyxonq.core.ir.circuit import Circuit  # type: ignore

    if "sv_expect" not in _saved:
        _saved["sv_expect"] = Circuit._expectation_statevector

    def _expectation_statevector(self, pauli_ops, nb, n):
        return engine_cls().expectation_product(self, pauli_ops)

    Circuit._expectation_statevector = _expectation_statevector


def uninstall():
    if "select" not in _saved:
        return
    import tyxonq.devices.simulators.driver as drv  # type: ignore
    import tyxonq.devices.simulators.statevector.engine as sv_mod  # type: ignore

    drv._select_engine = _saved["select"]
    sv_mod.StatevectorEngine = _saved["sv_cls"]
    if "sv_expect" in _saved:
        from tyxonq.core.ir.circuit import Circuit  # type: ignore

        Circuit._expectation_statevector = _saved.pop("sv_expect")
    unroute_hea_numeric()


def unroute_hea_numeric() -> None:
    for key in [k for k in _saved if k.startswith("hea_energy:")]:
        cls, fn = _saved.pop(key)
        cls.energy = fn
