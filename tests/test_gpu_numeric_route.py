"""The HEA numeric runtime's energy on the device Pauli sum (plugin route).

HEANumericRuntime (applications/chem/runtimes/hea_numeric_runtime.py) is not
importable without openfermion, so the route is exercised on a stand-in class
with its method contract: attributes n and hamiltonian [(coeff, [(P, q)])],
_build(params, get_circuit), energy(params, get_circuit), and an
energy_and_grad that differentiates energy with torch autograd, as
value_and_grad does with the pytorch backend (pytorch_backend.py:446-564).
The stand-in's own energy raises: after the route it never runs, and no
dense Hamiltonian is formed.  Tolerances: complex128 1e-10 (energy) and 1e-8
(gradient) against the oracle.
"""
import numpy as np
import pytest
import torch

from oracle import sv

pytestmark = pytest.mark.gpu


class _HeaNumericStandIn:
    def __init__(self, n, layers, hamiltonian):
        self.n, self.layers, self.hamiltonian = n, layers, list(hamiltonian)

    def _build(self, params, get_circuit):
        return get_circuit(params)

    def energy(self, params, get_circuit):
        raise AssertionError("the dense-matrix energy must not run after the route")

    def energy_and_grad(self, params, get_circuit):
        p = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
        e = self.energy(p, get_circuit)
        e.backward()
        return float(e.item()), p.grad.numpy()


def _circuit(n, layers):
    from tyxonq_gb300.circuit import Circuit

    def get_circuit(params):
        c = Circuit(n)
        k = 0
        for _ in range(layers):
            for q in range(n):
                c.ry(q, params[k])
                k += 1
            for q in range(n - 1):
                c.cx(q, q + 1)
        return c

    return get_circuit


def test_hea_numeric_energy_and_grad_on_device_pauli_sum(monkeypatch):
    from tyxonq_gb300 import plugin

    monkeypatch.setenv("TYXONQ_GB300_DTYPE", "complex128")
    n, layers = 10, 3
    rng = np.random.default_rng(5)
    ham = [(-1.0, [("Z", i), ("Z", i + 1)]) for i in range(n - 1)] + [(-0.7, [("X", i)]) for i in range(n)]
    ham += [(0.3, [("Y", 1), ("X", 4), ("Z", 8)])]
    rt = _HeaNumericStandIn(n, layers, ham)
    plugin.route_hea_numeric(_HeaNumericStandIn)
    try:
        theta = rng.uniform(0, 2 * np.pi, n * layers)
        e, g = rt.energy_and_grad(theta, _circuit(n, layers))
        e_only = rt.energy(theta, _circuit(n, layers))
    finally:
        plugin.unroute_hea_numeric()
    codes, coeffs = sv.terms_to_codes(n, ham)
    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in
             [g_ for l in range(layers) for g_ in
              [("ry", (q,), l * n + q) for q in range(n)] + [("cx", (q, q + 1), None) for q in range(n - 1)]]]
    e_ref, g_ref = sv.grad_adjoint(n, gates, theta, codes, coeffs)
    assert abs(e - e_ref) < 1e-10
    assert abs(float(e_only) - e_ref) < 1e-10
    np.testing.assert_allclose(g, g_ref, atol=1e-8)
    with pytest.raises(AssertionError):
        rt.energy(theta, _circuit(n, layers))  # unrouted again
