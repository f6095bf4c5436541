"""Drop-in wiring: the plugin routes TyxonQ's engine selection to the GPU
engine (CPU check, when TyxonQ's sources are importable in this checkout's
environment), and the chain API of the Circuit mirror runs end to end on
the GPU."""
import os
import sys

import numpy as np
import pytest


def _tyxonq_available():
    p = os.environ.get("TYXONQ_SRC")  # a TyxonQ source tree (its src/ folder)
    if p and os.path.isdir(p) and p not in sys.path:
        sys.path.append(p)
    try:
        import tyxonq.devices.simulators.driver  # noqa: F401

        return True
    except Exception:
        return False


def test_plugin_routes_engine_selection():
    if not _tyxonq_available():
        pytest.skip("TyxonQ not importable here")
    import tyxonq.devices.simulators.driver as drv
    import tyxonq.devices.simulators.statevector.engine as sv_mod

    import tyxonq_gb300
    from tyxonq_gb300 import GpuStatevectorEngine, plugin

    orig_cls = sv_mod.StatevectorEngine
    tyxonq_gb300.install(replace_statevector=False)
    try:
        assert drv._select_engine("statevector_gpu") is GpuStatevectorEngine
        assert drv._select_engine("simulator::statevector_gpu") is GpuStatevectorEngine
        assert drv._select_engine("statevector") is orig_cls
    finally:
        plugin.uninstall()
    tyxonq_gb300.install(replace_statevector=True)
    try:
        assert drv._select_engine("statevector") is GpuStatevectorEngine
        assert sv_mod.StatevectorEngine is GpuStatevectorEngine
        assert drv._select_engine("mps").__name__ != "GpuStatevectorEngine"
    finally:
        plugin.uninstall()
    assert sv_mod.StatevectorEngine is orig_cls


def test_engine_class_contract():
    from tyxonq_gb300 import GpuStatevectorEngine

    assert GpuStatevectorEngine.name == "statevector"
    assert GpuStatevectorEngine.capabilities == {"supports_shots": True}
    for m in ("run", "state", "probability", "amplitude", "perfect_sampling", "expval"):
        assert callable(getattr(GpuStatevectorEngine, m))


@pytest.mark.gpu
def test_chain_api_mirror_end_to_end():
    from tyxonq_gb300.circuit import Circuit

    c = Circuit(2)
    c.h(0).cx(0, 1)
    res = c.compile().device(provider="simulator", device="statevector").run(seed=7)
    counts = res[0]["result"]
    assert sum(counts.values()) == 1024 and set(counts) <= {"00", "11"}
    res0 = Circuit(2).h(0).cx(0, 1).run(shots=0)[0]["result_meta"]
    assert abs(res0["expectations"]["Z0"]) < 1e-6 and abs(res0["expectations"]["Z1"]) < 1e-6
    np.testing.assert_allclose(res0["probabilities"], [0.5, 0, 0, 0.5], atol=1e-6)
    # x -> rx(pi) rewrite of the compile pipeline gives the -i global phase on run()'s statevector
    r = Circuit(1).x(0).run(shots=0)[0]["result_meta"]
    np.testing.assert_allclose(r["statevector"], [0, -1j], atol=1e-6)
    psi = Circuit(1).x(0).state()  # state() does not compile
    psi = psi.cpu().numpy() if hasattr(psi, "cpu") else np.asarray(psi)  # numpy backend when TyxonQ is importable
    np.testing.assert_allclose(psi, [0, 1], atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_circuit_expectation_known_answers_on_gpu(dtype, monkeypatch):
    """The reference tests' known answers of Circuit.expectation
    (tests_core_module/test_circuit_expectation.py:9-69), on the device."""
    from tyxonq_gb300.circuit import Circuit
    from tyxonq_gb300.gates import gate_x, gate_y, gate_z

    monkeypatch.setenv("TYXONQ_GB300_DTYPE", dtype)
    tol = 1e-10 if dtype == "complex128" else 1e-6
    assert abs(Circuit(1).h(0).expectation((gate_x(), [0])) - 1.0) < tol
    assert abs(Circuit(1).expectation((gate_z(), [0])) - 1.0) < tol
    bell = Circuit(2).h(0).cx(0, 1)
    assert abs(bell.expectation((gate_z(), [0]), (gate_z(), [1])) - 1.0) < tol
    assert abs(bell.expectation((gate_x(), [0]), (gate_x(), [1])) - 1.0) < tol
    assert abs(bell.expval((gate_y(), [0]), (gate_y(), [1])) + 1.0) < tol  # <YY> = -1 on |Phi+>
    n = 3
    c = Circuit(n)
    for i in range(n):
        c.h(i)
    e = -sum(c.expectation((gate_x(), [i])) for i in range(n))
    e += sum(c.expectation((gate_z(), [i]), (gate_z(), [i + 1])) for i in range(n - 1))
    assert abs(e + 3.0) < tol
    # callables and two-qubit factors, as the reference accepts them
    assert abs(bell.expectation((gate_x, [0]), (gate_x(), [1])) - 1.0) < tol
    assert abs(bell.expectation((np.kron(gate_z(), gate_z()), [0, 1])) - 1.0) < tol
    assert abs(bell.expectation((np.kron(gate_x(), gate_x()), [0, 1]), (gate_x, [1])) - 0.0) < tol  # <X_0> = 0
    with pytest.raises(NotImplementedError):
        bell.expectation((np.eye(8), [0, 1, 1]))


@pytest.mark.gpu
def test_tyxonq_chain_on_gpu_matches_reference_engine():
    """TyxonQ's own Circuit (sources given by TYXONQ_SRC) through install():
    compile -> device -> run on the golden circuits gives the reference
    engine's expectations and result layout; state() and Circuit.expectation
    match too.  Skipped without TyxonQ sources."""
    if not _tyxonq_available():
        pytest.skip("TyxonQ sources not given (TYXONQ_SRC)")
    import tyxonq as tq
    import tyxonq.devices.simulators.statevector.engine as sv_mod
    from tyxonq.libs.quantum_library.kernels.gates import gate_x, gate_z

    from tests import golden_data
    from tyxonq_gb300 import plugin

    tq.set_backend("numpy")
    cases = [c for c in golden_data.circuit_cases() if not any(o[0] in ("unitary", "kraus") for o in c[2])]
    assert cases

    def build(n, ops):
        c = tq.Circuit(n)
        c.ops = [tuple(o) for o in ops]
        return c

    def outputs():
        out = []
        for name, n, ops, _uc, _state, _runz in cases:
            r = build(n, ops).compile().device(provider="simulator", device="statevector").run(shots=0)
            rm = r[0]["result_meta"] if isinstance(r, list) else r["result_meta"]
            psi = np.asarray(build(n, ops).state())
            bell = tq.Circuit(2).h(0).cx(0, 1)
            ex = bell.expectation((gate_z(), [0]), (gate_z(), [1])), bell.expectation((gate_x(), [0]))
            out.append((name, dict(rm.get("expectations", {})), sorted(rm.keys()), psi, ex))
        return out

    ref = outputs()
    plugin.install(replace_statevector=True)
    try:
        from tyxonq_gb300.engine import GpuStatevectorEngine

        assert sv_mod.StatevectorEngine is GpuStatevectorEngine
        gpu = outputs()
    finally:
        plugin.uninstall()
    for (nm, ez, keys, psi, ex), (_, ez2, keys2, psi2, ex2) in zip(ref, gpu):
        assert keys == keys2, nm
        assert ez.keys() == ez2.keys(), nm
        for k in ez:
            assert abs(ez[k] - ez2[k]) < 1e-6, (nm, k)
        np.testing.assert_allclose(psi2, psi, atol=1e-6, err_msg=nm)
        np.testing.assert_allclose(ex2, ex, atol=1e-6)


def test_engine_dtype_follows_tyxonq_set_dtype(monkeypatch):
    """The engine's state dtype: its own argument, else TyxonQ's set_dtype choice
    (an instance attribute of the numerics backend; the class default does not
    count), else TYXONQ_GB300_DTYPE, else complex64."""
    import torch

    from tyxonq_gb300.engine import resolve_dtype

    class _Backend:
        dtypestr = "complex128"  # the class default of the reference backends

    monkeypatch.delenv("TYXONQ_GB300_DTYPE", raising=False)
    b = _Backend()
    assert resolve_dtype(None, b) == torch.complex64  # nothing chosen
    b.dtypestr = "complex128"  # what set_dtype("complex128") does
    assert resolve_dtype(None, b) == torch.complex128
    assert resolve_dtype("complex64", b) == torch.complex64  # the engine argument wins
    monkeypatch.setenv("TYXONQ_GB300_DTYPE", "complex128")
    assert resolve_dtype(None, _Backend()) == torch.complex128
