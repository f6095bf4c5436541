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
    np.testing.assert_allclose(psi.cpu().numpy(), [0, 1], atol=1e-6)
