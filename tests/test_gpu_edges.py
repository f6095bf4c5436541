"""Edge cases of the reference's API on the GPU path: empty circuits and
Hamiltonians, one-qubit states, repeated qubits, out-of-range qubits, single
shots, tiny batches."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import sv

pytestmark = pytest.mark.gpu

C64, C128 = torch.complex64, torch.complex128


class _C:
    def __init__(self, n, ops):
        self.num_qubits = n
        self.ops = list(ops)


def _engine(dtype=C128, fusion="fused"):
    from tyxonq_gb300.engine import GpuStatevectorEngine

    return GpuStatevectorEngine(dtype=dtype, fusion=fusion, seed=3)


@pytest.mark.parametrize("fusion", ["plain", "fused"])
def test_empty_and_one_qubit_circuits(fusion):
    eng = _engine(fusion=fusion)
    np.testing.assert_allclose(eng.state(_C(0, [])).cpu().numpy(), [1.0])
    np.testing.assert_allclose(eng.state(_C(3, [])).cpu().numpy(), sv.init_state(3))
    out = eng.run(_C(2, []), shots=0)
    assert out["expectations"] == {}
    ops = [("h", 0), ("rx", 0, 0.3), ("s", 0), ("ry", 0, 1.1), ("sdg", 0), ("rz", 0, -0.7), ("x", 0)]
    psi = eng.state(_C(1, ops)).cpu().numpy()
    ref, _ = sv.run_ops(1, ops)
    np.testing.assert_allclose(psi, ref, atol=1e-12)
    res = eng.run(_C(1, ops + [("measure_z", 0)]), shots=1)
    assert sum(res["result"].values()) == 1 and set(res["result"]) <= {"0", "1"}


def test_repeated_qubit_two_qubit_gates_are_no_ops():
    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import kernels as K

    rng = np.random.default_rng(1)
    v = rng.normal(size=8) + 1j * rng.normal(size=8)
    psi = K.from_array(v / np.linalg.norm(v), dtype=C128)
    before = psi.clone()
    P = ctypes.c_void_p(psi.data_ptr())
    for name in ("tq_sv_apply_cx", "tq_sv_apply_cz", "tq_sv_apply_swap"):
        nat.call(name, P, 3, 1, 1, 1, K.stream_ptr())
    nat.call("tq_sv_apply_2q", P, 3, 1, 2, 2, K._mat(np.eye(4) * 1j, 4), K.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(psi, before)
    # through the engine: cx(q, q) and rxx(q, q, a) are skipped as in the reference
    ops = [("h", 0), ("cx", 1, 1), ("rxx", 2, 2, 0.4), ("cz", 0, 0)]
    np.testing.assert_allclose(_engine().state(_C(3, ops)).cpu().numpy(), sv.run_ops(3, ops)[0], atol=1e-12)


def test_out_of_range_qubits_raise():
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300._native import TqError

    psi = K.init_statevector(4, dtype=C64)
    with pytest.raises(TqError):
        K.apply_1q(psi, np.eye(2), 4)
    with pytest.raises(TqError):
        K.apply_cx(psi, 0, 7)
    with pytest.raises(ValueError):
        _engine().state(_C(2, [("h", 2)]))


def test_empty_and_identity_hamiltonians():
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.hamiltonian import PauliSum

    psi = K.init_statevector(5, dtype=C128)
    K.apply_1q(psi, np.array([[1, 1], [1, -1]]) / np.sqrt(2), 2)
    empty = PauliSum.from_terms(5, [])
    assert float(K.pauli_expectation(psi, empty).item()) == 0.0
    ident = PauliSum.from_terms(5, [(1.75, [])])
    assert abs(float(K.pauli_expectation(psi, ident).item()) - 1.75) < 1e-14


def test_large_shot_count_small_state():
    eng = _engine()
    ops = [("ry", 0, 1.0), ("measure_z", 0)]
    res = eng.run(_C(1, ops), shots=1_000_000)
    p1 = np.sin(0.5) ** 2
    frac1 = res["result"].get("1", 0) / 1e6
    assert abs(frac1 - p1) < 5 * np.sqrt(p1 * (1 - p1) / 1e6)


def test_kraus_status_boundaries():
    from tests import golden_data

    sets = golden_data.kraus_sets()
    eng = _engine()
    ops0 = [("h", 0), ("kraus", 0, "k", 0.0)]
    ops1 = [("h", 0), ("kraus", 0, "k", 1.0)]
    for ops in (ops0, ops1):
        c = _C(1, ops)
        c._kraus_cache = {"k": sets["amp_damp"]}
        psi = eng.state(c).cpu().numpy()
        ref, _ = sv.run_ops(1, ops, kraus_cache={"k": sets["amp_damp"]})
        np.testing.assert_allclose(psi, ref, atol=1e-12)


def test_tiny_batches():
    from tyxonq_gb300.batch import BatchedVQE
    from tyxonq_gb300.workloads import batched_vqe

    for insts in (batched_vqe(1, seed=4, n_range=(3, 3)), batched_vqe(3, seed=5, n_range=(2, 4))):
        bv = BatchedVQE(insts, dtype=C128)
        e, g = bv.run(np.concatenate([i.theta for i in insts]))
        e = e.cpu().numpy()
        grads = bv.split_grads(g.cpu().numpy())
        for k, inst in enumerate(insts):
            e_ref, g_ref = sv.grad_adjoint(inst.n, [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()],
                                           inst.theta, inst.H.codes, inst.H.coeffs)
            assert abs(e[k] - e_ref) < 1e-10
            np.testing.assert_allclose(grads[k], g_ref, atol=1e-10)
