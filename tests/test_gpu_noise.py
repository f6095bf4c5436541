"""GPU engine with Kraus channels and use_noise, against the reference's own
outputs (golden vectors) and the oracle's noisy sampling distribution."""
import math

import numpy as np
import pytest
import torch

from oracle import sv
from tests import golden_data

pytestmark = pytest.mark.gpu

C64, C128 = torch.complex64, torch.complex128


class _C:
    def __init__(self, n, ops, kraus=None, ucache=None):
        self.num_qubits = n
        self.ops = list(ops)
        self._kraus_cache = dict(kraus or {})
        self._unitary_cache = dict(ucache or {})


def _engine(dtype, fusion="fused", seed=7):
    from tyxonq_gb300.engine import GpuStatevectorEngine

    return GpuStatevectorEngine(dtype=dtype, fusion=fusion, seed=seed)


@pytest.mark.parametrize("fusion", ["plain", "fused"])
@pytest.mark.parametrize("case", golden_data.noise_cases(), ids=lambda c: c[0])
def test_kraus_golden_c128(case, fusion):
    name, n, ops, kc, state, runz, runz_depol = case
    eng = _engine(C128, fusion)
    psi = eng.state(_C(n, ops, kc)).cpu().numpy()
    np.testing.assert_allclose(psi, state, atol=1e-12, rtol=0)
    ops_m = list(ops) + [("measure_z", q) for q in range(n)]
    out = eng.run(_C(n, ops_m, kc), shots=0)
    np.testing.assert_allclose([out["expectations"][f"Z{q}"] for q in range(n)], runz, atol=1e-12, rtol=0)
    out = eng.run(_C(n, ops_m, kc), shots=0, use_noise=True, noise={"type": "depolarizing", "p": 0.05})
    np.testing.assert_allclose([out["expectations"][f"Z{q}"] for q in range(n)], runz_depol, atol=1e-12, rtol=0)


@pytest.mark.parametrize("case", golden_data.noise_cases(), ids=lambda c: c[0])
def test_kraus_golden_c64(case):
    name, n, ops, kc, state, runz, runz_depol = case
    psi = _engine(C64).state(_C(n, ops, kc)).cpu().numpy()
    np.testing.assert_allclose(psi, state, atol=2e-6 * math.sqrt(len(ops) + 1), rtol=0)


def test_kraus_without_status_uses_seeded_engine_rng():
    sets = golden_data.kraus_sets()
    n = 6
    ops = [("h", q) for q in range(n)] + [("kraus", q, f"k{q}") for q in range(n)]
    kc = {f"k{q}": sets["amp_damp"] for q in range(n)}
    a = _engine(C128, seed=11).state(_C(n, ops, kc)).cpu().numpy()
    b = _engine(C128, seed=11).state(_C(n, ops, kc)).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    assert abs(np.linalg.norm(a) - 1.0) < 1e-12


def test_kraus_trajectory_average_matches_channel():
    """Average of many trajectories of amplitude damping on |1>: P(0) -> gamma."""
    sets = golden_data.kraus_sets()
    eng = _engine(C128, seed=5)
    ones = 0
    T = 400
    for _ in range(T):
        psi = eng.state(_C(1, [("x", 0), ("kraus", 0, "k")], {"k": sets["amp_damp"]})).cpu().numpy()
        ones += abs(psi[1]) ** 2 > 0.5
    frac0 = 1 - ones / T
    assert abs(frac0 - 0.2) < 4 * math.sqrt(0.2 * 0.8 / T)


@pytest.mark.parametrize("noise", [
    {"type": "depolarizing", "p": 0.2},
    {"type": "readout", "cals": {0: np.array([[0.9, 0.2], [0.1, 0.8]]), 3: np.array([[0.85, 0.1], [0.15, 0.9]])}},
], ids=["depolarizing", "readout"])
def test_noisy_sampling_distribution(noise):
    n = 5
    rng = np.random.default_rng(9)
    ops = [("h", q) for q in range(n)] + [("ry", q, float(rng.uniform(0, 6))) for q in range(n)] + \
          [("cx", q, q + 1) for q in range(n - 1)]
    ops_m = ops + [("measure_z", q) for q in range(n)]
    eng = _engine(C128)
    out = eng.run(_C(n, ops_m), shots=200000, use_noise=True, noise=noise, seed=123)
    psi, _ = sv.run_ops(n, ops, mode="run")
    p = sv.noisy_probabilities(psi, n, noise)
    assert sv.chi2_pvalue(out["result"], p) > 1e-4


@pytest.mark.parametrize("dtype,tol", [(C128, 1e-12), (C64, 1e-5)])
def test_kraus_trajectory_batch_matches_oracle_per_trajectory(dtype, tol):
    """64 trajectories of a noisy circuit in one batch (run_trajectories):
    every trajectory's <Z_q> equals the oracle's single-trajectory unravelling
    (apply_kraus_statevector restated) with the same statuses, and the mean
    equals their average."""
    sets = golden_data.kraus_sets()
    n, T = 7, 64
    rng = np.random.default_rng(4)
    ops = []
    kc = {"ad": sets["amp_damp"], "pd": sets["phase_damp"], "dp": sets["depol"]}
    for layer in range(3):
        for q in range(n):
            ops.append(("ry", q, float(rng.uniform(0, 2 * np.pi))))
        for q in range(n - 1):
            ops.append(("cx", q, q + 1))
        for q in range(0, n, 2):
            ops.append(("kraus", q, ["ad", "pd", "dp"][(q + layer) % 3]))
    ops.append(("kraus", 1, "ad", 0.5))  # an explicit status: the same for every trajectory
    ops += [("measure_z", q) for q in range(n)]
    eng = _engine(dtype)
    out = eng.run_trajectories(_C(n, ops, kc), T, seed=21, per_trajectory=True)
    assert out["trajectories"] == T
    per = out["per_trajectory"]
    stat = out["statuses"]
    for t in range(T):
        j, ops_t = 0, []
        for op in ops:
            if op[0] == "kraus" and len(op) == 3:
                ops_t.append(("kraus", op[1], op[2], float(stat[j][t])))
                j += 1
            elif op[0] == "kraus":
                ops_t.append(op)
                j += 1
            else:
                ops_t.append(op)
        psi, meas = sv.run_ops(n, ops_t, mode="run", kraus_cache=kc)
        z = [sv.expect_z(psi, q, n) for q in meas]
        np.testing.assert_allclose(per[t], z, atol=tol, rtol=0, err_msg=f"trajectory {t}")
    mean = [out["expectations"][f"Z{q}"] for q in range(n)]
    np.testing.assert_allclose(mean, per.mean(axis=0), atol=tol, rtol=0)
    # distinct trajectories actually took different branches
    assert np.unique(np.round(per[:, 0], 6)).size > 1
