"""Batched persistent-kernel VQE: energies and adjoint gradients against the
oracle (reverse-sweep restatement of the reference's civector_ops adjoint),
against the plain one-launch-per-gate engine, across every size class, with
and without CUDA-graph replay.

Tolerances: complex128 1e-10 absolute; complex64 energies 1e-5 x ||c||_1 of
the instance's Hamiltonian, gradients 1e-4 x ||c||_1."""
import numpy as np
import pytest
import torch

from oracle import sv

pytestmark = pytest.mark.gpu


def _oracle(inst):
    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()]
    return sv.grad_adjoint(inst.n, gates, inst.theta, inst.H.codes, inst.H.coeffs)


def _instances(count, seed, n_range, depth_range=(1, 3), terms_range=(10, 60)):
    from tyxonq_gb300.workloads import batched_vqe

    return batched_vqe(count, seed=seed, n_range=n_range, depth_range=depth_range, terms_range=terms_range)


@pytest.mark.parametrize("large", ["waves", "cta"])
@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_batched_matches_oracle_all_classes(dtype, large):
    from tyxonq_gb300.batch import BatchedVQE, Schedule

    insts = _instances(40, 5, (3, 13))
    # small tiles so that 11- to 13-qubit instances take the large-instance path too
    sched = Schedule(res8_max=6, res4_max=8, res2_max=9, res1_max=10, t_fwd=9, t_adj=8, large=large, wave_t=9,
                     wave_hbits=8, wave_budget=1 << 16)
    if dtype == torch.complex128:
        sched = Schedule(res8_max=6, res4_max=8, res2_max=9, res1_max=10, t_fwd=8, t_adj=7, large=large, wave_t=9,
                         wave_hbits=8, wave_budget=1 << 16)
    bv = BatchedVQE(insts, dtype=dtype, schedule=sched)
    theta = np.concatenate([i.theta for i in insts])
    e, g = bv.run(theta)
    e = e.cpu().numpy()
    grads = bv.split_grads(g.cpu().numpy())
    assert {c.name for c in bv.launch_order} >= {"res1", "res8"}
    if large == "waves":
        assert bv.waves is not None and len(bv.waves.waves) > 1
    else:
        assert "streamed" in {c.name for c in bv.launch_order}
    for k, inst in enumerate(insts):
        e_ref, g_ref = _oracle(inst)
        nrm = inst.H.one_norm()
        if dtype == torch.complex128:
            assert abs(e[k] - e_ref) < 1e-10, (k, inst.n)
            np.testing.assert_allclose(grads[k], g_ref, atol=1e-10)
        else:
            assert abs(e[k] - e_ref) < 1e-5 * nrm, (k, inst.n, e[k], e_ref)
            np.testing.assert_allclose(grads[k], g_ref, atol=1e-4 * nrm)


def test_batched_default_schedule_vs_plain_engine_and_graph_replay():
    from tyxonq_gb300.batch import BatchedVQE, plain_energy_and_grad

    insts = _instances(24, 9, (8, 20), depth_range=(2, 4), terms_range=(50, 120))
    bv = BatchedVQE(insts, dtype=torch.complex64)
    theta = np.concatenate([i.theta for i in insts])
    e1, g1 = [x.cpu().numpy().copy() for x in bv.run(theta)]
    bv.capture()
    e2, g2 = [x.cpu().numpy().copy() for x in bv.run(theta)]
    np.testing.assert_array_equal(e1, e2)  # deterministic, graph replay identical
    np.testing.assert_array_equal(g1, g2)
    grads = bv.split_grads(g1)
    for k, inst in enumerate(insts):
        ep, gp = plain_energy_and_grad(inst)
        nrm = inst.H.one_norm()
        assert abs(e1[k] - ep) < 1e-5 * nrm, (k, inst.n)
        np.testing.assert_allclose(grads[k], gp, atol=1e-4 * nrm)
        if inst.n <= 12:
            e_ref, g_ref = _oracle(inst)
            assert abs(e1[k] - e_ref) < 1e-5 * nrm
            np.testing.assert_allclose(grads[k], g_ref, atol=1e-4 * nrm)


def test_plain_engine_gradient_matches_oracle_c128():
    from tyxonq_gb300.batch import plain_energy_and_grad

    for inst in _instances(6, 13, (5, 12)):
        e, g = plain_energy_and_grad(inst, dtype=torch.complex128)
        e_ref, g_ref = _oracle(inst)
        assert abs(e - e_ref) < 1e-10
        np.testing.assert_allclose(g, g_ref, atol=1e-10)


def test_new_theta_changes_results_consistently():
    from tyxonq_gb300.batch import BatchedVQE

    insts = _instances(8, 21, (6, 15))
    bv = BatchedVQE(insts, dtype=torch.complex128)
    bv.capture()
    rng = np.random.default_rng(4)
    for _ in range(2):
        th = rng.uniform(0, 2 * np.pi, bv.n_theta)
        e, g = bv.run(th)
        e = e.cpu().numpy()
        grads = bv.split_grads(g.cpu().numpy())
        o = 0
        for k, inst in enumerate(insts):
            inst.theta = th[o:o + inst.n_params]
            o += inst.n_params
            e_ref, g_ref = _oracle(inst)
            assert abs(e[k] - e_ref) < 1e-10
            np.testing.assert_allclose(grads[k], g_ref, atol=1e-10)


def test_three_bit_adjoint_stages_match_oracle():
    """Wave adjoint with 3-bit register stages (8 amplitudes of psi and lam per thread)."""
    from tyxonq_gb300.batch import BatchedVQE, Schedule

    insts = _instances(6, 33, (14, 15))
    sc = Schedule.default(torch.complex64)
    sc.wave_adj_stage_bits = 3
    bv = BatchedVQE(insts, dtype=torch.complex64, schedule=sc)
    assert bv.waves is not None and bv.waves.adj_rb == 3
    e, g = bv.run(np.concatenate([i.theta for i in insts]))
    e = e.cpu().numpy()
    grads = bv.split_grads(g.cpu().numpy())
    for k, inst in enumerate(insts):
        e_ref, g_ref = _oracle(inst)
        norm = inst.H.one_norm()
        assert abs(e[k] - e_ref) < 1e-5 * norm
        np.testing.assert_allclose(grads[k], g_ref, atol=1e-4 * norm)


def test_plain_engine_graph_replay_matches_oracle():
    """The benchmark's plain baseline: one launch per gate, captured once per
    instance as a CUDA graph and replayed."""
    from tyxonq_gb300.batch import PlainEngine

    for inst in _instances(4, 17, (6, 14)):
        eng = PlainEngine(inst, dtype=torch.complex128)
        eng.capture()
        for _ in range(2):  # replays start from |basis> every time
            eng.run()
            e, g = eng.result()
            e_ref, g_ref = _oracle(inst)
            assert abs(e - e_ref) < 1e-10
            np.testing.assert_allclose(g, g_ref, atol=1e-10)


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_specialised_wave_kernels_match_interpreter_and_oracle(dtype):
    """Wave passes through the circuit-specialised kernels against the library's
    interpreting wave kernels and the oracle (14-16 qubits: every instance in waves)."""
    from dataclasses import replace

    from tyxonq_gb300.batch import BatchedVQE, Schedule

    insts = _instances(10, 41, (14, 16), depth_range=(1, 4), terms_range=(20, 80))
    theta = np.concatenate([i.theta for i in insts])
    base = Schedule.builtin(dtype)
    res = {}
    for jit in (1, 0):
        bv = BatchedVQE(insts, dtype=dtype, schedule=replace(base, wave_jit=jit))
        assert bv.waves is not None and (len(bv.waves.jit_sub) > 0) == bool(jit)
        e, g = bv.run(theta)
        res[jit] = (e.cpu().numpy().copy(), bv.split_grads(g.cpu().numpy()))
    tol_e = 1e-10 if dtype == torch.complex128 else 1e-5
    tol_g = 1e-10 if dtype == torch.complex128 else 1e-4
    for k, inst in enumerate(insts):
        e_ref, g_ref = _oracle(inst)
        for jit in (1, 0):
            assert abs(res[jit][0][k] - e_ref) < tol_e, (jit, k)
            np.testing.assert_allclose(res[jit][1][k], g_ref, atol=tol_g)
