"""The benchmark's own 4096-instance batched workload against the oracle.

The whole workload (n ~ U{8..20}, HEA depth ~ U{2..8}, 50-500 Pauli terms,
seed 3) is compiled with the default schedule and replayed as a CUDA graph,
exactly as the benchmark runs it.  For every qubit count n = 8..20 the
deepest instance and the instance with the most Hamiltonian terms are
compared with the oracle's reverse-sweep energy and gradient
(``oracle.sv.grad_adjoint``, complex128).

Tolerances (complex64 state, FP64 accumulation): energies 1e-5 absolute;
gradients 1e-4 absolute.  The oracle runs in a spawn pool started before the
first CUDA call.
"""
import multiprocessing as mp

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E_TOL = 1e-5
G_TOL = 1e-4


def _oracle_one(args):
    n, structure, theta, codes, coeffs = args
    from oracle import sv

    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in structure]
    return sv.grad_adjoint(n, gates, theta, codes, coeffs)


def _selected(insts):
    by_n: dict = {}
    for i, inst in enumerate(insts):
        by_n.setdefault(inst.n, []).append(i)
    sel = []
    for n in sorted(by_n):
        ids = by_n[n]
        deep = max(ids, key=lambda i: (insts[i].depth, insts[i].H.n_terms))
        wide = max(ids, key=lambda i: (insts[i].H.n_terms, insts[i].depth))
        sel += [deep] + ([wide] if wide != deep else [])
    return sel


def test_bench_workload_matches_oracle_at_full_size():
    from tyxonq_gb300.workloads import batched_vqe

    insts = batched_vqe(4096, seed=3)
    sel = _selected(insts)
    assert {insts[i].n for i in sel} == set(range(8, 21))
    # largest first so the pool's longest jobs start first
    order = sorted(sel, key=lambda i: -(insts[i].n * 100 + insts[i].depth))
    jobs = [(insts[i].n, insts[i].structure(), insts[i].theta, insts[i].H.codes, insts[i].H.coeffs) for i in order]
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(min(len(jobs), 16))
    pending = pool.map_async(_oracle_one, jobs, chunksize=1)

    from tyxonq_gb300.batch import BatchedVQE

    bv = BatchedVQE(insts, dtype=torch.complex64)
    theta = np.concatenate([i.theta for i in insts])
    bv.capture()
    e, g = bv.run(theta)
    e = e.cpu().numpy()
    grads = bv.split_grads(g.cpu().numpy())
    ref = dict(zip(order, pending.get(timeout=1800)))
    pool.close()
    pool.join()
    rows = []
    for i in sel:
        e_ref, g_ref = ref[i]
        rows.append((abs(e[i] - e_ref), float(np.abs(grads[i] - g_ref).max()), i))
    rows.sort(reverse=True)
    print(f"\n{len(sel)} instances n=8..20: max |dE| = {rows[0][0]:.3e}, "
          f"max |dgrad| = {max(r[1] for r in rows):.3e}")
    for de, dg, i in rows[:6]:
        print(f"  instance {i}: n={insts[i].n} depth={insts[i].depth} terms={insts[i].H.n_terms} "
              f"|dE|={de:.3e} |dgrad|={dg:.3e}")
    for de, dg, i in rows:
        assert de < E_TOL, (i, insts[i].n, insts[i].depth, insts[i].H.n_terms, de)
        assert dg < G_TOL, (i, insts[i].n, insts[i].depth, insts[i].H.n_terms, dg)


@pytest.mark.parametrize("n,depth,terms", [(22, 6, 800), (24, 4, 500), (26, 2, 200)])
def test_serving_size_energies_match_c_oracle(n, depth, terms):
    """Serving-size requests (HEA, complex64, one state through the session
    estimator) against the C complex128 oracle: 1e-5 absolute on the energy."""
    from oracle import csv
    from tyxonq_gb300.serving import VqeRequest, default_estimator_factory
    from tyxonq_gb300.hamiltonian import random_pauli_sum
    from tyxonq_gb300.workloads import hea_rz_ops_params

    rng = np.random.default_rng(n)
    H = random_pauli_sum(n, terms, rng)
    struct = hea_rz_ops_params(n, depth)
    npar = 2 * n * depth
    theta = rng.uniform(0, 2 * np.pi, npar)
    req = VqeRequest("s", n, struct, npar, H, theta)
    est = default_estimator_factory(req, torch.complex64, torch.device("cuda"))
    e = est.energy(theta)
    ops = [(nm, *qs) if p is None else (nm, *qs, float(theta[p])) for nm, qs, p in struct]
    psi = csv.run_ops(n, ops)
    e_ref = csv.pauli_expectation(psi, H.codes, H.coeffs)
    print(f"\nn={n}: |dE| = {abs(e - e_ref):.3e}")
    assert abs(e - e_ref) < E_TOL
