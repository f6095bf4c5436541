"""Generate golden vectors by running the reference (TyxonQ) itself.

Run from the repository root, in a checkout that has the reference sources:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <TyxonQ src folder>

(or with the folder in the environment variable TYXONQ_SRC).

It imports TyxonQ from the given source tree and records, for seeded inputs:
  * final states of small circuits through StatevectorEngine.state() and the
    <Z_q> expectations of StatevectorEngine.run() (every supported gate,
    unitary ops, projections);
  * apply_kqubit_unitary outputs for k = 1..5;
  * Pauli-sum energies through pauli_string_sum_dense + dynamics.expectation;
  * the 12-qubit hardware-efficient TFIM energy (numpy and pytorch backends)
    and its PyTorch-autograd gradient;
  * circuits with one-qubit Kraus channels (explicit status): final states,
    <Z_q>, and <Z_q> under use_noise depolarizing attenuation;
  * expval_pauli_sum energies and per-term expectations from counts.
Outputs: tests/golden/golden.npz (arrays) and tests/golden/golden.json
(circuits and scalars).  The reference is not needed to *use* the fixtures.
"""
from __future__ import annotations

import json
import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def main(ref_src: str) -> None:
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_src)
    import warnings

    warnings.filterwarnings("ignore")
    import tyxonq as tq
    from tyxonq.core.ir import Circuit
    from tyxonq.devices.simulators.statevector.engine import StatevectorEngine
    from tyxonq.libs.quantum_library import dynamics
    from tyxonq.libs.quantum_library.kernels import statevector as ksv
    from tyxonq.libs.quantum_library.kernels.pauli import pauli_string_sum_dense

    tq.set_backend("numpy")
    arrays: dict[str, np.ndarray] = {}
    meta: dict = {"circuits": [], "kq": [], "pauli": [], "hea12": {}}
    rng = np.random.default_rng(20261203)

    one_q = ["h", "x", "s", "sdg", "y", "z", "t", "tdg"]
    rot1 = ["rx", "ry", "rz"]
    two_q = ["cx", "cz", "swap", "iswap"]
    rot2 = ["rxx", "ryy", "rzz", "cry"]

    def random_ops(n: int, depth: int) -> list:
        ops = []
        for _ in range(depth):
            r = rng.random()
            if r < 0.35:
                ops.append((str(rng.choice(one_q)), int(rng.integers(n))))
            elif r < 0.6:
                ops.append((str(rng.choice(rot1)), int(rng.integers(n)), float(rng.uniform(0, 2 * math.pi))))
            elif r < 0.8 and n >= 2:
                a, b = rng.choice(n, 2, replace=False)
                ops.append((str(rng.choice(two_q)), int(a), int(b)))
            elif n >= 2:
                a, b = rng.choice(n, 2, replace=False)
                ops.append((str(rng.choice(rot2)), int(a), int(b), float(rng.uniform(0, 2 * math.pi))))
        return ops

    eng = StatevectorEngine()
    cases = [(1, 6), (2, 12), (3, 20), (4, 30), (5, 40), (7, 60), (9, 80), (11, 80)]
    for ci, (n, depth) in enumerate(cases):
        ops = random_ops(n, depth)
        # a unitary op (1q and 2q) and a projection in the larger cases
        ucache = {}
        if n >= 3:
            q = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
            U2, _ = np.linalg.qr(q)
            q1 = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
            U1, _ = np.linalg.qr(q1)
            ucache = {"u2": U2, "u1": U1}
            ops.insert(len(ops) // 2, ("unitary", 1, 0, "u2"))
            ops.insert(len(ops) // 3, ("unitary", 2, "u1"))
            arrays[f"c{ci}_u2"] = U2
            arrays[f"c{ci}_u1"] = U1
        if n >= 4:
            ops.append(("project_z", 1, 0))
            ops.append(("h", 1))
        c = Circuit(n, ops=[tuple(o) for o in ops])
        if ucache:
            c._unitary_cache = dict(ucache)
        psi = np.asarray(eng.state(c), dtype=np.complex128)
        ops_m = list(ops) + [("measure_z", q) for q in range(n)]
        c2 = Circuit(n, ops=[tuple(o) for o in ops_m])
        if ucache:
            c2._unitary_cache = dict(ucache)
        out = eng.run(c2, shots=0)
        z = [out["expectations"][f"Z{q}"] for q in range(n)]
        arrays[f"c{ci}_state"] = psi
        arrays[f"c{ci}_runz"] = np.asarray(z, dtype=np.float64)
        meta["circuits"].append({"name": f"c{ci}", "n": n, "ops": [list(o) for o in ops],
                                 "unitaries": sorted(ucache)})

    # apply_kqubit_unitary, k = 1..5 on 7 qubits
    for k in range(1, 6):
        n = 7
        psi0 = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        psi0 /= np.linalg.norm(psi0)
        q = rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k))
        U, _ = np.linalg.qr(q)
        qubits = [int(x) for x in rng.choice(n, k, replace=False)]
        out = np.asarray(ksv.apply_kqubit_unitary(psi0, U, qubits, n), dtype=np.complex128)
        arrays[f"kq{k}_in"] = psi0
        arrays[f"kq{k}_u"] = U
        arrays[f"kq{k}_out"] = out
        meta["kq"].append({"k": k, "n": n, "qubits": qubits})

    # Pauli-sum energies via the dense reference path
    for pi_, n in enumerate([3, 5, 7, 8]):
        K = 12 + 6 * pi_
        codes = np.zeros((K, n), dtype=np.int64)
        for t in range(K):
            w = int(rng.integers(1, min(4, n) + 1))
            qs = rng.choice(n, w, replace=False)
            codes[t, qs] = rng.integers(1, 4, size=w)
        codes[0, :] = 0  # identity term
        weights = rng.standard_normal(K)
        psi0 = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        psi0 /= np.linalg.norm(psi0)
        H = np.asarray(pauli_string_sum_dense(codes.tolist(), weights.tolist()))
        e = float(np.real(np.asarray(dynamics.expectation(psi0, H))))
        arrays[f"ps{pi_}_codes"] = codes
        arrays[f"ps{pi_}_w"] = weights
        arrays[f"ps{pi_}_psi"] = psi0
        arrays[f"ps{pi_}_hpsi"] = H @ psi0
        meta["pauli"].append({"name": f"ps{pi_}", "n": n, "energy": e})

    # 12q HEA [RY all; CX ladder] x 4, TFIM, theta ~ U[0, 2pi) from default_rng(0)
    n, L = 12, 4
    theta = np.random.default_rng(0).uniform(0, 2 * math.pi, (L, n))
    codes = []
    weights = []
    for i in range(n - 1):
        t = [0] * n
        t[i] = 3
        t[i + 1] = 3
        codes.append(t)
        weights.append(-1.0)
    for i in range(n):
        t = [0] * n
        t[i] = 1
        codes.append(t)
        weights.append(-1.0)
    H = np.asarray(pauli_string_sum_dense(codes, weights))

    def build(th):
        c = Circuit(n)
        for l in range(L):
            for q in range(n):
                c.ry(q, th[l][q])
            for q in range(n - 1):
                c.cx(q, q + 1)
        return c

    psi = np.asarray(build(theta).state(), dtype=np.complex128)
    e_np = float(np.real(np.asarray(dynamics.expectation(psi, H))))
    import torch

    tq.set_backend("pytorch")
    th_t = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    psi_t = build(th_t).state()
    Ht = torch.as_tensor(H)
    e_t = torch.real(torch.conj(psi_t) @ (Ht @ psi_t))
    e_t.backward()
    grad = th_t.grad.detach().numpy().copy()
    tq.set_backend("numpy")
    arrays["hea12_theta"] = theta
    arrays["hea12_state"] = psi
    arrays["hea12_grad_autograd"] = grad
    arrays["hea12_codes"] = np.asarray(codes, dtype=np.int64)
    arrays["hea12_w"] = np.asarray(weights)
    meta["hea12"] = {"n": n, "layers": L, "energy_numpy": e_np, "energy_pytorch": float(e_t.item())}

    # Kraus channels (stochastic unravelling with explicit status) and use_noise
    meta["noise"] = []
    g1, g2 = 0.2, 0.3
    kraus_sets = {
        "amp_damp": [np.array([[1, 0], [0, math.sqrt(1 - g1)]]), np.array([[0, math.sqrt(g1)], [0, 0]])],
        "phase_damp": [np.array([[1, 0], [0, math.sqrt(1 - g2)]]), np.array([[0, 0], [0, math.sqrt(g2)]])],
        "depol": [math.sqrt(1 - 0.75 * 0.1) * np.eye(2), math.sqrt(0.1 / 4) * np.array([[0, 1], [1, 0]]),
                  math.sqrt(0.1 / 4) * np.array([[0, -1j], [1j, 0]]), math.sqrt(0.1 / 4) * np.array([[1, 0], [0, -1]])],
    }
    for ni, n in enumerate([3, 5, 6]):
        ops = random_ops(n, 12 + 4 * ni)
        c = Circuit(n, ops=[tuple(o) for o in ops])
        kr = []
        for j in range(4):
            name = ["amp_damp", "phase_damp", "depol", "amp_damp"][j]
            q = int(rng.integers(n))
            st = float(rng.uniform(0, 1))
            c.kraus(q, kraus_sets[name], status=st)
            kr.append([name, q, st])
            for o in random_ops(n, 3):
                c.ops.append(tuple(o))
        psi = np.asarray(eng.state(c), dtype=np.complex128)
        c_m = Circuit(n, ops=list(c.ops) + [("measure_z", q) for q in range(n)])
        c_m._kraus_cache = dict(c._kraus_cache)
        z = eng.run(c_m, shots=0)["expectations"]
        zn = eng.run(c_m, shots=0, use_noise=True, noise={"type": "depolarizing", "p": 0.05})["expectations"]
        arrays[f"nz{ni}_state"] = psi
        arrays[f"nz{ni}_runz"] = np.asarray([z[f"Z{q}"] for q in range(n)])
        arrays[f"nz{ni}_runz_depol"] = np.asarray([zn[f"Z{q}"] for q in range(n)])
        names = {id(v): k for k, v in kraus_sets.items()}
        meta["noise"].append({"name": f"nz{ni}", "n": n, "ops": [list(o) for o in c.ops],
                              "kraus": {k: names[id(v)] for k, v in c._kraus_cache.items()}})
    meta["kraus_sets"] = {k: [[[complex(x).real, complex(x).imag] for x in np.asarray(m).reshape(-1)] for m in v]
                          for k, v in kraus_sets.items()}

    # shot-count postprocessing: expval_pauli_sum over a random counts histogram
    from tyxonq.postprocessing.counts_expval import expval_pauli_sum

    meta["counts"] = []
    for ci, n in enumerate([3, 6]):
        keys = rng.integers(0, 1 << n, size=40)
        counts = {format(int(k), f"0{n}b"): int(rng.integers(1, 50)) for k in keys}
        items = []
        for _ in range(8):
            w = int(rng.integers(1, min(4, n) + 1))
            qs = sorted(int(x) for x in rng.choice(n, w, replace=False))
            items.append((tuple((q, "Z") for q in qs), float(rng.normal())))
        res = expval_pauli_sum(counts, items, identity_const=0.25)
        meta["counts"].append({"n": n, "counts": counts, "items": [[list(map(list, t)), c] for t, c in items],
                               "energy": res["energy"], "expvals": res["expvals"]})

    np.savez_compressed(HERE / "golden.npz", **arrays)
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1))
    print("energy hea12:", e_np, float(e_t.item()))


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TYXONQ_SRC")
    if not src:
        sys.exit("usage: make_golden.py <TyxonQ src folder>  (or set TYXONQ_SRC)")
    main(src)
