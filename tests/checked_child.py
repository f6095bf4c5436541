"""Child process of tests/test_gpu_checked.py: runs on the checked library
variant (TYXONQ_GB300_CHECKED=1, library kernels only) and prints one JSON
line with the largest deviation from the oracle per case family and the
device-side check status.

Exhaustive tiny cases: every gate kind of the single-gate kernels on every
qubit (and every ordered qubit pair, and several triples) of 1..6-qubit random
states in complex64 and complex128, Pauli rotations on every qubit pair; then
a 14-qubit fused program, the tiled H psi, sampling and a small batched VQE
with waves through the interpreting kernels."""
import itertools
import json
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
os.environ["TYXONQ_GB300_CHECKED"] = "1"
os.environ["TYXONQ_GB300_JIT"] = "0"

import numpy as np  # noqa: E402
import torch  # noqa: E402

from oracle import sv  # noqa: E402
from tyxonq_gb300 import _native as nat  # noqa: E402
from tyxonq_gb300 import kernels as K  # noqa: E402

rng = np.random.default_rng(17)
err: dict = {}


def note(kind, a, b):
    err[kind] = max(err.get(kind, 0.0), float(np.abs(np.asarray(a) - np.asarray(b)).max()))


def rand_state(n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def rand_u(d):
    return np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]


for dtype in (torch.complex64, torch.complex128):
    tag = "c64" if dtype == torch.complex64 else "c128"
    for n in range(1, 7):
        for q in range(n):
            v = rand_state(n)
            u = rand_u(2)
            note(f"1q_{tag}", K.apply_1q(K.from_array(v, dtype=dtype), u, q).cpu().numpy(), sv.apply_1q(v, u, q, n))
            d0, d1 = np.exp(1j * rng.uniform(0, 6.3, 2))
            note(f"diag_{tag}", K.apply_diag1(K.from_array(v, dtype=dtype), d0, d1, q).cpu().numpy(),
                 sv.apply_1q(v, np.diag([d0, d1]), q, n))
            note(f"phase_{tag}", K.apply_diag1(K.from_array(v, dtype=dtype), 1.0, d1, q).cpu().numpy(),
                 sv.apply_1q(v, np.diag([1.0, d1]), q, n))
        for a, b in itertools.permutations(range(n), 2):
            v = rand_state(n)
            u = rand_u(4)
            note(f"2q_{tag}", K.apply_2q(K.from_array(v, dtype=dtype), u, a, b).cpu().numpy(),
                 sv.apply_2q(v, u, a, b, n))
            note(f"cx_{tag}", K.apply_cx(K.from_array(v, dtype=dtype), a, b).cpu().numpy(),
                 sv.apply_2q(v, sv.g_cx(), a, b, n))
            note(f"cz_{tag}", K.apply_cz(K.from_array(v, dtype=dtype), a, b).cpu().numpy(),
                 sv.apply_2q(v, sv.g_cz(), a, b, n))
            note(f"swap_{tag}", K.apply_swap(K.from_array(v, dtype=dtype), a, b).cpu().numpy(),
                 sv.apply_2q(v, sv.g_swap(), a, b, n))
            for pa, pb in (("X", "X"), ("Y", "Z"), ("Z", "Y"), ("X", "Y")):
                t = float(rng.uniform(-3, 3))
                P = np.kron(sv.PAULI[pa], sv.PAULI[pb])
                note(f"prot_{tag}", K.apply_pauli_rotation(K.from_array(v, dtype=dtype), [(a, pa), (b, pb)],
                                                          t).cpu().numpy(),
                     sv.apply_kq(v, sv.g_rot(t, P), [a, b], n))
        for k in range(3, min(n, 5) + 1):
            for qs in list(itertools.permutations(range(n), k))[:12]:
                v = rand_state(n)
                u = rand_u(1 << k)
                note(f"kq_{tag}", K.apply_kq(K.from_array(v, dtype=dtype), u, qs).cpu().numpy(),
                     sv.apply_kq(v, u, list(qs), n))

# a fused program (interpreting staged kernel), the tiled H psi, sampling
from tyxonq_gb300.hamiltonian import random_pauli_sum  # noqa: E402
from tyxonq_gb300.ir import lower_ops  # noqa: E402
from tyxonq_gb300.program import compile_forward  # noqa: E402
from tyxonq_gb300.workloads import random_circuit  # noqa: E402


class _C:
    def __init__(self, n, ops):
        self.num_qubits, self.ops = n, ops


n = 14
ops = random_circuit(n, 12, seed=5)
gates, _ = lower_ops(_C(n, ops), mode="run")
psi = K.init_statevector(n, dtype=torch.complex128)
compile_forward(gates, n, torch.complex128).run(psi)
ref, _ = sv.run_ops(n, ops, mode="run")
note("program_c128", psi.cpu().numpy(), ref)
H = random_pauli_sum(n, 200, rng)
out = torch.empty_like(psi)
e = torch.empty(1, dtype=torch.float64, device="cuda")
K._pauli_sum_tiled(psi, H, n, out, e)
note("hpsi_c128", out.cpu().numpy(), sv.apply_pauli_sum(ref, H.codes, H.coeffs))
idx = K.sample(psi, 4096, seed=3).cpu().numpy()
err["sample_in_range"] = float(0.0 if (idx >= 0).all() and (idx < (1 << n)).all() else 1.0)

# a small batched VQE through the waves (interpreting wave kernels)
from tyxonq_gb300.batch import BatchedVQE  # noqa: E402
from tyxonq_gb300.workloads import batched_vqe  # noqa: E402

insts = [i for i in batched_vqe(256, seed=3) if i.n >= 14][:6] + batched_vqe(8, seed=4)
bv = BatchedVQE(insts, dtype=torch.complex64)
bv.set_theta(np.concatenate([i.theta for i in insts]))
energies, _ = bv.run()
energies = energies.cpu().numpy()
for i, inst in enumerate(insts):
    g = [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()]
    e_ref, _ = sv.grad_adjoint(inst.n, g, inst.theta, inst.H.codes, inst.H.coeffs)
    err["batched_energy_c64"] = max(err.get("batched_energy_c64", 0.0), abs(float(energies[i]) - e_ref))

torch.cuda.synchronize()
checked, site, index = nat.check_status()
print(json.dumps({"checked": checked, "site": site, "index": index, "library": str(nat.library_path()),
                  "err": err}))
