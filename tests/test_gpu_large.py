"""A 33-qubit complex64 state (2^33 amplitudes, 64 GiB): indices above 2^32
through the single-gate kernels and the fused register-staged passes.  A
random circuit run fused and then undone gate by gate returns |0...0>."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N_QUBITS = 33


def _inverse(g):
    from tyxonq_gb300.ir import Gate

    if g.kind in ("cx", "cz", "swap"):
        return g
    return Gate(g.kind, g.qubits, g.mat.conj().T)


def test_33_qubit_circuit_then_inverse():
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.engine import execute_plain
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward
    from tyxonq_gb300.workloads import random_circuit

    free, _ = torch.cuda.mem_get_info()
    if free < (80 << 30):
        pytest.skip("needs 80 GiB of free device memory")
    n = N_QUBITS

    class _C:
        def __init__(self, ops):
            self.num_qubits, self.ops = n, ops

    rng_ops = random_circuit(n, 4, seed=9)
    gates, _ = lower_ops(_C(rng_ops), mode="run")
    psi = K.init_statevector(n, dtype=torch.complex64)
    prog = compile_forward(gates, n, torch.complex64)
    prog.run(psi)
    nrm = float(K.norm2(psi).item())
    assert abs(nrm - 1.0) < 1e-3
    execute_plain(psi, [_inverse(g) for g in reversed(gates)])
    torch.cuda.synchronize()
    a0 = complex(psi[0].item())
    assert abs(abs(a0) - 1.0) < 1e-3, a0
    # an amplitude above 2^32 stays zero
    assert abs(complex(psi[(1 << 32) + 12345].item())) < 1e-3
    del psi
    torch.cuda.empty_cache()
