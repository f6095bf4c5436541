"""tyxonq_gb300 -- GB300-native statevector engine for TyxonQ.

Hot path: hand-written sm_103a CUDA kernels in libtyxonq_gb300.so (C ABI in
include/tq_sv.h) for gate application (single gates and fused shared-memory
tile passes), Pauli-sum expectation and H*psi, probabilities and shot
sampling, and adjoint gradients.  Python host code mirrors the reference's
engine / numerics interfaces so it drops into TyxonQ:

    from tyxonq_gb300 import GpuStatevectorEngine, install
    install()   # TyxonQ's simulator driver and Circuit.state() now use the GPU engine
"""
from __future__ import annotations

__version__ = "0.1.0"

from .engine import GpuStatevectorEngine  # noqa: E402
from .hamiltonian import PauliSum  # noqa: E402


def install(replace_statevector: bool = True, alias: str = "statevector_gpu"):
    from .plugin import install as _install

    return _install(replace_statevector=replace_statevector, alias=alias)


def library():
    """Load (building if needed) libtyxonq_gb300.so and return the ctypes handle."""
    from . import _native

    return _native.load()
