"""ctypes binding of libtyxonq_gb300.so (the C ABI in ``include/tq_sv.h``).

The shared library is the only compute path of this package: there is no
CPU fallback.  If the library is missing and cannot be built (no nvcc), or no
CUDA device is visible, the first call raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, c_double, c_int, c_int64, c_size_t, c_uint64, c_void_p

from . import _build

TQ_C64 = 0
TQ_C128 = 1
TQ_MAX_QUBITS = 34
TQ_MAX_KQ = 5

TQ_OK = 0
ERR_NAMES = {
    -1: "TQ_ERR_ARG",
    -2: "TQ_ERR_CUDA",
    -3: "TQ_ERR_RANGE",
    -4: "TQ_ERR_TIMEOUT",
    -5: "TQ_ERR_WORKSPACE",
    -6: "TQ_ERR_UNSUPPORTED",
}


class TqError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


class PauliGroup(ctypes.Structure):
    _fields_ = [("flip", ctypes.c_uint64), ("first_term", ctypes.c_int32), ("n_terms", ctypes.c_int32)]


class PauliTerm(ctypes.Structure):
    _fields_ = [("zy", ctypes.c_uint64), ("w_re", ctypes.c_double), ("w_im", ctypes.c_double),
                ("f_re", ctypes.c_float), ("f_im", ctypes.c_float)]


_P = c_void_p
_D = POINTER(c_double)
_I = POINTER(c_int)

# name -> (restype, argtypes); the set of names is exactly the exported ABI.
SIGNATURES: dict[str, tuple] = {
    "tq_version": (c_int, []),
    "tq_last_error": (c_int, [ctypes.c_char_p, c_size_t]),
    "tq_sv_init_basis": (c_int, [_P, c_int, c_int, c_int64, _P]),
    "tq_sv_apply_1q": (c_int, [_P, c_int, c_int, c_int, _D, _P]),
    "tq_sv_apply_diag1": (c_int, [_P, c_int, c_int, c_int, _D, _P]),
    "tq_sv_apply_2q": (c_int, [_P, c_int, c_int, c_int, c_int, _D, _P]),
    "tq_sv_apply_cx": (c_int, [_P, c_int, c_int, c_int, c_int, _P]),
    "tq_sv_apply_cz": (c_int, [_P, c_int, c_int, c_int, c_int, _P]),
    "tq_sv_apply_swap": (c_int, [_P, c_int, c_int, c_int, c_int, _P]),
    "tq_sv_apply_kq": (c_int, [_P, c_int, c_int, _I, c_int, _D, _P]),
    "tq_sv_apply_pauli_rotation": (c_int, [_P, c_int, c_int, c_uint64, c_uint64, c_double, _P]),
    "tq_sv_scale": (c_int, [_P, c_int, c_int, c_double, c_double, _P]),
    "tq_sv_expect_z_workspace_bytes": (c_size_t, [c_int]),
    "tq_sv_expect_z_all": (c_int, [_P, c_int, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_probabilities": (c_int, [_P, c_int, c_int, _P, _P]),
    "tq_sv_qubit_rdm_workspace_bytes": (c_size_t, [c_int]),
    "tq_sv_qubit_rdm": (c_int, [_P, c_int, c_int, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_norm_workspace_bytes": (c_size_t, [c_int]),
    "tq_sv_norm2": (c_int, [_P, c_int, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_sample_workspace_bytes": (c_size_t, [c_int, c_int64]),
    "tq_sv_sample": (c_int, [_P, c_int, c_int, c_int64, c_uint64, _P, _P, c_size_t, _P]),
    "tq_sv_sample_noalloc": (c_int, [_P, c_int, c_int, c_int64, c_uint64, _P, _P]),
    "tq_sv_pauli_expectation_workspace_bytes": (c_size_t, [c_int, c_int]),
    "tq_sv_pauli_expectation": (c_int, [_P, c_int, c_int, _P, c_int, _P, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_apply_pauli_sum": (c_int, [_P, _P, c_int, c_int, _P, c_int, _P, c_int, _P]),
    "tq_sv_tile_max_bits": (c_int, [c_int]),
    "tq_sv_run_staged": (c_int, [_P, c_int, c_int, _P, c_int, _P, _P, _P, _P]),
    "tq_sv_run_tiles": (c_int, [_P, c_int, c_int, _P, c_int, _P, _P, _P]),
    "tq_traj_kraus_workspace_bytes": (c_size_t, [c_int, c_int]),
    "tq_traj_kraus": (c_int, [_P, c_int, c_int, c_int, c_int, _P, c_int, _P, _P, _P, c_size_t, _P]),
    "tq_jit_build": (c_int, [ctypes.c_char_p, _P, c_int, _P, _P, ctypes.c_char_p, c_size_t]),
    "tq_jit_free_host": (None, [_P]),
    "tq_jit_load": (c_int, [_P, c_size_t, ctypes.c_char_p, _P]),
    "tq_jit_unload": (c_int, [_P]),
    "tq_jit_rops_bytes": (c_size_t, [c_int, c_int]),
    "tq_jit_run_staged": (c_int, [_P, c_int, _P, c_int, c_int, _P, c_int, _P, _P, _P, c_int, _P, _P, c_size_t, _P]),
    "tq_jit_wave_run": (c_int, [_P, c_int, c_int, _P, c_int, c_int, _P, _P, _P, _P, _P, _P, _P, c_int, _P]),
    "tq_wave_rops": (c_int, [c_int, _P, c_int, _P, _P, _P, _P]),
    "tq_check_status": (c_int, [_P, _P]),
    "tq_sv_adjoint_tiles_workspace_bytes": (c_size_t, [c_int, c_int]),
    "tq_sv_adjoint_tiles": (c_int, [_P, _P, c_int, c_int, _P, c_int, _P, _P, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_generator_im": (c_int, [_P, _P, c_int, c_int, c_uint64, c_uint64, c_uint64, _P, _P, c_size_t, _P]),
    "tq_sv_inner_workspace_bytes": (c_size_t, [c_int]),
    "tq_sv_inner_re": (c_int, [_P, _P, c_int, c_int, _P, _P, c_size_t, _P]),
    "tq_ci_apply_excitations": (c_int, [_P, _P, c_int64, _P, _P, _P, _P, _P, c_int, c_int, _P]),
    "tq_ci_adjoint_workspace_bytes": (c_size_t, [c_int64, c_int]),
    "tq_ci_adjoint": (c_int, [_P, _P, c_int64, _P, _P, _P, _P, _P, c_int, _P, _P, c_size_t, _P]),
    "tq_ci_dot_workspace_bytes": (c_size_t, [c_int64]),
    "tq_ci_dot": (c_int, [_P, _P, c_int64, _P, _P, c_size_t, _P]),
    "tq_ci_embed": (c_int, [_P, _P, c_int64, _P, c_int, c_int, _P]),
    "tq_ci_gather": (c_int, [_P, _P, c_int64, c_int, _P, _P]),
    "tq_ci_spmv": (c_int, [_P, _P, _P, c_int64, _P, _P, _P]),
    "tq_sv_pauli_sum_tiled_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int]),
    "tq_sv_pauli_sum_tiled": (c_int, [_P, _P, c_int, c_int, _P, c_int, _P, c_int, _P, _P, c_size_t, _P]),
    "tq_sv_apply_excitations": (c_int, [_P, c_int, c_int, _P, c_int, _P, c_int, _P]),
    "tq_sv_excitation_adjoint_workspace_bytes": (c_size_t, [c_int, c_int]),
    "tq_sv_excitation_adjoint": (c_int, [_P, _P, c_int, c_int, _P, c_int, _P, _P, _P, c_size_t, _P]),
    "tq_ci_pairs_max_dim": (c_int64, [c_int]),
    "tq_ci_energy_grad_workspace_bytes": (c_size_t, [c_int64, c_int64]),
    "tq_ci_energy_grad": (c_int, [c_int64, c_int64, c_int, _P, _P, c_int64, _P, c_int64, _P, _P, _P, _P, c_int, c_int,
                                  _P, _P, _P, c_size_t, _P]),
    "tq_batch_smem_bytes": (c_size_t, [c_int, c_int, c_int, c_int]),
    "tq_wave_run": (c_int, [c_int, c_int, _P, c_int, c_int, c_int, c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, c_int,
                            _P]),
    "tq_wave_normalize": (c_int, [_P, _P, _P, _P, _P, _P, c_int, _P, _P, _P]),
    "tq_wave_reduce": (c_int, [_P, _P, _P, _P, _P, _P, c_int, _P, c_int, _P]),
    "tq_batch_run": (c_int, [c_int, _P, _P, c_int, c_int, c_int, c_int, c_int, c_size_t, _P, _P, _P, _P, _P, _P,
                             _P, _P, _P, _P]),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def checked() -> bool:
    """TYXONQ_GB300_CHECKED=1 selects the checked library variant (device-side
    index checks; read with check_status())."""
    return os.environ.get("TYXONQ_GB300_CHECKED", "0") not in ("", "0")


def library_path():
    return _build.CHECKED_LIB_PATH if checked() else _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the shared library and bind its ABI."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        chk = checked()
        if _build.needs_build(chk):
            if not build_if_missing:
                raise RuntimeError(f"{library_path()} is not built; run tyxonq_gb300._build.build()")
            _build.build(checked=chk)
        lib = ctypes.CDLL(str(library_path()))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check_status() -> tuple[bool, int, int]:
    """(checked build, first failing check site TQ_SITE_* or 0, its index);
    clears the recorded failure."""
    lib = load()
    site, index = ctypes.c_uint(0), ctypes.c_longlong(0)
    rc = lib.tq_check_status(ctypes.byref(site), ctypes.byref(index))
    if rc < 0:
        check(rc)
    return rc == 1, int(site.value), int(index.value)


def last_error() -> tuple[int, str]:
    lib = load()
    buf = ctypes.create_string_buffer(512)
    code = lib.tq_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != TQ_OK:
        _, msg = last_error()
        raise TqError(rc, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def dbl_array(values) -> ctypes.Array:
    vals = [float(v) for v in values]
    return (c_double * len(vals))(*vals)


def int_array(values) -> ctypes.Array:
    vals = [int(v) for v in values]
    return (c_int * len(vals))(*vals)
