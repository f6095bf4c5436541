"""tq_sv_sample_noalloc: sampling for callers that cannot allocate device memory.

The entry point uses a fixed scratch array inside the library instead of a
caller workspace.  It must give exactly the indices tq_sv_sample gives for the
same state, shots and seed (sampled indices are integers: compared exactly),
on consecutive calls that reuse the shared scratch, and it must refuse sizes
beyond its fixed scratch.  Collected last (file name) so a failure here does
not hide the rest of the suite under -x.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib, psi, n, dtag, shots, seed):
    out = torch.full((shots,), -1, dtype=torch.int64, device=psi.device)
    rc = lib.tq_sv_sample_noalloc(ctypes.c_void_p(psi.data_ptr()), n, dtag, shots, seed,
                                  ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out


def _with_workspace(lib, psi, n, dtag, shots, seed):
    ws = torch.empty(lib.tq_sv_sample_workspace_bytes(n, shots), dtype=torch.uint8, device=psi.device)
    out = torch.full((shots,), -1, dtype=torch.int64, device=psi.device)
    rc = lib.tq_sv_sample(ctypes.c_void_p(psi.data_ptr()), n, dtag, shots, seed, ctypes.c_void_p(out.data_ptr()),
                          ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out


def _state(n, seed, dtype):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v[rng.random(1 << n) < 0.3] = 0  # zero-probability amplitudes must never be drawn
    v /= np.linalg.norm(v)
    return torch.from_numpy(v).to(dtype=dtype, device="cuda"), v


@pytest.mark.parametrize("dtype,dtag", [(torch.complex64, 0), (torch.complex128, 1)])
def test_noalloc_matches_workspace_sampler_on_consecutive_calls(dtype, dtag):
    from tyxonq_gb300 import _native

    lib = _native.load()
    # two calls in a row with different sizes: the second reuses the scratch the first left behind
    for n, shots, seed in ((14, 50_000, 7), (9, 3_000, 8)):
        psi, v = _state(n, seed, dtype)
        rc1, a = _noalloc(lib, psi, n, dtag, shots, seed)
        rc2, b = _with_workspace(lib, psi, n, dtag, shots, seed)
        torch.cuda.synchronize()
        assert rc1 == 0 and rc2 == 0, _native.last_error()
        a, b = a.cpu().numpy(), b.cpu().numpy()
        np.testing.assert_array_equal(a, b)
        assert (np.diff(a) >= 0).all() and a.min() >= 0 and a.max() < (1 << n)
        assert np.all(np.abs(v[a]) > 0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from tyxonq_gb300 import _native

    lib = _native.load()
    psi = torch.zeros(1 << 10, dtype=torch.complex64, device="cuda")
    psi[0] = 1
    rc, _ = _noalloc(lib, psi, 10, 0, 2_000_000, 1)
    assert rc == -3
    code, msg = _native.last_error()
    assert "scratch" in msg
