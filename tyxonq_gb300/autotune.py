"""Schedule autotuner: tile width (local qubits per shared-memory tile pass)
and batched-kernel launch shape, picked by timing candidates on the device.

Tuned choices are kept in memory per process and can be saved to / loaded
from a JSON file (``TYXONQ_GB300_TUNE``, default ``~/.cache/tyxonq_gb300/tune.json``).
Untuned sizes use defaults derived from shared-memory capacity: a complex64
tile of 2^13 amplitudes is 64 KiB, so two forward tiles fit per SM.
"""
from __future__ import annotations

import json
import os
import time
from pathlib import Path
from typing import Callable, Sequence

import torch

_TUNED: dict[str, int] = {}


def _key(kind: str, n: int, dtype) -> str:
    return f"{kind}:{n}:{'c64' if dtype == torch.complex64 else 'c128'}"


def _default(n: int, dtype, adjoint: bool) -> int:
    cap = 13 if dtype == torch.complex64 else 12
    if adjoint:
        cap -= 1
    return max(1, min(n, cap))


def tile_bits_for(n: int, dtype, adjoint: bool = False) -> int:
    k = _key("adj" if adjoint else "fwd", n, dtype)
    if k in _TUNED:
        return min(_TUNED[k], n)
    return _default(n, dtype, adjoint)


def set_tile_bits(n: int, dtype, adjoint: bool, t: int) -> None:
    _TUNED[_key("adj" if adjoint else "fwd", n, dtype)] = int(t)


def cache_path() -> Path:
    return Path(os.environ.get("TYXONQ_GB300_TUNE", Path.home() / ".cache" / "tyxonq_gb300" / "tune.json"))


def save(path: Path | None = None) -> None:
    p = Path(path or cache_path())
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps(_TUNED, indent=1, sort_keys=True))


def load(path: Path | None = None) -> None:
    p = Path(path or cache_path())
    if p.exists():
        _TUNED.update({k: int(v) for k, v in json.loads(p.read_text()).items()})


def time_callable(fn: Callable[[], None], reps: int = 5, warmup: int = 2) -> float:
    """Median device time (ms) of fn() with CUDA events on the current stream."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    ts.sort()
    return ts[len(ts) // 2]


def tune_tile_bits(make_fn: Callable[[int], Callable[[], None]], candidates: Sequence[int], reps: int = 5) -> tuple[int, dict]:
    """Time make_fn(t)() for each candidate t; return (best t, {t: ms})."""
    res = {}
    for t in candidates:
        try:
            res[t] = time_callable(make_fn(t), reps=reps)
        except Exception:  # a candidate that does not fit is skipped
            continue
    if not res:
        raise RuntimeError("no tile width candidate ran")
    best = min(res, key=res.get)
    return best, res


def tune_forward(gates, n: int, dtype=torch.complex64, candidates: Sequence[int] | None = None) -> tuple[int, dict]:
    """Pick the forward tile width for an n-qubit gate program by timing."""
    from . import kernels as K
    from .program import compile_forward

    cap = 14 if dtype == torch.complex64 else 13
    cands = [t for t in (candidates or range(max(6, n - 16), cap + 1)) if 1 <= t <= min(n, cap)]
    psi = K.init_statevector(n, dtype=dtype)

    def make(t):
        prog = compile_forward(gates, n, dtype, t=t)
        return lambda: prog.run(psi)

    best, res = tune_tile_bits(make, cands)
    set_tile_bits(n, dtype, False, best)
    return best, res


_ = time  # re-exported for callers timing on the host
