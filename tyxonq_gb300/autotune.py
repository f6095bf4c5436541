"""Schedule autotuner, timing candidates on the device.

* Batched VQE (``tune_batched``): coordinate descent over the launch schedule
  of ``BatchedVQE`` -- size-class boundaries (which qubit counts stay in one
  CTA's shared memory), wave tile width, wave L2 budget, number of wave lanes,
  adjoint register-stage width, ops per wave pass -- each candidate built,
  captured as a CUDA graph and timed over whole evaluation steps.  The result
  is saved as JSON (``save_schedule``); ``Schedule.default`` loads the file
  for the current GPU (``TYXONQ_GB300_SCHEDULE`` or the package's
  ``tuned/<gpu>.json``), so the benchmark and the tests run the tuned
  schedule.  ``python -m tyxonq_gb300.autotune`` re-tunes on the benchmark's
  4096-instance workload and writes the file.
* Single-state programs (``tune_forward``, ``tune_forward_sizes``;
  ``python -m tyxonq_gb300.autotune --forward 20 24 28``): tile width (local
  qubits per shared-memory tile pass) per (n, dtype), saved in
  ``TYXONQ_GB300_TUNE`` (default ``~/.cache/tyxonq_gb300/tune.json``) and
  read once per process by ``tile_bits_for``, which ``compile_forward`` and the
  adjoint paths use when no width is given.  Untuned sizes use defaults from
  shared-memory capacity: a complex64 tile of 2^13 amplitudes is 64 KiB.
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


_LOADED = False


def tile_bits_for(n: int, dtype, adjoint: bool = False) -> int:
    """Tile width for an n-qubit program: the tuned one (the cache file is read
    once per process) or the shared-memory default."""
    global _LOADED
    if not _LOADED:
        _LOADED = True
        try:
            load()
        except (OSError, ValueError):  # an unreadable cache only costs the defaults
            pass
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



# ---------------------------------------------------------------- batched schedule
TUNED_DIR = Path(__file__).resolve().parent / "tuned"
SCHEDULE_FIELDS = ("res8_max", "res4_max", "res2_max", "res1_max", "wave_t", "wave_hbits", "wave_budget",
                   "wave_lanes", "wave_max_ops", "wave_adj_stage_bits", "wave_jit", "wave_fork")


def _gpu_tag(device=None) -> str:
    name = torch.cuda.get_device_name(device) if torch.cuda.is_available() else "cpu"
    return "".join(c if c.isalnum() else "_" for c in name).strip("_").lower()


def schedule_path(device=None) -> Path:
    env = os.environ.get("TYXONQ_GB300_SCHEDULE")
    return Path(env) if env else TUNED_DIR / f"{_gpu_tag(device)}.json"


def load_schedule(dtype, device=None) -> dict | None:
    """Tuned schedule fields for dtype on this GPU, or None."""
    p = schedule_path(device)
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    ent = d.get("c64" if dtype == torch.complex64 else "c128")
    if not ent:
        return None
    return {k: int(v) for k, v in ent["schedule"].items() if k in SCHEDULE_FIELDS}


def save_schedule(dtype, fields: dict, table: list, workload: str, device=None, path: Path | None = None) -> Path:
    p = Path(path or schedule_path(device))
    p.parent.mkdir(parents=True, exist_ok=True)
    d = json.loads(p.read_text()) if p.exists() else {}
    d["gpu"] = torch.cuda.get_device_name(device)
    d["c64" if dtype == torch.complex64 else "c128"] = {
        "schedule": {k: int(fields[k]) for k in SCHEDULE_FIELDS}, "workload": workload,
        "tuned_at": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
        "candidates_ms": table}
    p.write_text(json.dumps(d, indent=1))
    return p


def _candidates(field: str, cur: dict, dtype) -> list:
    c64 = dtype == torch.complex64
    top = 13 if c64 else 12
    if field == "res1_max":
        return [top - 1, top]
    if field == "res2_max":
        return [v for v in (top - 2, top - 1) if v <= cur["res1_max"]]
    if field == "res4_max":
        return [v for v in (top - 3, top - 2) if v <= cur["res2_max"]]
    if field == "res8_max":
        return [v for v in (top - 4, top - 3) if v <= cur["res4_max"]]
    if field == "wave_t":
        return [11, 12, 13] if c64 else [11, 12]
    if field == "wave_budget":
        return [32 << 20, 48 << 20, 64 << 20, 96 << 20, 128 << 20]
    if field == "wave_lanes":
        return [1, 2, 3, 4]
    if field == "wave_fork":
        return [0, 1]
    if field == "wave_adj_stage_bits":
        return [3, 4]
    if field == "wave_max_ops":
        return [128, 256]
    return [cur[field]]


def time_batched(instances, schedule, dtype=torch.complex64, steps: int = 3, flush=None) -> float:
    """Median ms of one graph-replayed evaluation of the instances under `schedule`
    (an L2-sized buffer written before every timed step)."""
    import numpy as np

    from .batch import BatchedVQE

    bv = BatchedVQE(instances, dtype=dtype, schedule=schedule)
    bv.set_theta(np.concatenate([i.theta for i in instances]))
    bv.capture()
    if flush is None:
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=bv.device)
    bv.run()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        bv.run()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    del bv
    ts.sort()
    return ts[len(ts) // 2]


def tune_batched(instances, dtype=torch.complex64, steps: int = 3, order: Sequence[str] | None = None,
                 log: Callable[[str], None] | None = None):
    """Coordinate descent over the batched schedule, from the faster of the
    builtin schedule and the one saved for this GPU; returns (Schedule,
    [(fields, ms)] of every candidate timed)."""
    from dataclasses import asdict, replace

    from .batch import Schedule

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    table = []
    starts = [Schedule.builtin(dtype)]
    saved = load_schedule(dtype)
    if saved:
        starts.append(replace(starts[0], **saved))
    best, best_ms = None, float("inf")
    for st in starts:
        ms = time_batched(instances, st, dtype, steps, flush)
        table.append(({k: asdict(st)[k] for k in SCHEDULE_FIELDS}, ms))
        if log:
            log(f"start {'saved' if st is not starts[0] else 'builtin'}: {ms:.2f} ms")
        if ms < best_ms:
            best, best_ms = st, ms
    cur = asdict(best)
    for field in order or ("wave_fork", "wave_lanes", "wave_budget", "wave_adj_stage_bits", "wave_t", "wave_max_ops",
                           "res1_max", "res2_max", "res4_max", "res8_max"):
        for v in _candidates(field, cur, dtype):
            if v == cur[field]:
                continue
            trial = dict(cur)
            trial[field] = v
            if field == "wave_t":
                trial["wave_hbits"] = v
            try:
                ms = time_batched(instances, replace(best, **{k: trial[k] for k in SCHEDULE_FIELDS}), dtype, steps,
                                  flush)
            except Exception as e:  # a candidate that does not fit (shared memory, L2) is skipped
                if log:
                    log(f"{field}={v}: skipped ({e})")
                continue
            table.append(({k: trial[k] for k in SCHEDULE_FIELDS}, ms))
            if log:
                log(f"{field}={v}: {ms:.2f} ms (best {best_ms:.2f})")
            if ms < best_ms:
                best_ms, cur = ms, trial
                best = replace(best, **{k: trial[k] for k in SCHEDULE_FIELDS})
    return best, table


def tune_forward_sizes(sizes: Sequence[int], depth: int = 40, dtype=torch.complex64,
                       log: Callable[[str], None] | None = None) -> dict:
    """Forward tile widths for random circuits (the 28-qubit benchmark circuit's
    generator) of the given sizes; saved to the cache file that tile_bits_for
    reads.  Returns {n: (best t, {t: ms})}."""
    from .ir import lower_ops
    from .workloads import random_circuit

    class _C:
        def __init__(self, n, ops):
            self.num_qubits, self.ops = n, ops

    out = {}
    for n in sizes:
        gates, _ = lower_ops(_C(n, random_circuit(n, depth, seed=1)), mode="run")
        best, res = tune_forward(gates, n, dtype)
        out[n] = (best, res)
        if log:
            log(f"forward n={n}: t={best} ({', '.join(f'{t}: {ms:.2f} ms' for t, ms in sorted(res.items()))})")
    save()
    return out


def main() -> None:
    import argparse

    from .workloads import batched_vqe

    ap = argparse.ArgumentParser(description="tune the batched VQE schedule (and optionally the single-state "
                                             "forward tile widths) on this GPU")
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--out", default=None)
    ap.add_argument("--forward", type=int, nargs="*", default=None,
                    help="also tune the forward tile width for random circuits of these qubit counts")
    args = ap.parse_args()
    if args.forward:
        tune_forward_sizes(args.forward, log=lambda m: print(m, flush=True))
    insts = batched_vqe(args.count, seed=3)
    sched, table = tune_batched(insts, steps=args.steps, log=lambda m: print(m, flush=True))
    from dataclasses import asdict

    p = save_schedule(torch.complex64, asdict(sched), [[f, ms] for f, ms in table],
                      f"batched_vqe({args.count}, seed=3)", path=args.out)
    print(json.dumps({"schedule": {k: asdict(sched)[k] for k in SCHEDULE_FIELDS}, "file": str(p)}))


if __name__ == "__main__":
    main()
