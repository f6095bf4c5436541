"""Benchmark: VQE energy+grad evals/s (batched vs plain GPU), gate HBM GB/s.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).  See the design doc for the workload definitions,
algorithmic-byte formulas and how each number is measured.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "VQE energy+grad evals/s batched vs plain GPU; p50/p99 latency; gate HBM GB/s"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self._p = None
        self._t = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self._p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._p = None
        return self

    def _read(self):
        for line in self._p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self._p is not None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
        if self._t is not None:
            self._t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    """The reference's CPU algorithm (oracle port: state by per-gate tensor
    contraction, Pauli-sum energy, adjoint gradient) on a bounded sample of the
    batched workload, across host cores."""
    import multiprocessing as mp

    import numpy as np

    from tyxonq_gb300.workloads import batched_vqe

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    insts = batched_vqe(4096, seed=3)
    rng = np.random.default_rng(11)
    sample_ids = rng.choice(len(insts), size=48, replace=False)
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t_steps = []
    with ctx.Pool(cores) as pool:
        for s in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_ref_one, [(int(i),) for i in sample_ids])
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                t_steps.append(dt)
    per_step = sum(t_steps) / len(t_steps)
    evals_s = len(sample_ids) / per_step
    line = {"impl": "reference", "metric": METRIC, "value": evals_s, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "batched_vqe_4096 (8-20 qubits, depth 2-8, 50-500 Pauli terms)",
                       "parallelism": f"{cores} host processes"},
            "cpu_baseline": {"value": evals_s, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": f"{len(sample_ids)} random instances of the 4096 per step"},
            "e2e": {"value": evals_s, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


_REF_CACHE = {}


def _ref_one(arg):
    (i,) = arg
    from oracle import sv
    from tyxonq_gb300.workloads import batched_vqe

    if "insts" not in _REF_CACHE:
        _REF_CACHE["insts"] = batched_vqe(4096, seed=3)
    inst = _REF_CACHE["insts"][i]
    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()]
    e, g = sv.grad_adjoint(inst.n, gates, inst.theta, inst.H.codes, inst.H.coeffs)
    return e


# ------------------------------------------------------------------ our arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.build()
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward
    from tyxonq_gb300.workloads import random_circuit

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    class _C:
        def __init__(self, n, ops):
            self.num_qubits, self.ops = n, ops

    # ---------------- config 2: 28 qubits, depth 40, complex64, fused tile passes
    n2 = 28
    ops = random_circuit(n2, 40, seed=1)
    gates, _ = lower_ops(_C(n2, ops), mode="run")
    prog = compile_forward(gates, n2, torch.complex64)
    psi = K.init_statevector(n2, dtype=torch.complex64)
    S = 8
    N = 1 << n2
    launch_ms = []

    def timed_fused():
        # per-launch events on the launching stream
        st = torch.cuda.current_stream()
        evs = []
        from tyxonq_gb300 import _native as nat
        import ctypes

        for kind, obj in prog.segments:
            assert kind == "tiles"
            ops_d = obj.device_ops(psi.device)
            for p in range(obj.n_passes):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(st)
                nat.call("tq_sv_run_tiles", ctypes.c_void_p(psi.data_ptr()), n2, 0,
                         ctypes.byref(obj.passes[p]), 1, ctypes.c_void_p(ops_d.data_ptr()), None, K.stream_ptr())
                b.record(st)
                evs.append((a, b))
        return evs

    for _ in range(args.warmup):
        prog.run(psi)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        t_total = 0.0
        for _ in range(args.steps):
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            evs = timed_fused()
            b.record()
            torch.cuda.synchronize()
            t_total += a.elapsed_time(b)
            launch_ms += [x.elapsed_time(y) for x, y in evs]
    fused_ms = t_total / args.steps
    n_pass = prog.n_passes
    avg_launch_ms = sum(launch_ms) / len(launch_ms)
    alg_bytes = 2 * N * S
    achieved = alg_bytes / (avg_launch_ms * 1e-3) / 1e9
    peak, peak_kind = _peaks()

    # unfused plain engine on the same circuit (one step)
    from tyxonq_gb300.engine import execute_plain

    psi2 = K.init_statevector(n2, dtype=torch.complex64)
    execute_plain(psi2, gates[:40])
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    execute_plain(psi2, gates)
    b.record()
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b)
    del psi, psi2
    torch.cuda.empty_cache()

    # ---------------- interim batched value: per-instance fused adjoint on a sample
    from tyxonq_gb300.adjoint import AdjointEstimator, ParamGate
    from tyxonq_gb300.ir import Gate, _rot_gate
    from tyxonq_gb300.workloads import batched_vqe

    insts = batched_vqe(4096, seed=3)[:64]
    ests = []
    for inst in insts:
        pg = [ParamGate(_rot_gate(nm, qs, 0.0), p) if p is not None else ParamGate(Gate(nm, qs))
              for nm, qs, p in inst.structure()]
        ests.append((AdjointEstimator(inst.n, pg, inst.n_params, inst.H), inst.theta))
    for e, th in ests[:4]:
        e.energy_and_grad(th)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for e, th in ests:
        e.energy_and_grad(th)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    evals_s = len(ests) / seq_s

    line = {
        "metric": METRIC, "value": evals_s, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": seq_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": "interim: first 64 instances of batched_vqe_4096, sequential fused adjoint",
                   "l2": "28q state 2 GiB > L2"},
        "gate_kernels": {"fused_28q_depth40_ms": fused_ms, "plain_28q_depth40_ms": plain_ms, "passes": n_pass,
                         "gates": len(gates)},
        "roofline": {"kernel": "k_tile_forward (28q c64 tile pass)", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": peak_kind},
        "clocks": clk.summary(),
        "gpu_launches": len(launch_ms),
    }
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
