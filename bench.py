"""Benchmark: VQE energy+grad evals/s (batched vs plain GPU), gate HBM GB/s.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0): batched energy + adjoint-gradient evaluations
per second of 4096 seeded VQE instances (graph replay, L2 flushed between
steps), the same end to end from host parameters to host results, the plain
one-launch-per-gate engine on a sample, serving latency percentiles, the
28-qubit fused circuit and single-gate HBM bandwidths, per-call times of the
12-qubit HEA (energy, gradient, 4096 shots) and the 16-qubit UCCSD, the
roofline of the fused pass kernel, a CPU baseline and SM clocks sampled during
the timed steps.
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

# DRAM bytes read + written by one tq_jit_staged_pass launch of the 28-qubit
# circuit (mean of the two passes of the ncu capture summarised in
# profiles/tq_jit_staged_pass_28q_c64.txt)
STAGED_PASS_DRAM_BYTES = 4.2358e9
# DRAM bytes per item of the specialised wave adjoint (psi and lam tiles of 2^12
# complex64 amplitudes): ncu capture of tq_jit_wave_adjoint on the 512-instance
# batch, 256 / 512 / 768 items per launch, 65.7-66.5 KB each; ncu flushes the
# caches before a captured launch, so this is the cold-cache figure (the tiles'
# first reads), an upper bound for the benchmark's L2-resident waves
WAVE_ADJ_DRAM_BYTES_PER_ITEM = 6.6e4
# fraction of cycles the same capture's schedulers issued an instruction
# (smsp__issue_active, 768-item launch)
WAVE_ADJ_ISSUE_ACTIVE = 0.497


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
    contraction, Pauli-sum energy, adjoint gradient) on a bounded, size-
    stratified sample of the batched workload, one single-threaded process per
    host core.  Each timed step evaluates two instances of every size n = 8..20;
    the per-size mean CPU time, weighted by the workload's count of each size and
    divided by the cores, gives the evals/s of the whole 4096-instance workload
    (perfect scaling over cores assumed, which favours the reference).  Warm-up
    steps evaluate the instances up to 12 qubits."""
    import multiprocessing as mp

    from tyxonq_gb300.workloads import batched_vqe

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    insts = batched_vqe(4096, seed=3)
    by_n: dict = {}
    for i, inst in enumerate(insts):
        by_n.setdefault(inst.n, []).append(i)
    sample = [i for n in sorted(by_n) for i in by_n[n][:2]]
    warm = [i for i in sample if insts[i].n <= 12]
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t_steps, est = [], []
    with ctx.Pool(cores, initializer=_ref_worker_init) as pool:
        for s in range(args.warmup + args.steps):
            ids = warm if s < args.warmup else sample
            t0 = time.perf_counter()
            times = pool.map(_ref_one, [(int(i),) for i in ids], chunksize=1)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                t_steps.append(dt)
                per_n: dict = {}
                for i, t in zip(ids, times):
                    per_n.setdefault(insts[i].n, []).append(t)
                cpu_s = sum(len(by_n[n]) * sum(v) / len(v) for n, v in per_n.items())
                est.append(cpu_s / cores)
    whole_s = sum(est) / len(est)
    evals_s = len(insts) / whole_s
    per_step = sum(t_steps) / len(t_steps)
    desc = (f"2 instances of each size n = 8..20 per step ({len(sample)} of 4096); per-size CPU time x "
            f"the workload's size counts / {cores} cores")
    line = {"impl": "reference", "metric": METRIC, "value": evals_s, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "batched_vqe_4096 (8-20 qubits, depth 2-8, 50-500 Pauli terms)",
                       "parallelism": f"{cores} single-threaded host processes",
                       "whole_workload_s_estimate": whole_s},
            "cpu_baseline": {"value": evals_s, "unit": "evals/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": evals_s, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


_REF_CACHE = {}


def _ref_worker_init():
    # one BLAS thread per process: the pool already uses every core
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"


def _ref_one(arg):
    """CPU seconds of one instance's energy + adjoint gradient (oracle port)."""
    (i,) = arg
    from oracle import sv
    from tyxonq_gb300.workloads import batched_vqe

    if "insts" not in _REF_CACHE:
        _REF_CACHE["insts"] = batched_vqe(4096, seed=3)
    inst = _REF_CACHE["insts"][i]
    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()]
    t0 = time.perf_counter()
    sv.grad_adjoint(inst.n, gates, inst.theta, inst.H.codes, inst.H.coeffs)
    return time.perf_counter() - t0


# ------------------------------------------------------------------ our arm
def _print_scaled_line(args, rank, world, value, ms, e2e, h2d, d2h, bv, insts, build_s, clk, waves_prof, l2_gbs):
    """The report line of a multi-rank run (rank 0 prints): the headline over all
    ranks (max step time over ranks), its e2e, the wave-phase roofline of rank 0;
    the single-GPU sections (plain engine, gate kernels, small configurations,
    serving, CPU baseline) belong to the one-GPU run."""
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": args.scaling,
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
        "config": {"workload": f"batched_vqe_{len(insts)} per rank" if args.scaling == "weak" else
                   f"batched_vqe_{args.count} split over {world} ranks by estimated cost",
                   "l2": "512 MiB buffer written between timed steps", "graph": "CUDA graph replay",
                   "parallelism": f"{world} ranks, one GPU each, no data-path collective",
                   "build_s": build_s, "schedule": _schedule_fields(bv.sched)},
        "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": "tq_jit_wave_adjoint (rank 0)", "bound": "l2",
                     "achieved": waves_prof["adjoint"]["gbs"] if "adjoint" in waves_prof else None,
                     "peak": l2_gbs, "unit": "GB/s",
                     "frac": waves_prof["adjoint"]["frac_of_l2_copy"] if "adjoint" in waves_prof else None,
                     "traffic": WAVE_ADJ_DRAM_BYTES_PER_ITEM, "peak_kind": "measured in this run: L2-resident copy"},
        "cpu_baseline": None,
        "clocks": clk.summary(),
        "gpu_launches": bv.kernel_launches() * args.steps,
    }
    print(json.dumps(line), flush=True)


def _schedule_fields(sched) -> dict:
    """The complex64 batched schedule's fields and where they came from (the
    autotuned file for this GPU, or the builtin defaults)."""
    from dataclasses import asdict

    import torch

    from tyxonq_gb300.autotune import SCHEDULE_FIELDS, load_schedule, schedule_path

    out = {k: v for k, v in asdict(sched).items() if k in SCHEDULE_FIELDS}
    try:
        out["source"] = str(schedule_path().name) if load_schedule(torch.complex64) else "builtin"
    except (OSError, ValueError, RuntimeError) as e:  # the report line must not fail on this field
        out["source"] = f"unknown ({type(e).__name__})"
    return out


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_gate_kernels(args, dev):
    """28 qubits, depth 40 random circuit, complex64: fused tile passes with the
    interpreting kernel (per-launch events) and with the circuit-specialised
    kernels (events around the whole program), the one-launch-per-gate engine,
    full probabilities and 8192 shots."""
    import ctypes

    import torch

    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.engine import execute_plain
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward
    from tyxonq_gb300.workloads import random_circuit

    class _C:
        def __init__(self, n, ops):
            self.num_qubits, self.ops = n, ops

    n2 = 28
    N, S = 1 << n2, 8
    gates, _ = lower_ops(_C(n2, random_circuit(n2, 40, seed=1)), mode="run")
    prog = compile_forward(gates, n2, torch.complex64)
    psi = K.init_statevector(n2, dtype=torch.complex64)
    st = torch.cuda.current_stream()
    for _ in range(2):
        prog.run(psi)
    torch.cuda.synchronize()
    launch_ms, step_ms = [], []
    for _ in range(2):
        a, b = _events()
        a.record(st)
        evs = []
        for kind, obj in prog.segments:
            for p in range(obj.n_passes):
                x, y = _events()
                x.record(st)
                if kind == "staged":
                    st_d, ops_d = obj.device_tables(psi.device)
                    nat.call("tq_sv_run_staged", ctypes.c_void_p(psi.data_ptr()), n2, 0,
                             ctypes.byref(obj.passes[p]), 1, ctypes.c_void_p(st_d.data_ptr()),
                             ctypes.c_void_p(ops_d.data_ptr()), None, K.stream_ptr())
                else:
                    ops_d = obj.device_ops(psi.device)
                    nat.call("tq_sv_run_tiles", ctypes.c_void_p(psi.data_ptr()), n2, 0, ctypes.byref(obj.passes[p]),
                             1, ctypes.c_void_p(ops_d.data_ptr()), None, K.stream_ptr())
                y.record(st)
                evs.append((x, y))
        b.record(st)
        torch.cuda.synchronize()
        step_ms.append(a.elapsed_time(b))
        launch_ms += [x.elapsed_time(y) for x, y in evs]
    avg_launch = sum(launch_ms) / len(launch_ms)
    # circuit-specialised kernels (compiled at run time, cached per structure): tile widths
    # 12-14 with 4- or 5-bit register stages, the fastest reported
    t0 = time.perf_counter()
    tile_ms = {}
    best = None
    for tw, rb in ((12, 4), (12, 5), (13, 4), (13, 5), (14, 5)):
        pr = compile_forward(gates, n2, torch.complex64, t=tw, staged=True)
        n_spec = pr.specialise(torch.complex64, stage_bits=rb)
        if n_spec != pr.n_passes:
            continue
        for _ in range(2):
            pr.run(psi)
        torch.cuda.synchronize()
        spec_ms = []
        for _ in range(3):
            a, b = _events()
            a.record(st)
            pr.run(psi)
            b.record(st)
            torch.cuda.synchronize()
            spec_ms.append(a.elapsed_time(b))
        tile_ms[f"t{tw}_s{rb}"] = {"ms": sum(spec_ms) / len(spec_ms), "passes": pr.n_passes}
        if best is None or tile_ms[f"t{tw}_s{rb}"]["ms"] < tile_ms[best[0]]["ms"]:
            best = (f"t{tw}_s{rb}", pr)
        else:
            del pr
    spec_build_s = time.perf_counter() - t0
    if best is None:  # no combination compiled: report the interpreting kernel's passes
        prog = compile_forward(gates, n2, torch.complex64, t=13, staged=True)
        a, b = _events()
        a.record(st)
        prog.run(psi)
        b.record(st)
        torch.cuda.synchronize()
        best = ("t13_interpreter", prog)
        tile_ms["t13_interpreter"] = {"ms": a.elapsed_time(b), "passes": prog.n_passes}
    best_t, prog = best
    spec_total = tile_ms[best_t]["ms"]
    spec_pass = spec_total / prog.n_passes
    # full probabilities (float32) and 8192 shots of the final state
    probs = K.probabilities(psi)
    K.sample(psi, 8192, seed=1)
    torch.cuda.synchronize()
    prob_ms, shot_ms = [], []
    for r in range(3):
        a, b = _events()
        a.record(st)
        K.probabilities(psi, out=probs)
        b.record(st)
        c, d = _events()
        c.record(st)
        K.sample(psi, 8192, seed=2 + r)
        d.record(st)
        torch.cuda.synchronize()
        prob_ms.append(a.elapsed_time(b))
        shot_ms.append(c.elapsed_time(d))
    del probs
    psi2 = K.init_statevector(n2, dtype=torch.complex64)
    execute_plain(psi2, gates[:40])
    torch.cuda.synchronize()
    a, b = _events()
    a.record()
    execute_plain(psi2, gates)
    b.record()
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b)
    del psi, psi2
    torch.cuda.empty_cache()
    pm, sm = sum(prob_ms) / len(prob_ms), sum(shot_ms) / len(shot_ms)
    return {"fused_ms": spec_total, "fused_interpreter_ms": sum(step_ms) / len(step_ms), "plain_ms": plain_ms,
            "passes": prog.n_passes, "gates": len(gates), "pass_alg_bytes": 2 * N * S,
            "avg_pass_ms": spec_pass, "pass_gbs": 2 * N * S / (spec_pass * 1e-3) / 1e9,
            "specialised_passes": prog.n_passes, "specialise_s": spec_build_s, "tile_bits": best_t,
            "tile_sweep": tile_ms,
            "interpreter_avg_pass_ms": avg_launch,
            "interpreter_pass_gbs": 2 * N * S / (avg_launch * 1e-3) / 1e9,
            "probabilities": {"ms": pm, "alg_bytes": N * (S + 4), "gbs": N * (S + 4) / (pm * 1e-3) / 1e9},
            "shots_8192": {"ms": sm, "alg_bytes": N * S, "gbs": N * S / (sm * 1e-3) / 1e9},
            "single_gate": bench_single_gates(n2)}


def bench_fused_28q(args) -> dict:
    """The 28-qubit depth-40 random circuit (complex64) through the
    circuit-specialised fused passes only: warm-up runs, then timed runs."""
    import torch

    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.ir import lower_ops
    from tyxonq_gb300.program import compile_forward
    from tyxonq_gb300.workloads import random_circuit

    class _C:
        def __init__(self, n, ops):
            self.num_qubits, self.ops = n, ops

    n2 = 28
    gates, _ = lower_ops(_C(n2, random_circuit(n2, 40, seed=1)), mode="run")
    prog = compile_forward(gates, n2, torch.complex64, t=args.tile_bits, staged=True)
    prog.specialise(torch.complex64)
    psi = K.init_statevector(n2, dtype=torch.complex64)
    for _ in range(args.warmup):
        prog.run(psi)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        a, b = _events()
        a.record()
        prog.run(psi)
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    m = sum(ms) / len(ms)
    return {"passes": prog.n_passes, "ms": m, "pass_ms": m / prog.n_passes,
            "pass_gbs": 2 * (1 << n2) * 8 / (m / prog.n_passes * 1e-3) / 1e9}


def measure_l2_copy_gbs(mib: int = 24, reps: int = 50) -> float:
    """Bandwidth of a copy whose source and destination stay in L2 together
    (2 x `mib` MiB < 126 MiB): read + write bytes / device time, best of 3."""
    import torch

    a = torch.empty(mib << 20, dtype=torch.uint8, device="cuda").fill_(1)
    b = torch.empty_like(a)
    for _ in range(5):
        b.copy_(a)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        x, y = _events()
        x.record()
        for _ in range(reps):
            b.copy_(a)
        y.record()
        torch.cuda.synchronize()
        best = max(best, 2 * a.numel() * reps / (x.elapsed_time(y) * 1e-3) / 1e9)
    del a, b
    return best


def bench_serving(args) -> list:
    """Serving sweep: for each arrival rate, a Poisson trace of
    args.serving_requests requests (sessions of two optimizer steps, HEA
    n ~ U{10..26}, depth ~ U{2..10}, 20-1000 Pauli terms, 30% energy+gradient,
    complex64) replayed in real time; p50 / p99 latency and served throughput."""
    import torch

    from tyxonq_gb300.serving import VqeServer, make_trace, replay

    serving = []
    # warm-up trace (not reported): first use of every kernel and of the per-request streams
    warm = make_trace(16, rate=80.0, seed=99, n_range=(10, 26), depth_range=(2, 10), terms_range=(20, 1000),
                      grad_fraction=0.5, iterations=2)
    replay(VqeServer(max_inflight=8), warm)
    torch.cuda.empty_cache()
    for rate in args.serving_rates:
        trace = make_trace(args.serving_requests, rate=rate, seed=int(rate), n_range=(10, 26), depth_range=(2, 10),
                           terms_range=(20, 1000), grad_fraction=0.3, iterations=2)
        srv = VqeServer(max_inflight=8)
        st = replay(srv, trace)
        st["rate_rps"] = rate
        serving.append(st)
        del srv
        torch.cuda.empty_cache()
    return serving


def bench_small_configs(reps: int = 10) -> dict:
    """Per-call times, host parameters in and host results out, of
    * the 12-qubit HEA (4 layers of [RY on every qubit; CX ladder]) with the
      open-chain TFIM (23 terms): complex128 energy + adjoint gradient, and
      4096 Z-basis shots (forward, sampling, counts dictionary);
    * the 16-qubit UCCSD from the Hartree-Fock bitstring (8 orbitals, 4
      electrons, 198 excitations, Jordan-Wigner H of seeded random integrals):
      adjoint energy + gradient with the excitations as 1440 Pauli-string
      exponentials (fused-pass engine) and as exact pair rotations, each in
      complex128 and complex64, and the FP64 CI-space engine."""
    import numpy as np
    import torch

    from tyxonq_gb300 import chem
    from tyxonq_gb300 import kernels as K
    from tyxonq_gb300.adjoint import ParamGate, ParametricEstimator
    from tyxonq_gb300.ir import Gate, _rot_gate
    from tyxonq_gb300.vqe import UCCSD
    from tyxonq_gb300.workloads import hea_tfim

    def per_call_ms(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps

    _, H12, th12 = hea_tfim(12, 4, seed=0)
    pg = []
    for l in range(4):
        pg += [ParamGate(_rot_gate("ry", (q,), 0.0), l * 12 + q) for q in range(12)]
        pg += [ParamGate(Gate("cx", (q, q + 1))) for q in range(11)]
    est = ParametricEstimator(12, pg, 48, H12, dtype=torch.complex128)
    theta = th12.reshape(-1)

    def shots():
        psi = est._forward(theta)
        return K.counts_from_indices(K.sample(psi, 4096, seed=11).cpu().numpy(), 12)

    out = {"hea12_tfim": {"energy": est.energy(theta),
                          "energy_grad_ms": per_call_ms(lambda: est.energy_and_grad(theta)),
                          "energy_ms": per_call_ms(lambda: est.energy(theta)),
                          "shots4096_ms": per_call_ms(shots), "dtype": "c128"}}
    # the same circuit through the drop-in chain API (the engine the plug-in installs):
    # c.compile().device(provider="simulator", device="statevector").run(shots=4096) and
    # c.state(), host results, per call; default complex64 and the complex128 option
    from tyxonq_gb300.circuit import Circuit

    chain = {}
    for dname in ("complex64", "complex128"):
        c = Circuit(12)
        for l in range(4):
            for q in range(12):
                c.ry(q, theta=float(th12[l, q]))
            for q in range(11):
                c.cx(q, q + 1)
        run = lambda: c.compile().device(provider="simulator", device="statevector", dtype=dname).run(shots=4096)
        st = lambda: c.state(dtype=dname, form="numpy")
        chain[dname] = {"run_shots4096_ms": per_call_ms(run), "state_ms": per_call_ms(st)}
    out["hea12_chain_api"] = chain
    h, g = chem.random_integrals(8, seed=7)
    ucc = {}
    for name, kw in (("c128_rotations", {"dtype": torch.complex128, "trotter": True}),
                     ("c64_rotations", {"dtype": torch.complex64, "trotter": True}),
                     ("c128_excitations", {"dtype": torch.complex128}),
                     ("c64_excitations", {"dtype": torch.complex64}),
                     ("civector_f64", {"engine": "civector"})):
        m = UCCSD(h, g, n_elec=4, **kw)
        p = np.random.default_rng(2).uniform(-0.3, 0.3, m.n_params)
        ucc[name] = {"energy_grad_ms": per_call_ms(lambda: m.energy_and_grad(p)), "energy": m.energy(p)}
        ucc["terms"], ucc["params"], ucc["rotations"] = len(m.hamiltonian.coeffs), m.n_params, len(m.param_gates)
        del m
    out["uccsd16"] = ucc
    torch.cuda.empty_cache()
    return out


def bench_single_gates(n: int, reps: int = 4) -> dict:
    """One launch per gate on an n-qubit complex64 state (2 GiB at 28 qubits, far
    above L2): device time per launch and GB/s over the algorithmic bytes of the
    gate (amplitudes it can change, read and written once), and over the bytes
    of the 32-byte DRAM sectors that hold such amplitudes (the least traffic a
    gate on the lowest index bits can cause)."""
    import ctypes

    import numpy as np
    import torch

    from tyxonq_gb300 import _native as nat
    from tyxonq_gb300 import kernels as K

    N, S = 1 << n, 8
    psi = K.init_statevector(n, dtype=torch.complex64)
    P = ctypes.c_void_p(psi.data_ptr())
    st = K.stream_ptr()
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    u2 = np.linalg.qr(np.random.default_rng(5).normal(size=(4, 4)) + 1j)[0]
    qs = [0, n // 4, n // 2, 3 * n // 4, n - 1]
    d_rz = (ctypes.c_double * 4)(np.cos(0.3), -np.sin(0.3), np.cos(0.3), np.sin(0.3))
    d_ph = (ctypes.c_double * 4)(1.0, 0.0, np.cos(0.7), np.sin(0.7))
    mh, m2 = K._mat(h, 2), K._mat(u2, 4)
    def sector_frac(*bits):
        # share of 32-byte sectors (4 complex64 amplitudes: index bits 0-1) that hold an
        # amplitude the gate changes, when the changed amplitudes are those with all `bits` set
        f = 1.0
        for b in bits:
            f *= 1.0 if b < 2 else 0.5
        return f

    kinds = {
        "dense_1q": (2 * N * S, lambda q, r: 1.0, lambda q, r: nat.call("tq_sv_apply_1q", P, n, 0, q, mh, st)),
        "diag_1q": (2 * N * S, lambda q, r: 1.0, lambda q, r: nat.call("tq_sv_apply_diag1", P, n, 0, q, d_rz, st)),
        "phase_1q": (N * S, lambda q, r: sector_frac(n - 1 - q),
                     lambda q, r: nat.call("tq_sv_apply_diag1", P, n, 0, q, d_ph, st)),
        "cx": (N * S, lambda q, r: sector_frac(n - 1 - q), lambda q, r: nat.call("tq_sv_apply_cx", P, n, 0, q, r, st)),
        "cz": (N * S // 2, lambda q, r: sector_frac(n - 1 - q, n - 1 - r),
               lambda q, r: nat.call("tq_sv_apply_cz", P, n, 0, q, r, st)),
        "dense_2q": (2 * N * S, lambda q, r: 1.0, lambda q, r: nat.call("tq_sv_apply_2q", P, n, 0, q, r, m2, st)),
    }
    out = {}
    for name, (alg, frac, fn) in kinds.items():
        pairs = [(q, qs[(i + 2) % len(qs)]) for i, q in enumerate(qs)]
        for q, r in pairs:  # warm-up
            fn(q, r)
        torch.cuda.synchronize()
        times, sector_bytes = [], []
        for _ in range(reps):
            for q, r in pairs:
                a, b = _events()
                a.record()
                fn(q, r)
                b.record()
                torch.cuda.synchronize()
                times.append(a.elapsed_time(b))
                sector_bytes.append(2 * N * S * frac(q, r))
        ms = sum(times) / len(times)
        out[name] = {"ms": ms, "alg_bytes": alg, "gbs": alg / (ms * 1e-3) / 1e9, "launches": len(times),
                     "sector_bytes": sum(sector_bytes) / len(sector_bytes),
                     "sector_gbs": sum(sector_bytes) / (sum(times) * 1e-3) / 1e9,
                     "qubit_pairs": pairs}
    # dense k-qubit unitaries (k = 3..5) on spread qubits: 2^k complex MACs (8 * 2^k flops) per
    # amplitude on the FP32 cores; GB/s over the read+write of every amplitude
    rng = np.random.default_rng(9)
    for k in (3, 4, 5):
        d = 1 << k
        uk = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]
        mk, qk = K._mat(uk, d), nat.int_array(qs[:k])
        for _ in range(2):
            nat.call("tq_sv_apply_kq", P, n, 0, qk, k, mk, st)
        torch.cuda.synchronize()
        times = []
        for _ in range(reps):
            a, b = _events()
            a.record()
            nat.call("tq_sv_apply_kq", P, n, 0, qk, k, mk, st)
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        ms = sum(times) / len(times)
        out[f"dense_{k}q"] = {"ms": ms, "alg_bytes": 2 * N * S, "gbs": 2 * N * S / (ms * 1e-3) / 1e9,
                              "tflops": 8 * d * N / (ms * 1e-3) / 1e12, "launches": len(times),
                              "qubits": qs[:k]}
    del psi
    torch.cuda.empty_cache()
    return out


def run_case(args):
    """One part of the benchmark alone (used for profiler captures)."""
    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.build()
    torch.cuda.set_device(0)
    if args.case == "gates":
        print(json.dumps({"case": "gates", **bench_gate_kernels(args, 0)}))
        return
    if args.case == "small":
        print(json.dumps({"case": "small", **bench_small_configs()}))
        return
    if args.case == "fused":
        print(json.dumps({"case": "fused", **bench_fused_28q(args)}))
        return
    if args.case == "serving":
        print(json.dumps({"case": "serving", "sweep": bench_serving(args)}))
        return
    if args.case == "civector":
        from tyxonq_gb300 import chem
        from tyxonq_gb300.vqe import UCCSD

        h, g = chem.random_integrals(8, seed=7)
        m = UCCSD(h, g, n_elec=4, engine="civector")
        p = np.random.default_rng(2).uniform(-0.3, 0.3, m.n_params)
        for _ in range(args.warmup + args.steps):
            e, _ = m.energy_and_grad(p)
        print(json.dumps({"case": "civector", "D": m._est.D, "energy": e}))
        return
    from tyxonq_gb300.batch import BatchedVQE
    from tyxonq_gb300.workloads import batched_vqe

    insts = batched_vqe(args.count, seed=3)
    bv = BatchedVQE(insts, dtype=torch.complex64)
    bv.set_theta(np.concatenate([i.theta for i in insts]))
    for _ in range(args.warmup):
        bv.run()
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        a, b = _events()
        a.record()
        bv.run()
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    print(json.dumps({"case": "batched", "count": len(insts), "ms_per_step": sum(ms) / len(ms)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--tile-bits", type=int, default=13, help="--case fused: local qubits per pass")
    ap.add_argument("--serving-requests", type=int, default=1000, help="requests per arrival rate")
    ap.add_argument("--serving-rates", type=float, nargs="+", default=[25.0, 50.0, 100.0, 200.0])
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: every rank evaluates its own --count instances; strong: one --count workload "
                         "split over the ranks by estimated cost")
    ap.add_argument("--case", default="full",
                    choices=["full", "gates", "fused", "batched", "small", "civector", "serving"],
                    help="gates / fused (28-qubit circuit, specialised passes only) / batched / small / civector "
                         "(16-qubit UCCSD in CI space): run only that part "
                         "(profiling captures); full: the benchmark line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.case != "full":
        return run_case(args)

    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.build()
    from tyxonq_gb300.batch import BatchedVQE
    from tyxonq_gb300.workloads import batched_vqe

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    # ---------------- batched workload: weak scaling = every rank evaluates its own 4096 instances;
    # strong scaling = one 4096-instance workload split over the ranks by estimated cost
    if args.scaling == "strong":
        from tyxonq_gb300.distributed import shard_instances

        insts_all = batched_vqe(args.count, seed=3)
        insts = [insts_all[i] for i in shard_instances(insts_all, rank, world)]
        job_count = len(insts_all)
    else:
        insts = batched_vqe(args.count, seed=3 + 1000 * rank)
        job_count = world * len(insts)
    t0 = time.perf_counter()
    bv = BatchedVQE(insts, dtype=torch.complex64)
    build_s = time.perf_counter() - t0
    theta_host = torch.from_numpy(np.concatenate([i.theta for i in insts])).pin_memory()
    bv.set_theta(theta_host)
    bv.capture()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")  # > L2 (129 MB)
    for _ in range(args.warmup):
        bv.run()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a, b = _events()
            a.record()
            bv.run()
            b.record()
            torch.cuda.synchronize()
            step_ms.append(a.elapsed_time(b))
    if world > 1:
        dist.barrier()
    ms = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = job_count / (ms * 1e-3)

    # ---------------- per-phase device time of the wave kernels (one evaluation, serialised on
    # one stream, CUDA events around every launch) against the measured L2 copy bandwidth
    # (these per-GPU figures and the sections below them are taken on one GPU only: with
    # several ranks the line reports the scaled headline and its e2e)
    waves_prof = bv.profile_waves()
    torch.cuda.synchronize()
    l2_gbs = measure_l2_copy_gbs()
    for ph in waves_prof.values():
        ph["gbs"] = ph["alg_bytes"] / (ph["ms"] * 1e-3) / 1e9
        ph["frac_of_l2_copy"] = ph["gbs"] / l2_gbs
        ph["avg_launch_ms"] = ph["ms"] / ph["launches"]

    # ---------------- e2e: host theta -> device, evaluate, energies + gradients -> host
    e_host = torch.empty(bv.count, dtype=torch.float64).pin_memory()
    g_host = torch.empty(bv.grads.numel(), dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        a, b = _events()
        a.record()
        bv.run(theta_host)
        e_host.copy_(bv.energies, non_blocking=True)
        g_host.copy_(bv.grads, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        e2e_ms.append(a.elapsed_time(b))
    e2e_local = sum(e2e_ms) / len(e2e_ms)
    if world > 1:
        t = torch.tensor([e2e_local], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_local = float(t.item())
    e2e = job_count / (e2e_local * 1e-3)
    h2d = theta_host.numel() * 8
    d2h = (e_host.numel() + g_host.numel()) * 8
    energies = e_host.numpy().copy()

    if world > 1:
        _print_scaled_line(args, rank, world, value, ms, e2e, h2d, d2h, bv, insts, build_s, clk, waves_prof,
                           l2_gbs)
        return

    # ---------------- plain single-circuit engine on an every-16th-instance sample: one launch per
    # gate, each instance's evaluation captured once as a CUDA graph and replayed (GPU-bound)
    from tyxonq_gb300.batch import PlainEngine

    sample = list(range(0, len(insts), 16))
    engines = []
    for i in sample:
        eng = PlainEngine(insts[i])
        eng.capture()
        engines.append(eng)
    for eng in engines:
        eng.run()
    torch.cuda.synchronize()
    a, b = _events()
    a.record()
    for eng in engines:
        eng.run()
    b.record()
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b)
    plain_evals = len(sample) / (plain_ms * 1e-3)
    worst = 0.0
    for i, eng in zip(sample, engines):
        e_p, _ = eng.result()
        worst = max(worst, abs(e_p - energies[i]))
    del engines
    torch.cuda.empty_cache()

    # ---------------- 28q gate kernels (memory-bound case) + roofline
    gk = bench_gate_kernels(args, dev)
    peak, peak_kind = _peaks()
    small = bench_small_configs()

    # ---------------- serving: Poisson arrivals, 70% energy / 30% energy+gradient, 10-26 qubits
    serving = bench_serving(args)

    # ---------------- CPU baseline: oracle port, one instance of every size, one core
    cpu = None
    if rank == 0:
        from oracle import sv

        by_n: dict = {}
        for i, inst in enumerate(insts):
            by_n.setdefault(inst.n, []).append(i)
        cpu_s = 0.0
        for n in sorted(by_n):
            inst = insts[by_n[n][0]]
            t0 = time.perf_counter()
            sv.grad_adjoint(inst.n, [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()], inst.theta,
                            inst.H.codes, inst.H.coeffs)
            cpu_s += len(by_n[n]) * (time.perf_counter() - t0)
        cpu = {"value": len(insts) / cpu_s, "unit": "evals/s", "cores": 1, "kind": "port",
               "sample": f"one instance of each size n = {min(by_n)}..{max(by_n)} (energy + adjoint gradient, "
                         "complex128), its time weighted by the workload's count of that size"}

    launches_per_step = bv.kernel_launches()
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": args.scaling,
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
        "config": {"workload": f"batched_vqe_{len(insts)}: n~U{{8..20}}, HEA depth~U{{2..8}} [RY;RZ;CX ladder], "
                               "50-500 random Pauli terms (weight 1-4, N(0,1)), energy + adjoint gradient",
                   "l2": "512 MiB buffer written between timed steps", "graph": "CUDA graph replay",
                   "classes": {c.name: len(c.work) for c in bv.launch_order}, "structures": bv.n_structures,
                   "build_s": build_s, "schedule": _schedule_fields(bv.sched)},
        "plain_gpu": {"value": plain_evals, "unit": "evals/s",
                      "sample": f"{len(sample)} of {len(insts)} (every 16th), each evaluation a replayed CUDA graph "
                                "of one launch per gate",
                      "speedup_batched": value / world / plain_evals, "max_energy_diff_abs": worst},
        "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "latency": {"p50_ms": serving[0]["p50_ms"], "p99_ms": serving[0]["p99_ms"],
                    "at_rate_rps": serving[0]["rate_rps"], "sweep": serving,
                    "workload": f"Poisson arrivals, {args.serving_requests // 2} sessions x 2 optimizer steps per "
                                "rate, HEA n~U{10..26} depth~U{2..10}, 20-1000 Pauli terms, 30% energy+gradient, "
                                "complex64"},
        "gate_kernels_28q": gk,
        "small_configs": small,
        "roofline": {"kernel": "tq_jit_wave_adjoint (circuit-specialised adjoint pass of the L2-resident waves, "
                               "the largest share of the batched step; 4 * 2^12 * 8 B per item: psi and lam tiles "
                               "read and written once)",
                     "bound": "l2", "achieved": waves_prof["adjoint"]["gbs"], "peak": l2_gbs, "unit": "GB/s",
                     "frac": waves_prof["adjoint"]["frac_of_l2_copy"], "traffic": WAVE_ADJ_DRAM_BYTES_PER_ITEM,
                     "traffic_unit": "DRAM bytes per item (ncu)",
                     "peak_kind": "measured in this run: L2-resident copy (2 x 24 MiB)",
                     "issue_active": WAVE_ADJ_ISSUE_ACTIVE,
                     "issue_note": "smsp__issue_active of the same kernel from ncu: the pass is bound by "
                                   "instruction issue and latency on L2-resident tiles, not by L2 bandwidth"},
        "roofline_c2": {"kernel": "tq_jit_staged_pass (circuit-specialised fused pass of the 28-qubit complex64 "
                                  "depth-40 random circuit, 2*N*8 B per launch)", "bound": "hbm",
                        "achieved": gk["pass_gbs"], "peak": peak, "unit": "GB/s", "frac": gk["pass_gbs"] / peak,
                        "traffic": STAGED_PASS_DRAM_BYTES, "peak_kind": peak_kind},
        "wave_kernels": {"phases": waves_prof, "l2_copy_gbs": l2_gbs},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches_per_step * args.steps,
    }
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
