"""Benchmark: the 30-qubit random circuit (Haar 1q on every qubit,
controlledPhaseShift on a random perfect matching, CNOT brickwork; 20 layers)
through the GB300 library, plus the QuEST-CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = the whole circuit once (initZeroState, all gates, calcTotalProb)
on one register.  `value` is the per-gate FP64 algorithmic throughput: the
bytes a per-gate FP64 simulator must stream for this circuit (1q gate
2*2^n*16 B, CNOT 2^n*16 B, CPhase 2^(n-1)*16 B; 28.2 TB at 30 qubits, 20
layers) divided by the time per circuit.  The same definition is used for
every engine and for the CPU reference, so ratios are time-to-solution
ratios.  The state (16 GiB FP64) is far larger than L2, so no L2 flush is
needed between steps.

Prints ONE JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fused-FP32 vs plain-FP64 gate GB/s at 30q (1-F≤1e-6); batched swap tests/s"
FALLBACK_HBM = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except OSError:
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def barrier_max(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world == 1:
        return
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    dist.barrier()


# ----------------------------------------------------------------- GB300 arm
def run_gpu(args, rank, world):
    import quantumlab_gb300 as qg
    from quantumlab_gb300 import workloads as W
    from quantumlab_gb300.quest import Complex

    L = qg.load()
    lib = L.lib
    n = args.qubits
    ops = W.c2_circuit(n=n, layers=args.layers, seed=2)
    alg_bytes = W.algorithmic_bytes(ops, n)
    q = L.create(n)

    def step(time_kernels=False, slot_base=100):
        lib.initZeroState(q)
        k = 0
        for op in ops:
            kind = op[0]
            if kind == "cu":
                if time_kernels:
                    lib.quest_gb300_eventRecord(slot_base + 2 * k)
                lib.compactUnitary(q, op[1], Complex(op[2], op[3]), Complex(op[4], op[5]))
                if time_kernels:
                    lib.quest_gb300_eventRecord(slot_base + 2 * k + 1)
                k += 1
            elif kind == "cx":
                lib.controlledNot(q, op[1], op[2])
            else:
                lib.controlledPhaseShift(q, op[1], op[2], op[3])
        total = lib.calcTotalProb(q)
        kern = []
        if time_kernels:
            kern = [lib.quest_gb300_eventElapsedMs(slot_base + 2 * i, slot_base + 2 * i + 1) for i in range(k)]
        return total, kern

    for _ in range(args.warmup):
        step()
    barrier(world)
    launches0 = lib.quest_gb300_launchCount()
    kern_ms = []
    with Clocks(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        lib.quest_gb300_eventRecord(0)
        t0 = time.perf_counter()
        for s in range(args.steps):
            total, kern = step(time_kernels=True)
            kern_ms += kern
        lib.quest_gb300_eventRecord(1)
        ms = lib.quest_gb300_eventElapsedMs(0, 1)
        wall = time.perf_counter() - t0
    launches = lib.quest_gb300_launchCount() - launches0
    ms_step = barrier_max(ms / args.steps, world)
    value = world * alg_bytes / (ms_step / 1e3) / 1e9

    # end to end through the C ABI with host buffers: the pinned host mirror
    # holds |0..0>; each step copies it in, runs the circuit, reads the total
    # probability and copies the whole state back (QLSimulatorVector pattern)
    lib.initZeroState(q)
    lib.copyStateFromGPU(q)
    e2e_steps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        lib.copyStateToGPU(q)
        for op in ops:
            kind = op[0]
            if kind == "cu":
                lib.compactUnitary(q, op[1], Complex(op[2], op[3]), Complex(op[4], op[5]))
            elif kind == "cx":
                lib.controlledNot(q, op[1], op[2])
            else:
                lib.controlledPhaseShift(q, op[1], op[2], op[3])
        lib.calcTotalProb(q)
        lib.copyStateFromGPU(q)
    e2e_s = barrier_max((time.perf_counter() - t0) / e2e_steps, world)
    state_bytes = (1 << n) * 16
    L.destroy(q)

    peak, peak_kind = peaks()
    one_q_bytes = 2 * (1 << n) * 16
    avg_kernel_ms = statistics.mean(kern_ms) if kern_ms else float("nan")
    achieved = one_q_bytes / (avg_kernel_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        t = json.load(open(tp)).get("plain_compactUnitary_per_amp_bytes")
        if t:
            traffic = t * (1 << n)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Haar/CPhase-matching/CNOT-brickwork circuit)",
        "config": {"workload": f"{n}-qubit random circuit, {args.layers} layers, plain FP64 per-gate engine",
                   "qubits": n, "layers": args.layers, "gates_per_circuit": len(ops),
                   "algorithmic_bytes_per_circuit": alg_bytes, "engine": "plain-fp64",
                   "l2": "state 16 GiB >> 129 MB L2, no flush needed", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "kernel": "compactUnitary (kPairVec<OpCompact>)",
                     "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "avg_launch_ms": round(avg_kernel_ms, 4), "launches_timed": len(kern_ms)},
        "e2e": {"value": round(world * alg_bytes / e2e_s / 1e9, 2), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
                "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes + 16},
        "gpu_launches": int(launches),
        "total_prob": total,
        "wall_s": round(wall, 3),
    }
    clk_sum = clk.summary()
    if clk_sum:
        out["clocks"] = clk_sum
    return out


# --------------------------------------------------------- CPU (QuEST) side
def cpu_library():
    """The reference's own QuEST CPU build when it is built for this host,
    else the oracle port (both export the same C ABI)."""
    from quantumlab_gb300.quest import QuESTLibrary
    ref = os.path.join(ROOT, "oracle", "_ref", "libquest_ref.so")
    if os.path.exists(ref):
        try:
            return QuESTLibrary(ref), "reference"
        except OSError:
            pass
    port = os.path.join(ROOT, "oracle", "_build", "libquest_oracle.so")
    if not os.path.exists(port):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return QuESTLibrary(port), "port"


def cpu_sample(n, layers, sample_ops, repeats=1):
    """Time the first `sample_ops` gates of the circuit on the CPU library at
    full size; returns (GB/s, seconds, kind, ops_timed)."""
    from quantumlab_gb300 import workloads as W
    L, kind = cpu_library()
    ops = W.c2_circuit(n=n, layers=layers, seed=2)[:sample_ops]
    q = L.create(n)
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        W.run_ops(L, q, ops)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    L.destroy(q)
    return W.algorithmic_bytes(ops, n) / best / 1e9, best, kind, len(ops)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    n = args.qubits
    sample_ops = args.cpu_sample_ops
    vals = []
    kind = "port"
    for i in range(args.warmup + args.steps):
        gbs, dt, kind, nops = cpu_sample(n, args.layers, sample_ops)
        if i >= args.warmup:
            vals.append((gbs, dt))
    value = statistics.median(v for v, _ in vals)
    ms = statistics.median(d for _, d in vals) * 1e3
    cores = os.cpu_count()
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "GB/s (per-gate FP64 algorithmic bytes)", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Haar/CPhase-matching/CNOT-brickwork circuit)",
        "config": {"workload": f"{n}-qubit random circuit, {args.layers} layers (first {sample_ops} gates per step)",
                   "qubits": n, "layers": args.layers},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s (per-gate FP64 algorithmic bytes)", "cores": cores,
                         "kind": kind, "sample": f"first {sample_ops} gates of the {n}-qubit circuit per step, OpenMP on all host threads"},
        "e2e": {"value": round(value, 3), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--cpu-sample-ops", type=int, default=30)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_info()
    os.environ.setdefault("QUEST_GB300_DEVICE", str(local))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    out = run_gpu(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            gbs, dt, kind, nops = cpu_sample(args.qubits, args.layers, args.cpu_sample_ops)
            out["cpu_baseline"] = {"value": round(gbs, 3), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
                                   "cores": os.cpu_count(), "kind": kind,
                                   "sample": f"first {nops} gates of the {args.qubits}-qubit circuit ({dt:.1f} s), OpenMP on all host threads"}
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
