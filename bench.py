"""Benchmark: the 30-qubit random circuit (Haar 1q on every qubit,
controlledPhaseShift on a random perfect matching, CNOT brickwork; 20 layers)
through the GB300 library, plus the QuEST-CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = the whole circuit once on one register through the fused FP32
engine (initZeroState, every fused pass, FP64 total probability); the plain
FP64 per-gate engine runs the same circuit once for the comparison and the
1 - fidelity check.  `value` is the per-gate FP64 algorithmic throughput: the
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fused-FP32 vs plain-FP64 gate GB/s at 30q (1-F≤1e-6); batched swap tests/s"
FALLBACK_HBM = 6800.0
# operand forms of the pipelined tensor-core kernel (setTensorCorePrecision)
# and their MMA terms per product
PREC_NAMES = {0: "split-TF32", 1: "split-BF16", 2: "split-FP16"}
PREC_TERMS = {0: 3, 1: 4, 2: 3}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region.  The samples go to
    $QUEST_GB300_CLOCKS_DIR (default: the system temporary directory); the
    bench line carries their summary."""

    def __init__(self, index: int = 0):
        import tempfile
        self.index = index
        self.proc = None
        out_dir = os.environ.get("QUEST_GB300_CLOCKS_DIR", tempfile.gettempdir())
        self.path = os.path.join(out_dir, f"quest_gb300_clocks_{os.getpid()}.csv")

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
def run_plain_step(L, q, ops):
    from quantumlab_gb300.quest import Complex
    lib = L.lib
    for op in ops:
        kind = op[0]
        if kind == "cu":
            lib.compactUnitary(q, op[1], Complex(op[2], op[3]), Complex(op[4], op[5]))
        elif kind == "cx":
            lib.controlledNot(q, op[1], op[2])
        else:
            lib.controlledPhaseShift(q, op[1], op[2], op[3])


def link_probe(nbytes: int = 1 << 30):
    """Best of three plain copies of nbytes each way between page-locked host
    memory and the device, in GB/s: the host link as this process sees it."""
    try:
        import torch
        h = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
        d = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
        out = {}
        for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
            best = float("inf")
            for _ in range(3):
                torch.cuda.synchronize()
                t = time.perf_counter()
                dst.copy_(src, non_blocking=True)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t)
            out[name] = round(nbytes / best / 1e9, 1)
        del h, d
        return out
    except Exception as e:   # diagnostics only
        return {"error": str(e)[:120]}


def run_gpu(args, rank, world):
    import ctypes as C
    import quantumlab_gb300 as qg
    from quantumlab_gb300 import workloads as W

    L = qg.load()
    lib = L.lib
    n, k = args.qubits, args.fusion
    ops = W.c2_circuit(n=n, layers=args.layers, seed=2)
    alg_bytes = W.algorithmic_bytes(ops, n)
    pass_bytes = 2 * (1 << n) * 8                   # one fused pass: read + write the FP32 state

    # ---- end to end through the QuEST C ABI with host buffers ------------
    # The lab's call pattern, unchanged: initStateFromAmps from pinned host
    # FP64 arrays, every gate of the circuit as one QuEST API call,
    # calcTotalProb, then copyStateFromGPU of every amplitude into the
    # register's host mirror.  Op-stream capture is on for the register, so
    # the gate calls are queued and applied by the fused FP32 engine at
    # calcTotalProb.  Two untimed warm-up steps (FP32 scratch, plan upload).
    # The end-to-end registers: src (whose pinned host mirror holds the
    # input) and qe (the lab's register).  This runs first, before the
    # other arms load the GPU, as an application that only loops over
    # circuits would run.
    src = L.create(n)
    qe = L.create(n)
    # The input, prepared just before the steps as an application looping
    # over circuits would produce it: a seeded random product state (every
    # amplitude nonzero, no two host pages alike), made on the device and
    # copied into src's pinned mirror.  (Pinned buffers left untouched for a
    # minute were measured copying at a fraction of the link's rate on a
    # virtual machine whose host reclaims idle guest pages.)
    lib.initPlusState(src)
    rng_in = np.random.default_rng(2024)
    from quantumlab_gb300.quest import Complex as _Cx
    for t in range(n):
        v = rng_in.normal(size=4)
        v /= np.linalg.norm(v)
        lib.compactUnitary(src, t, _Cx(v[0], v[1]), _Cx(v[2], v[3]))
    lib.copyStateFromGPU(src)
    lib.quest_gb300_setCapture(qe, 1)

    split = [0.0, 0.0, 0.0]                            # host -> device, gates + flush, device -> host
    d2h_each = []

    def e2e_step():
        t = time.perf_counter()
        lib.initStateFromAmps(qe, src.stateVec.real, src.stateVec.imag)
        t1 = time.perf_counter()
        run_plain_step(L, qe, ops)
        p = lib.calcTotalProb(qe)
        t2 = time.perf_counter()
        lib.copyStateFromGPU(qe)
        t3 = time.perf_counter()
        for i, d in enumerate((t1 - t, t2 - t1, t3 - t2)):
            split[i] += d
        d2h_each.append(round((t3 - t2) * 1e3, 1))
        return p

    for _ in range(2):                                 # untimed warm-up steps
        e2e_step()
    split[:] = [0.0, 0.0, 0.0]
    d2h_each.clear()
    e2e_steps = max(1, min(args.steps, 3))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_prob = e2e_step()
    e2e_s = barrier_max((time.perf_counter() - t0) / e2e_steps, world)
    split = [x / e2e_steps for x in split]
    # the same device->host copy again with nothing in between: whether a slow
    # copy in the steps is the copy itself or the state the step left
    d2h_repeat = []
    for _ in range(3):
        t = time.perf_counter()
        lib.copyStateFromGPU(qe)
        d2h_repeat.append(round((time.perf_counter() - t) * 1e3, 1))
    lib.quest_gb300_setCapture(qe, 0)
    # what the host link gave this process: whether both host mirrors are
    # page-locked, and plain 1 GiB copies between pinned and device memory
    mirrors_pinned = [lib.quest_gb300_hostMirrorPinned(src) == 1, lib.quest_gb300_hostMirrorPinned(qe) == 1]
    link = link_probe()
    state_bytes = (1 << n) * 16
    L.destroy(src)
    L.destroy(qe)

    # ---- fused FP32 engine (the headline) --------------------------------
    prec = {"tf32": 0, "bf16": 1, "fp16": 2}[args.precision]
    pname = PREC_NAMES[prec]
    lib.quest_gb300_setTensorCorePrecision(prec)
    # the autotuner: per-pass costs and the fastest tensor-core variant of
    # every (width, target layout) class, for split-TF32 and split-BF16 (or
    # split-FP16 alone when it is the headline form), then the fusion width
    # with the lowest predicted time
    t0 = time.perf_counter()
    for pr in ((1 - prec, prec) if prec < 2 else (prec,)):
        lib.quest_gb300_setTensorCorePrecision(pr)
        lib.quest_gb300_autotune(n)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    plan = L.plan(n, k, ops)
    tuned_k = lib.quest_gb300_planCompileTuned(plan, min(4, k), k) if not args.no_tune else k
    plan_s = time.perf_counter() - t0
    npass = lib.quest_gb300_planCompile(plan)              # the chosen width's passes (same plan again)
    tc = [lib.quest_gb300_planPassUsesTensorCores(plan, i) for i in range(npass)]
    kk = [lib.quest_gb300_planPass(plan, i, None, None, None) for i in range(npass)]
    ctl = [lib.quest_gb300_planPassControls(plan, i, None) for i in range(npass)]
    q32 = lib.quest_gb300_createQuregF32(n)

    def fused_step():
        lib.quest_gb300_initZeroStateF32(q32)
        lib.quest_gb300_applyPlanF32(q32, plan)
        return lib.quest_gb300_calcTotalProbF32(q32), None

    for _ in range(args.warmup):
        fused_step()
    barrier(world)
    launches0 = lib.quest_gb300_launchCount()
    pass_ms = [0.0] * npass
    pt = (C.c_double * max(1, npass))()
    # each pass's duration from CUDA events the library records around it on
    # its stream, inside the timed steps (no extra host calls between passes)
    lib.quest_gb300_setPassEvents(1)
    with Clocks(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        lib.quest_gb300_eventRecord(0)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            total32, _ = fused_step()                  # ends with a synchronising FP64 reduction
            lib.quest_gb300_passTimesMs(pt, npass)
            pass_ms = [a + pt[i] for i, a in enumerate(pass_ms)]
        lib.quest_gb300_eventRecord(1)
        ms = lib.quest_gb300_eventElapsedMs(0, 1)
        wall = time.perf_counter() - t0
    lib.quest_gb300_setPassEvents(0)
    launches = lib.quest_gb300_launchCount() - launches0
    ms_step = barrier_max(ms / args.steps, world)
    value = world * alg_bytes / (ms_step / 1e3) / 1e9
    pass_ms = [x / args.steps for x in pass_ms]

    # the same plan with the fixed per-width kernel defaults instead of the
    # tuned variants
    lib.quest_gb300_setKernelTuning(0)
    fused_step()
    lib.quest_gb300_eventRecord(8)
    for _ in range(args.steps):
        fused_step()
    lib.quest_gb300_eventRecord(9)
    default_kernels_ms = lib.quest_gb300_eventElapsedMs(8, 9) / args.steps
    lib.quest_gb300_setKernelTuning(1)
    tuned_classes = {}
    msc = C.c_double(0)
    for kw in (4, 5, 6):
        for lay, lname in enumerate(("targets>=5", "a target<5", "targets 0,1")):
            v = lib.quest_gb300_tunedKernel(n, kw, lay, C.byref(msc))
            if v:
                tuned_classes[f"k{kw} {lname}"] = {"variant": v, "ms_per_pass": round(msc.value, 3)}
    autotune = {"tune_s": round(tune_s, 2), "chosen_width": tuned_k, "kernel_variants": tuned_classes,
                "ms_per_circuit_tuned": round(ms_step, 2), "ms_per_circuit_fixed_defaults": round(default_kernels_ms, 2),
                "variants": "2: two loader groups on alternate chunks + one epilogue group; 3: one + one; "
                            "4: one + two; 5: two loader groups splitting each chunk + two epilogue groups"}

    # dominant kernel: group passes by applier and k
    groups = {}
    keys = []
    for i in range(npass):
        key = {0: f"kApplySimt<{kk[i]}> (FP32 FFMA)", 1: f"kApplyTC<{kk[i]}> (tcgen05 split-TF32, direct loads)",
               2: f"kApplyTC2<{kk[i]},2,1,1> (tcgen05 {pname}, pipelined)",
               3: f"kApplyTC2<{kk[i]},1,1,1> (tcgen05 {pname}, pipelined)",
               4: f"kApplyTC2<{kk[i]},1,2,1> (tcgen05 {pname}, pipelined)",
               5: f"kApplyTC2<{kk[i]},2,2,2> (tcgen05 {pname}, pipelined)"}[tc[i]]
        keys.append(key)
        g = groups.setdefault(key, [0, 0.0])
        g[0] += 1
        g[1] += pass_ms[i]
    dom_name, (dom_count, dom_ms) = max(groups.items(), key=lambda kv: kv[1][1])
    dom_avg = dom_ms / dom_count

    # ---- plain FP64 engine on the same circuit (per-gate, QuEST API) ------
    q64 = L.create(n)
    plain_ms = None
    if not args.skip_plain:
        lib.initZeroState(q64)
        run_plain_step(L, q64, ops)
        lib.calcTotalProb(q64)
        lib.initZeroState(q64)
        lib.quest_gb300_eventRecord(2)
        run_plain_step(L, q64, ops)
        lib.calcTotalProb(q64)
        lib.quest_gb300_eventRecord(3)
        plain_ms = lib.quest_gb300_eventElapsedMs(2, 3)
        err = C.c_double(0)
        one_minus_f = lib.quest_gb300_compareF32(q32, q64, C.byref(err))
        max_amp_err = err.value
    else:
        one_minus_f = max_amp_err = None

    # ---- the plain path's double-float mode, and one plain gate alone ----
    plain_df = None
    gate_roof = None
    if not args.skip_plain:
        qdf = L.create(n)
        lib.quest_gb300_setPlainArithmetic(1)
        lib.initZeroState(qdf)
        run_plain_step(L, qdf, ops)
        lib.calcTotalProb(qdf)
        lib.initZeroState(qdf)
        lib.quest_gb300_eventRecord(10)
        run_plain_step(L, qdf, ops)
        lib.calcTotalProb(qdf)
        lib.quest_gb300_eventRecord(11)
        df_ms = lib.quest_gb300_eventElapsedMs(10, 11)
        ip = lib.calcInnerProduct(q64, qdf)
        n64, ndf = lib.calcTotalProb(q64), lib.calcTotalProb(qdf)
        plain_df = {"ms_per_circuit": round(df_ms, 1), "gbs": round(alg_bytes / (df_ms / 1e3) / 1e9, 1),
                    "speedup_vs_fp64": round(plain_ms / df_ms, 2),
                    "one_minus_fidelity_vs_fp64": 1 - (ip.real ** 2 + ip.imag ** 2) / (n64 * ndf),
                    "total_prob": ndf, "total_prob_err_vs_fp64": abs(ndf - n64),
                    "mode": "quest_gb300_setPlainArithmetic(1): general 2x2 gates in double-float on the FP32 pipes"}
        # one compactUnitary on qubit 10 of the 30-qubit state (no controls):
        # 32 B per amplitude (read + write of the FP64 complex state)
        from quantumlab_gb300.quest import Complex
        gate_roof = {}
        a_, b_ = Complex(0.6, 0.0), Complex(0.0, 0.8)
        for mode, name in ((0, "fp64"), (1, "double_float")):
            lib.quest_gb300_setPlainArithmetic(mode)
            lib.compactUnitary(qdf, 10, a_, b_)
            lib.quest_gb300_eventRecord(12)
            for _ in range(8):
                lib.compactUnitary(qdf, 10, a_, b_)
            lib.quest_gb300_eventRecord(13)
            gms = lib.quest_gb300_eventElapsedMs(12, 13) / 8
            gate_roof[name] = {"kernel": "kPairVec<" + ("OpCompact" if mode == 0 else "OpMatrix2DF") + ">",
                               "avg_launch_ms": round(gms, 4), "achieved_gbs": round((1 << n) * 32 / gms / 1e6, 1)}
        lib.quest_gb300_setPlainArithmetic(0)
        L.destroy(qdf)

    # ---- the same plan with the pipelined kernel's other operands ---------
    # (3-term split-TF32 is the default; 4-term split-BF16 and 3-term
    # split-FP16 are the others)
    others = {}
    dom_idx = [i for i in range(npass) if keys[i] == dom_name]
    for opr in (pr for pr in (0, 1, 2) if pr != prec):
        if lib.quest_gb300_setTensorCorePrecision(opr) != 0:
            continue
        fused_step()                                   # warm-up
        tf_pass = [0.0] * npass
        lib.quest_gb300_setPassEvents(1)
        lib.quest_gb300_eventRecord(4)
        for _ in range(args.steps):
            fused_step()
            lib.quest_gb300_passTimesMs(pt, npass)
            tf_pass = [a + pt[i] for i, a in enumerate(tf_pass)]
        lib.quest_gb300_eventRecord(5)
        lib.quest_gb300_setPassEvents(0)
        tf_ms = lib.quest_gb300_eventElapsedMs(4, 5) / args.steps
        tf_dom = sum(tf_pass[i] for i in dom_idx) / args.steps / max(1, len(dom_idx))
        other = {"ms_per_circuit": round(tf_ms, 2), "gbs": round(alg_bytes / (tf_ms / 1e3) / 1e9, 1),
                 "dominant_kernel_avg_ms": round(tf_dom, 4),
                 "note": "same plan; the applier choice of this precision may differ per pass"
                         + ("; fixed per-width kernel defaults (not tuned)" if opr == 2 else "")}
        if plain_ms:
            err = C.c_double(0)
            other["one_minus_fidelity"] = lib.quest_gb300_compareF32(q32, q64, C.byref(err))
            other["max_amp_err"] = err.value
            other["speedup_vs_plain"] = round(plain_ms / tf_ms, 2)
        others["fused_fp32_" + PREC_NAMES[opr].lower().replace("-", "_")] = other
    lib.quest_gb300_setTensorCorePrecision(prec)

    # ---- the same circuit at the other fusion widths ---------------------
    # (k = 4, 5 and the headline's 6 against the per-gate FP64 engine)
    widths = {}
    if not args.skip_widths:
        for kw in (4, 5, 6):
            if kw == k:
                widths[str(kw)] = {"passes": npass, "ms_per_circuit": round(ms_step, 2), "gbs": round(value / world, 1),
                                   "one_minus_fidelity": one_minus_f, "max_amp_err": max_amp_err,
                                   "speedup_vs_plain": round(plain_ms / ms_step, 2) if plain_ms else None,
                                   "note": "the headline arm"}
                continue
            pw = L.plan(n, kw, ops)
            npw = lib.quest_gb300_planCompile(pw)

            def width_step():
                lib.quest_gb300_initZeroStateF32(q32)
                lib.quest_gb300_applyPlanF32(q32, pw)
                return lib.quest_gb300_calcTotalProbF32(q32)

            width_step()                                   # warm-up (plan upload)
            lib.quest_gb300_eventRecord(6)
            for _ in range(args.steps):
                width_step()
            lib.quest_gb300_eventRecord(7)
            wms = lib.quest_gb300_eventElapsedMs(6, 7) / args.steps
            entry = {"passes": npw, "ms_per_circuit": round(wms, 2), "gbs": round(alg_bytes / (wms / 1e3) / 1e9, 1)}
            if plain_ms:
                err = C.c_double(0)
                entry["one_minus_fidelity"] = lib.quest_gb300_compareF32(q32, q64, C.byref(err))
                entry["max_amp_err"] = err.value
                entry["speedup_vs_plain"] = round(plain_ms / wms, 2)
            widths[str(kw)] = entry
            lib.quest_gb300_planDestroy(pw)

    # ---- the same width without control qubits (every controlled phase of
    # the random matching then needs both its qubits in one pass) ----------
    without_ctl = None
    if max(ctl) > 0:
        p0 = L.plan(n, tuned_k, ops, controls=0)
        np0 = lib.quest_gb300_planCompile(p0)

        def step0():
            lib.quest_gb300_initZeroStateF32(q32)
            lib.quest_gb300_applyPlanF32(q32, p0)
            return lib.quest_gb300_calcTotalProbF32(q32)

        step0()                                        # warm-up (plan upload)
        lib.quest_gb300_eventRecord(10)
        for _ in range(args.steps):
            step0()
        lib.quest_gb300_eventRecord(11)
        ms0 = lib.quest_gb300_eventElapsedMs(10, 11) / args.steps
        without_ctl = {"passes": np0, "ms_per_circuit": round(ms0, 2), "gbs": round(alg_bytes / (ms0 / 1e3) / 1e9, 1)}
        if plain_ms:
            err = C.c_double(0)
            without_ctl["one_minus_fidelity"] = lib.quest_gb300_compareF32(q32, q64, C.byref(err))
            without_ctl["max_amp_err"] = err.value
        lib.quest_gb300_planDestroy(p0)

    lib.quest_gb300_planDestroy(plan)
    lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)

    peak, peak_kind = peaks()
    if gate_roof:
        for g in gate_roof.values():
            g["frac"] = round(g["achieved_gbs"] / peak, 4)
    achieved = pass_bytes / (dom_avg / 1e3) / 1e9
    # the dominant kernel's tensor work: algorithmic complex MACs of a dense
    # 2^k x 2^k pass, 8 * 2^k real flops per amplitude, and what the
    # compensated form executes (3 MMA terms split-TF32, 4 split-BF16)
    tensor_rates = None
    if "kApplyTC2" in dom_name:
        kd = int(dom_name.split("<")[1].split(",")[0])
        alg_flops = 8.0 * (1 << kd) * (1 << n)
        terms = PREC_TERMS[prec]
        tensor_rates = {"k": kd, "algorithmic_flops_per_launch": alg_flops,
                        "algorithmic_tflops": round(alg_flops / (dom_avg / 1e3) / 1e12, 1),
                        "executed_tflops": round(terms * alg_flops / (dom_avg / 1e3) / 1e12, 1),
                        "executed_form": f"{terms} MMA terms ({pname})"}
    for other in others.values():
        other["dominant_kernel_frac"] = round(pass_bytes / (other["dominant_kernel_avg_ms"] / 1e3) / 1e9 / peak, 4)
    traffic = tensor_pct = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        prof = json.load(open(tp))
        kname = dom_name.split(" ")[0] + ((" " + ("tf32", "bf16", "fp16")[prec]) if "kApplyTC2" in dom_name else "")
        t = prof.get(kname)
        if t:
            traffic = t * (1 << n)
        tensor_pct = prof.get("_tensor_pipe_pct", {}).get(kname)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": (f"f32 state ({PREC_TERMS[prec]}-term {pname} tensor-core products, FP32 accumulation; "
                  + "; ".join(f"{PREC_TERMS[o]}-term {PREC_NAMES[o]} arm in fused_fp32_{PREC_NAMES[o].lower().replace('-', '_')}"
                              for o in (0, 1, 2) if o != prec)
                  + "; FP64 fusion products and reductions)"),
        "data": "synthetic (seeded Haar/CPhase-matching/CNOT-brickwork circuit)",
        "config": {"workload": f"{n}-qubit random circuit, {args.layers} layers: fused FP32 engine (k<={k}) vs plain FP64 per-gate engine",
                   "qubits": n, "layers": args.layers, "gates_per_circuit": len(ops), "fusion_max_qubits": k,
                   "fusion_max_control_qubits": max(ctl), "fused_passes": npass,
                   "algorithmic_bytes_per_circuit": alg_bytes,
                   "value_definition": "per-gate FP64 algorithmic bytes of the circuit / time per circuit",
                   "value_timed_region": ("initZeroStateF32, every fused pass of the compiled plan, FP64 total "
                                          "probability; the plan's search and FP64 products (plan_compile_s) and "
                                          "FP64<->FP32 conversions are outside it (e2e includes them)"),
                   "l2": "state 8 GiB (FP32) / 16 GiB (FP64) >> 129 MB L2, no flush needed",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "fused_fp32": {"ms_per_circuit": round(ms_step, 2), "gbs": round(value, 1), "passes": npass,
                       "controlled_passes": sum(1 for c in ctl if c > 0),
                       "plan_compile_s": round(plan_s, 3), "one_minus_fidelity": one_minus_f,
                       "max_amp_err": max_amp_err,
                       "kernels": {name: {"passes": c, "ms_per_circuit": round(t, 2)} for name, (c, t) in groups.items()}},
        **others,
        "fused_fp32_by_width": widths or None,
        "fused_fp32_without_control_qubits": without_ctl,
        "autotune": autotune,
        "plain_fp64": ({"ms_per_circuit": round(plain_ms, 1), "gbs": round(alg_bytes / (plain_ms / 1e3) / 1e9, 1),
                        "launches": len(ops)} if plain_ms else None),
        "plain_double_float": plain_df,
        "plain_gate_30q": gate_roof,
        "speedup_fused_vs_plain": round(plain_ms / ms_step, 2) if plain_ms else None,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "avg_launch_ms": round(dom_avg, 4), "launches_per_circuit": dom_count,
                     "bytes_per_launch": pass_bytes,
                     "tensor_pipe_active_pct_ncu": tensor_pct,
                     "tensor": tensor_rates},
        "e2e": {"value": round(world * alg_bytes / e2e_s / 1e9, 2), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
                "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes + 8,
                "ms_per_step": round(e2e_s * 1e3, 2),
                "path": "QuEST C ABI: initStateFromAmps (pinned host FP64; a seeded random product state), one API "
                        "call per gate with op-stream capture on, calcTotalProb, copyStateFromGPU",
                "total_prob": e2e_prob,
                "split_ms": {"h2d_initStateFromAmps": round(split[0] * 1e3, 1),
                             "gates_and_flush": round(split[1] * 1e3, 1),
                             "d2h_copyStateFromGPU": round(split[2] * 1e3, 1)},
                "d2h_ms_each_step": d2h_each, "d2h_ms_repeated_alone": d2h_repeat,
                "host_mirrors_pinned": mirrors_pinned, "link_probe_1GiB": link},
        "gpu_launches": int(launches // max(1, args.steps)),
        "gpu_launches_timed_region": int(launches),
        "total_prob_fp32": total32,
        "wall_s": round(wall, 3),
    }
    clk_sum = clk.summary()
    if clk_sum:
        out["clocks"] = clk_sum
    return out


# ------------------------------------------------------- batched swap tests
def run_swaps(args, rank=0, world=1):
    """65,536 QKMeans swap tests (4096 vectors x 16 centroids, 9..21 qubits):
    the batched engine (one persistent kernel, CUDA-graph replay) against one
    circuit at a time through the QuEST API (the reference pattern, per-gate
    FP64 kernels) on a per-size subsample, extrapolated over the size mix.
    With N ranks the tests are dealt by size (no device collective); the
    batch time is the maximum over ranks and the results are gathered to
    rank 0.  Returns None on ranks other than 0."""
    import ctypes as C
    import quantumlab_gb300 as qg
    from quantumlab_gb300 import sharding
    from quantumlab_gb300 import workloads as W

    L = qg.load()
    lib = L.lib
    ds, comps, vecs, cents = W.gaussian_mixture_vectors(count=args.swap_vectors, seed=5)
    pool, offsets, dims, ia_all, ib_all = W.swap_test_pool(vecs, cents)
    mine = sharding.shard_units(sharding.swap_test_cost(dims[ia_all]), world, rank)
    ia = np.ascontiguousarray(ia_all[mine])
    ib = np.ascontiguousarray(ib_all[mine])
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    t0 = time.perf_counter()
    h = lib.quest_gb300_swapTestBatchCreate(P(pool, C.c_double), P(offsets, C.c_longlong), P(dims, C.c_int),
                                            len(offsets), P(ia, C.c_int), P(ib, C.c_int), len(ia))
    create_s = time.perf_counter() - t0
    tc, ts_, tb, td = C.c_int(0), C.c_int(0), C.c_double(0), C.c_double(0)
    lib.quest_gb300_swapTestBatchTune(h, C.byref(tc), C.byref(ts_), C.byref(tb), C.byref(td))
    swap_tune = {"ctas_per_sm": tc.value, "smem_max_amps": ts_.value, "ms_tuned": round(tb.value, 3),
                 "ms_default_4ctas_8192": round(td.value, 3)}
    out = np.zeros(len(ia))
    for _ in range(3):
        lib.quest_gb300_swapTestBatchRun(h, P(out, C.c_double))
    reps = 5
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(reps):
        lib.quest_gb300_swapTestBatchRun(h, P(out, C.c_double))
    batch_s = sharding.max_over_ranks((time.perf_counter() - t0) / reps, world)
    lib.quest_gb300_swapTestBatchDestroy(h)
    full = sharding.gather_to_rank0(mine, out, len(ia_all), world)
    if rank != 0:
        return None
    ia, ib, out = ia_all, ib_all, full
    items = list(vecs) + [m for d in range(4, 11) for m in cents[d]]
    want = np.array([(1 + np.dot(items[a], items[b]) ** 2) / 2 for a, b in zip(ia, ib)])
    err = float(np.max(np.abs(out - want)))
    # one circuit at a time through the QuEST API, per size class
    per_size = {}
    counts = {d: int(np.sum(dims[ia] == d)) for d in range(4, 11)}
    for d in range(4, 11):
        pick = [k for k in range(len(ia)) if dims[ia[k]] == d][: args.swap_sample]
        q = L.create(2 * d + 1)
        W.swap_test_plain(L, q, items[ia[pick[0]]], items[ib[pick[0]]], d)     # warm-up
        t0 = time.perf_counter()
        for k in pick:
            p = W.swap_test_plain(L, q, items[ia[k]], items[ib[k]], d)
        per_size[d] = (time.perf_counter() - t0) / len(pick)
        L.destroy(q)
    plain_total = sum(counts[d] * per_size[d] for d in counts)
    return {
        "tests": int(len(ia)), "qubits": "9..21", "tests_per_s": round(len(ia) / batch_s, 1),
        "ranks": world, "partitioning": "tests dealt by state size, no device collective" if world > 1 else "1 GPU",
        "batch_ms": round(batch_s * 1e3, 3), "create_s": round(create_s, 3), "autotune": swap_tune,
        "max_abs_err_vs_fp64_closed_form": err,
        "per_gate_tests_per_s": round(len(ia) / plain_total, 1),
        "per_gate_sample": f"{args.swap_sample} circuits per size d=4..10, extrapolated over the size mix",
        "speedup_batched_vs_per_gate": round(plain_total / batch_s, 1),
    }


# ------------------------------------------------ the other configurations
def c4_batch(L, reps=3, keep_states=False):
    """All 64 Fermi-Hubbard instances of configuration 4 (U in {2, 4, 8}, dt in
    {0.1, 0.05, 0.01}, order 1 or 2: 10 to 100 steps) evolved as one Trotter
    batch at 24 qubits.  The batch falls into classes of one (order, steps)
    shape; per class one plan and one launch per pass over all its states;
    the whole run is one CUDA graph after the first run; energies come from
    the FP32 states.  Returns the energies and the time per run (CUDA events
    over `reps` replays); with keep_states the batch handle is returned for
    trotterBatchCopyState (the caller destroys it)."""
    import ctypes as C
    from quantumlab_gb300 import workloads as W

    lib = L.lib
    sites, n4, T = 12, 24, 1.0
    inst = W.hubbard_instances(64)
    hb, consts = [], []
    batch = lib.quest_gb300_trotterBatchCreate(n4, len(inst))
    for i, (U, dt, order) in enumerate(inst):
        codes, coeffs, const = W.hubbard_terms(sites, U)
        hb.append(L.pauli_hamil(codes, coeffs))
        consts.append(const)
        lib.quest_gb300_trotterBatchSetInstance(batch, i, hb[-1], T, order, int(round(T / dt)), W.neel_index(sites))
    eb = (C.c_double * len(inst))()
    t0 = time.perf_counter()
    rc = lib.quest_gb300_trotterBatchRun(batch, eb)            # compile, eager run, graph capture
    first_s = time.perf_counter() - t0
    lib.quest_gb300_eventRecord(32)
    for _ in range(reps):
        rc |= lib.quest_gb300_trotterBatchRun(batch, eb)
    lib.quest_gb300_eventRecord(33)
    batch_ms = lib.quest_gb300_eventElapsedMs(32, 33) / max(1, reps)
    out = {"rc": rc, "energies": [e + c for e, c in zip(eb, consts)], "batch_ms": batch_ms,
           "passes": lib.quest_gb300_trotterBatchNumPasses(batch),
           "classes": lib.quest_gb300_trotterBatchNumClasses(batch), "first_s": first_s,
           "batch": None}
    for h in hb:
        lib.destroyPauliHamil(h)
    if keep_states:
        out["batch"] = batch
    else:
        lib.quest_gb300_trotterBatchDestroy(batch)
    return out


def run_configs(args):
    """Secondary lines for the configurations the headline does not cover
    (their parity is in tests/): C1 the 20-qubit plain FP64 circuit (GPU
    per-gate engine against the CPU QuEST path, whole circuit); C3 the noisy
    14-qubit density matrix (per-gate FP64, and with op-stream capture: gates
    fused between the channels); C4 Fermi-Hubbard Trotter instances at 24
    qubits (one multiRotatePauli pass per term, and captured: the Trotter
    rotations fused), on a sample of instances, and the instances of one
    shape batched."""
    import ctypes as C

    import quantumlab_gb300 as qg
    from quantumlab_gb300 import workloads as W

    L = qg.load()
    lib = L.lib
    out = {}

    def gpu_ms(fn):
        lib.quest_gb300_eventRecord(30)
        r = fn()
        lib.quest_gb300_eventRecord(31)
        return lib.quest_gb300_eventElapsedMs(30, 31), r

    # ---- C1 ----
    n1 = 20
    ops1 = W.c1_circuit(n=n1, layers=40, seed=1)
    alg1 = W.algorithmic_bytes(ops1, n1)

    def c1(L_, q_):
        L_.lib.initZeroState(q_)
        W.run_ops(L_, q_, ops1)
        return L_.lib.calcTotalProb(q_)

    q = L.create(n1)
    c1(L, q)
    ms1 = statistics.median([gpu_ms(lambda: c1(L, q))[0] for _ in range(3)])
    amps_fp64 = L.amps(q).copy()
    lib.quest_gb300_setPlainArithmetic(1)
    c1(L, q)
    ms1df = statistics.median([gpu_ms(lambda: c1(L, q))[0] for _ in range(3)])
    err1df = float(np.max(np.abs(L.amps(q) - amps_fp64)))
    lib.quest_gb300_setPlainArithmetic(0)
    L.destroy(q)
    Lc, kind = cpu_library()
    qc = Lc.create(n1)
    t0 = time.perf_counter()
    c1(Lc, qc)
    cpu1 = (time.perf_counter() - t0) * 1e3
    Lc.destroy(qc)
    out["c1_plain_fp64_20q"] = {"gates": len(ops1), "gpu_ms": round(ms1, 2), "gpu_gbs": round(alg1 / ms1 / 1e6, 1),
                                "gpu_ms_double_float": round(ms1df, 2), "double_float_max_amp_err_vs_fp64": err1df,
                                "cpu_ms": round(cpu1, 1), "cpu_kind": kind, "cpu_cores": os.cpu_count(),
                                "speedup_gpu_vs_cpu": round(cpu1 / ms1, 1)}
    # ---- C3 ----
    n3 = 14
    ops3 = W.c3_circuit(nq=n3, layers=10, seed=3)
    res3 = {}
    for mode in (0, 1):
        q = L.create(n3, density=True)
        lib.quest_gb300_setCapture(q, mode)
        lib.initZeroState(q)
        W.run_ops(L, q, ops3[:63])                     # warm-up: one layer
        lib.calcTotalProb(q)

        def c3():
            lib.initZeroState(q)
            W.run_ops(L, q, ops3)
            return lib.calcPurity(q)

        res3[mode] = gpu_ms(c3)
        trace = lib.calcTotalProb(q)
        p1 = np.array([lib.calcProbOfOutcome(q, t, 1) for t in range(n3)])
        rho = L.amps(q)
        res3[mode] = res3[mode] + (trace, p1, rho)
        L.destroy(q)
    (ms_p, pur_p, tr_p, p1_p, rho_p), (ms_c, pur_c, tr_c, p1_c, rho_c) = res3[0], res3[1]
    out["c3_noisy_dm_14q"] = {"ops": len(ops3), "plain_ms": round(ms_p, 1), "captured_ms": round(ms_c, 1),
                              "purity_plain": pur_p, "purity_captured": pur_c,
                              "purity_rel_err": abs(pur_c / pur_p - 1),
                              "trace_plain": tr_p, "trace_captured": tr_c, "trace_err": abs(tr_c - tr_p),
                              "max_p1_err": float(np.max(np.abs(p1_c - p1_p))),
                              "max_entry_err": float(np.max(np.abs(rho_c - rho_p))),
                              "errors_vs": "the same calls on the plain FP64 per-gate path",
                              "speedup_captured": round(ms_p / ms_c, 2)}
    del rho_p, rho_c
    # ---- C4 ----
    # One instance per (dt, order) class runs through the plain FP64 path (one
    # multiRotatePauli pass per term) and through op-stream capture; then all
    # 64 instances run as one Trotter batch, and each sampled instance's batch
    # state is checked against its FP64 state (1 - F, max |d amp|, energy,
    # site occupations <n_q> = P(q = 1)).
    sites, n4, T = 12, 24, 1.0
    inst = W.hubbard_instances(64)
    sample = [0, 3, 6, 9, 12, 15]                      # dt .1/.05/.01 at order 1, then order 2
    rows, plain_states = [], {}
    ws = L.create(n4)
    for i in sample:
        U, dt, order = inst[i]
        codes, coeffs, const = W.hubbard_terms(sites, U)
        h = L.pauli_hamil(codes, coeffs)
        steps = int(round(T / dt))
        r = {}
        for mode in (0, 1):
            q = L.create(n4)
            lib.quest_gb300_setCapture(q, mode)

            def c4():
                lib.initClassicalState(q, W.neel_index(sites))
                lib.applyTrotterCircuit(q, h, T, order, steps)
                return lib.calcExpecPauliHamil(q, h, ws) + const

            if mode == 1:
                c4()                                   # warm-up (plan upload, FP32 scratch)
            r[mode] = gpu_ms(c4)
            if mode == 0:
                occ = [lib.calcProbOfOutcome(q, t, 1) for t in range(n4)]
                plain_states[i] = (q, occ)
            else:
                L.destroy(q)
        lib.destroyPauliHamil(h)
        rows.append({"instance": i, "U": U, "dt": dt, "order": order, "steps": steps,
                     "plain_ms": round(r[0][0], 2), "captured_ms": round(r[1][0], 2),
                     "energy_plain": r[0][1], "energy_captured": r[1][1],
                     "coeff_abs_sum": float(np.sum(np.abs(coeffs)))})
    L.destroy(ws)
    # The lab's own Trotter builder (PauliProduct::OneStepGate): every term as
    # a basis change + CNOT ladder into an ancilla + Rz + inverse, one QuEST
    # call per gate, on 24 + 1 qubits (instance 0, first order, 10 steps).
    U, dt, order = inst[0]
    codes, coeffs, const = W.hubbard_terms(sites, U)
    lab_ops = W.lab_trotter_ops(codes, coeffs, dt, int(round(T / dt)), ancilla=n4)
    h25 = L.pauli_hamil(np.concatenate([codes, np.zeros((len(codes), 1), dtype=codes.dtype)], axis=1), coeffs)
    ws = L.create(n4 + 1)
    lab = {}
    for mode in (0, 1):
        q = L.create(n4 + 1)
        lib.quest_gb300_setCapture(q, mode)

        def c4lab():
            lib.initClassicalState(q, W.neel_index(sites))
            W.run_ops(L, q, lab_ops)
            return lib.calcExpecPauliHamil(q, h25, ws) + const

        c4lab()
        lab[mode] = gpu_ms(c4lab)
        L.destroy(q)
    lib.destroyPauliHamil(h25)
    L.destroy(ws)
    # all 64 instances in one batch (tensor-core variants tuned at 24 qubits)
    lib.quest_gb300_autotune(n4)
    bat = c4_batch(L, reps=2, keep_states=True)
    checks = []
    qb = L.create(n4)
    for r in rows:
        i = r["instance"]
        qp, occ_plain = plain_states[i]
        lib.quest_gb300_trotterBatchCopyState(bat["batch"], i, qb)
        a, b = L.amps(qp), L.amps(qb)
        fid = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
        occ_b = [lib.calcProbOfOutcome(qb, t, 1) for t in range(n4)]
        checks.append({"instance": i, "one_minus_fidelity": float(1 - fid), "max_amp_err": float(np.max(np.abs(a - b))),
                       "energy_err": abs(bat["energies"][i] - r["energy_plain"]),
                       "energy_err_rel_coeff_sum": abs(bat["energies"][i] - r["energy_plain"]) / r["coeff_abs_sum"],
                       "max_occupation_err": float(np.max(np.abs(np.array(occ_b) - np.array(occ_plain))))})
        L.destroy(qp)
    L.destroy(qb)
    lib.quest_gb300_trotterBatchDestroy(bat["batch"])
    # the per-instance cost depends on (dt, order) only: the sampled instance
    # of each class stands for the class's members
    cls = {(inst[r["instance"]][1], inst[r["instance"]][2]): r for r in rows}
    plain_all = sum(cls[(dt, o)]["plain_ms"] for _, dt, o in inst)
    capt_all = sum(cls[(dt, o)]["captured_ms"] for _, dt, o in inst)
    batched = {"instances": len(inst), "classes": bat["classes"], "qubits": n4,
               "pass_launches_per_run": bat["passes"], "batch_ms": round(bat["batch_ms"], 2),
               "ms_per_instance": round(bat["batch_ms"] / len(inst), 3), "first_run_s": round(bat["first_s"], 3),
               "checks_vs_fp64": checks,
               "max_one_minus_fidelity": max(c["one_minus_fidelity"] for c in checks),
               "max_energy_err_rel_coeff_sum": max(c["energy_err_rel_coeff_sum"] for c in checks),
               "max_occupation_err": max(c["max_occupation_err"] for c in checks),
               "checked": "one instance per (dt, order) class against its plain FP64 run",
               "plain_ms_all_64": round(plain_all, 1), "captured_ms_all_64": round(capt_all, 1),
               "estimate": "plain/captured totals: each class's sampled instance time x the class's members",
               "speedup_vs_plain": round(plain_all / bat["batch_ms"], 1),
               "speedup_vs_captured_one_at_a_time": round(capt_all / bat["batch_ms"], 2)}
    out["c4_hubbard_24q"] = {"instances_timed": len(rows), "rows": rows, "batched": batched,
                             "max_abs_energy_diff_captured": max(abs(x["energy_plain"] - x["energy_captured"]) for x in rows),
                             "speedup_captured": round(sum(x["plain_ms"] for x in rows) / sum(x["captured_ms"] for x in rows), 2),
                             "lab_builder": {"instance": 0, "qubits": n4 + 1, "gates": len(lab_ops),
                                             "plain_ms": round(lab[0][0], 1), "captured_ms": round(lab[1][0], 1),
                                             "energy_plain": lab[0][1], "energy_captured": lab[1][1],
                                             "speedup_captured": round(lab[0][0] / lab[1][0], 1)}}
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


def cpu_sample(n, layers, sample_ops, repeats=1, warmup=0):
    """Time the first `sample_ops` gates of the circuit (by default its first
    layer: one-qubit gates, CPhase matching and CNOT brickwork in the
    circuit's proportions) on the CPU library at full size, on one register
    reused across repetitions.  Returns ([GB/s per repetition], [seconds],
    kind, gates timed)."""
    from quantumlab_gb300 import workloads as W
    L, kind = cpu_library()
    ops = W.c2_circuit(n=n, layers=layers, seed=2)[:sample_ops]
    q = L.create(n)
    gbs, secs = [], []
    for i in range(warmup + repeats):
        t0 = time.perf_counter()
        W.run_ops(L, q, ops)
        dt = time.perf_counter() - t0
        if i >= warmup:
            secs.append(dt)
            gbs.append(W.algorithmic_bytes(ops, n) / dt / 1e9)
    L.destroy(q)
    return gbs, secs, kind, len(ops)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    n = args.qubits
    gbs, secs, kind, nops = cpu_sample(n, args.layers, args.cpu_sample_ops, repeats=args.steps, warmup=args.warmup)
    value = statistics.median(gbs)
    ms = statistics.median(secs) * 1e3
    cores = os.cpu_count()
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "GB/s (per-gate FP64 algorithmic bytes)", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Haar/CPhase-matching/CNOT-brickwork circuit)",
        "config": {"workload": f"{n}-qubit random circuit, {args.layers} layers (first {nops} gates = the first layer, per step)",
                   "qubits": n, "layers": args.layers},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s (per-gate FP64 algorithmic bytes)", "cores": cores,
                         "kind": kind, "sample": f"first {nops} gates (one layer) of the {n}-qubit circuit per step, OpenMP on all host threads"},
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
    ap.add_argument("--cpu-sample-ops", type=int, default=60)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fusion", type=int, default=6, help="max qubits per fused pass (1..6)")
    ap.add_argument("--precision", default="tf32", choices=["tf32", "bf16", "fp16"],
                    help="operands of the pipelined tensor-core kernel for the headline arm")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-widths", action="store_true", help="skip the k = 4 and k = 5 fused arms")
    ap.add_argument("--no-tune", action="store_true", help="fixed fusion width (the kernel variants are still tuned)")
    ap.add_argument("--no-swap", action="store_true")
    ap.add_argument("--swap-vectors", type=int, default=4096)
    ap.add_argument("--swap-sample", type=int, default=6)
    ap.add_argument("--no-configs", action="store_true", help="skip the configuration 1/3/4 lines")
    ap.add_argument("--c4-batch-only", action="store_true",
                    help="only the batched Trotter run of configuration 4 (64 instances, 24 qubits); for profiling")
    args = ap.parse_args()
    rank, world, local = dist_info()
    os.environ.setdefault("QUEST_GB300_DEVICE", str(local))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if args.c4_batch_only:
        import quantumlab_gb300 as qg
        bat = c4_batch(qg.load(), reps=args.steps)
        print(json.dumps({"c4_batch": {k: v for k, v in bat.items() if k != "batch"}}), flush=True)
        return
    out = run_gpu(args, rank, world)
    if not args.no_swap:
        sw = run_swaps(args, rank, world)
        if rank == 0:
            out["swap_tests"] = sw
    if not args.no_configs and rank == 0:
        out["configs"] = run_configs(args)
    if rank == 0:
        if not args.no_cpu_baseline:
            gbs, secs, kind, nops = cpu_sample(args.qubits, args.layers, args.cpu_sample_ops)
            out["cpu_baseline"] = {"value": round(gbs[0], 3), "unit": "GB/s (per-gate FP64 algorithmic bytes)",
                                   "cores": os.cpu_count(), "kind": kind,
                                   "sample": f"first {nops} gates (one layer) of the {args.qubits}-qubit circuit ({secs[0]:.1f} s), OpenMP on all host threads"}
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
