"""The product's plain FP64 kernels against the reference's own GPU kernels.

oracle/_ref/quest_gpu_ref.cubin is the device code of the reference's GPU
backend (Code/QuEST340/QuEST/src/GPU/QuEST_gpu.cu), compiled for sm_103a from
the reference sources by `make -C oracle refgpu` where those sources are
mounted (the cubin travels with the tree; the tests skip without it).  Its
kernels have C linkage, so they are launched here by name through the CUDA
driver API, with the launch shapes of the reference's host wrappers (128
threads per block; QuEST_gpu.cu:825-830 compactUnitary, 1521-1530
controlledPhaseShift, 1867-1873 controlledNot), on the device state of a
register the product created (the Qureg layout is the reference's).

Parity: the same circuit through the product's API and through the reference
kernels agrees to 1e-12 x max|amp| (it is bit-identical on GB300).  Timing
(printed; -s): the random circuit of the fused benchmark, layers of Haar
compactUnitary on every qubit, controlledPhaseShift on a random matching and
CNOT brickwork, one kernel per gate on each side, at QG_REF_GPU_QUBITS qubits
(default 24), and each gate kind alone.
"""
import ctypes as C
import math
import os
import time

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W
from quantumlab_gb300.quest import Complex

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "quest_gpu_ref.cubin")
THREADS = 128                      # threadsPerCUDABlock of every wrapper used here


class RefKernels:
    """The reference's state-vector gate kernels, loaded from the cubin into
    the current (primary) context."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 7 + [C.c_void_p, C.POINTER(C.c_void_p),
                                                                             C.POINTER(C.c_void_p)]
        self.cu.cuModuleUnload.argtypes = [C.c_void_p]
        self.mod = C.c_void_p()
        self._check(self.cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("statevec_compactUnitaryKernel", "statevec_controlledPhaseShiftKernel",
                     "statevec_controlledNotKernel"):
            f = C.c_void_p()
            self._check(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def _launch(self, name, num_tasks, args):
        # each argument is a ctypes object; cuLaunchKernel copies it by value
        params = (C.c_void_p * len(args))(*[C.addressof(a) for a in args])
        blocks = (num_tasks + THREADS - 1) // THREADS
        self._check(self.cu.cuLaunchKernel(self.fn[name], blocks, 1, 1, THREADS, 1, 1, 0, None, params, None), name)

    def run(self, q, ops):
        """Apply the circuit's gates to register q, one reference kernel each
        (the state-vector paths of the reference's front-end)."""
        n_amps = q.numAmpsPerChunk
        for op in ops:
            if op[0] == "cu":
                _, t, ar, ai, br, bi = op
                self._launch("statevec_compactUnitaryKernel", n_amps >> 1,
                             [q, C.c_int(t), Complex(ar, ai), Complex(br, bi)])
            elif op[0] == "cp":
                _, c, t, theta = op
                self._launch("statevec_controlledPhaseShiftKernel", n_amps,
                             [q, C.c_int(c), C.c_int(t), C.c_double(math.cos(theta)), C.c_double(math.sin(theta))])
            elif op[0] == "cx":
                _, c, t = op
                self._launch("statevec_controlledNotKernel", n_amps, [q, C.c_int(c), C.c_int(t)])
            else:
                raise ValueError(op)

    def sync(self):
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def close(self):
        self.cu.cuModuleUnload(self.mod)


@pytest.fixture(scope="module")
def ref_kernels(gpulib):
    if not os.path.exists(CUBIN):
        pytest.skip("the reference's GPU device code is not built (make -C oracle refgpu)")
    q = gpulib.create(3)                 # the product's context is current on this thread
    k = RefKernels()
    yield k
    k.close()
    gpulib.destroy(q)


def _random_state(n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return psi / np.linalg.norm(psi)


@pytest.mark.parametrize("n,layers", [(12, 6), (20, 4)])
def test_plain_kernels_match_reference_gpu_kernels(gpulib, ref_kernels, n, layers):
    L = gpulib
    ops = W.c2_circuit(n=n, layers=layers, seed=31 + n)
    psi = _random_state(n, n)
    out = []
    for side in ("product", "reference"):
        q = L.create(n)
        L.set_amps(q, psi)
        L.lib.syncQuESTEnv(L.env)
        if side == "product":
            W.run_ops(L, q, ops)
        else:
            ref_kernels.run(q, ops)
            ref_kernels.sync()
        out.append(L.amps(q).copy())
        L.destroy(q)
    err = float(np.max(np.abs(out[0] - out[1])))
    print(f"n={n} gates={len(ops)}: max|d amp| product vs reference GPU kernels = {err:.2e}")
    assert err <= 1e-12 * float(np.max(np.abs(out[1])))


def _timed(L, ref_kernels, q, ops, side, reps=2):
    best = math.inf
    for _ in range(reps):
        L.lib.initZeroState(q)
        L.lib.syncQuESTEnv(L.env)
        ref_kernels.sync()
        t0 = time.perf_counter()
        if side == "reference":
            ref_kernels.run(q, ops)
            ref_kernels.sync()
        else:
            W.run_ops(L, q, ops)
            L.lib.syncQuESTEnv(L.env)
        best = min(best, time.perf_counter() - t0)
    return best * 1e3


def test_reference_gpu_kernel_timing(gpulib, ref_kernels):
    """Per-gate time of the 20-layer random circuit: the reference's kernels
    against the product's plain path (both one kernel per gate; FP64, and the
    double-float mode), and the product's fused FP32 engine on the same
    circuit; then each gate kind alone (12 gates of a kind, spread targets)."""
    L = gpulib
    n = int(os.environ.get("QG_REF_GPU_QUBITS", "24"))
    ops = W.c2_circuit(n=n, layers=20, seed=2)
    res = {}
    q = L.create(n)
    for side in ("reference", "product", "product_df"):
        L.lib.quest_gb300_setPlainArithmetic(1 if side == "product_df" else 0)
        res[side] = _timed(L, ref_kernels, q, ops, "reference" if side == "reference" else "product")
        res[side + "_prob"] = L.lib.calcTotalProb(q)
    L.lib.quest_gb300_setPlainArithmetic(0)
    kinds = {}
    for kind in ("cu", "cx", "cp"):
        sample = [o for o in ops if o[0] == kind]
        sample = [sample[i * len(sample) // 12] for i in range(12)]
        kinds[kind] = [_timed(L, ref_kernels, q, sample, side) / len(sample) for side in ("reference", "product")]
    L.destroy(q)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    plan = L.plan(n, 6, ops)
    best = math.inf
    for _ in range(2):
        L.lib.quest_gb300_initZeroStateF32(q32)
        L.lib.syncQuESTEnv(L.env)
        t0 = time.perf_counter()
        assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
        L.lib.syncQuESTEnv(L.env)
        best = min(best, time.perf_counter() - t0)
    res["fused"] = best * 1e3
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    alg = W.algorithmic_bytes(ops, n)
    print(f"\n{n} qubits, {len(ops)} gates ({alg / 1e9:.1f} GB of per-gate FP64 algorithmic bytes):")
    for side in ("reference", "product", "product_df", "fused"):
        print(f"  {side:10s} {res[side]:10.2f} ms  {alg / res[side] / 1e6:9.1f} GB/s  "
              f"{res['reference'] / res[side]:6.2f}x the reference's GPU kernels")
    names = {"cu": "compactUnitary", "cx": "controlledNot", "cp": "controlledPhaseShift"}
    for kind, (r, p) in kinds.items():
        print(f"  {names[kind]:20s} per gate: reference {r:8.3f} ms, product {p:8.3f} ms ({r / p:5.2f}x)")
    for side in ("reference", "product", "product_df"):
        assert abs(res[side + "_prob"] - 1) < 1e-10
