"""quest_gb300_sampleMeasurements against QuantumLab's shot loop (GPU).

The loop (QLSimulatorMeasure.cpp:70-109): for every shot, measure each listed
qubit in order; restore the state with copyStateToGPU before every shot but
the first.  With the same seed the sampler must give the same outcome codes
and leave the MT19937 stream at the same position.  Two measured qubits are
certain (|0> and |1>), which QuEST resolves without a draw."""
import ctypes as C
import time

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu

QUBITS = [3, 10, 0, 11, 7]
SHOTS = 300


def prepared(L, n=12):
    q = L.create(n)
    L.lib.initZeroState(q)
    ops = [op for op in W.c2_circuit(n=10, layers=4, seed=9)]      # qubits 0..9 only
    W.run_ops(L, q, ops)
    L.lib.pauliX(q, 11)                                              # qubit 10 stays |0>, 11 is |1>
    pre = np.array(L.amps(q))                                        # also syncs the host mirror
    return q, pre


def marker(L, k=16):
    """k outcomes of measuring |+>: reveals the MT stream position."""
    p = L.create(1)
    out = []
    for _ in range(k):
        L.lib.initPlusState(p)
        out.append(L.lib.measure(p, 0))
    L.destroy(p)
    return out


def test_sampler_reproduces_the_lab_shot_loop(gpulib):
    L = gpulib
    lib = L.lib
    q, pre = prepared(L)
    L.seed([7, 11])
    loop = []
    for shot in range(SHOTS):
        if shot:
            lib.copyStateToGPU(q)
        code = 0
        for j, t in enumerate(QUBITS):
            code |= lib.measure(q, t) << j
        loop.append(code)
    after_loop = marker(L)

    lib.copyStateToGPU(q)
    L.seed([7, 11])
    out = (C.c_int * SHOTS)()
    qs = (C.c_int * len(QUBITS))(*QUBITS)
    assert lib.quest_gb300_sampleMeasurements(q, qs, len(QUBITS), SHOTS, out) == 0
    sampled = list(out)
    after_sampler = marker(L)
    assert sampled == loop
    assert after_sampler == after_loop
    # qubit 10 (bit 1) is always 0, qubit 11 (bit 3) always 1
    assert all((c >> 1) & 1 == 0 and (c >> 3) & 1 == 1 for c in sampled)
    # the register still holds the pre-measurement state
    assert np.max(np.abs(L.amps(q) - pre)) == 0
    L.destroy(q)


def test_sampler_frequencies_follow_the_outcome_probabilities(gpulib):
    L = gpulib
    lib = L.lib
    q, _ = prepared(L)
    L.seed([3])
    shots = 20000
    out = (C.c_int * shots)()
    qs = (C.c_int * 3)(0, 3, 7)
    assert lib.quest_gb300_sampleMeasurements(q, qs, 3, shots, out) == 0
    freq = np.bincount(np.array(out), minlength=8) / shots
    probs = L.calcProbOfAllOutcomes(q, [0, 3, 7])
    assert np.max(np.abs(freq - probs)) < 5 * np.sqrt(0.25 / shots)
    L.destroy(q)


def test_sampler_timing_against_the_lab_shot_loop(gpulib):
    """Wall time of 64 shots of 5 qubits on a 24-qubit register: the lab's
    loop (copyStateToGPU + one measure per qubit, every shot) against one
    sampleMeasurements call; both draw the same outcomes (printed; -s)."""
    L = gpulib
    lib = L.lib
    n, shots = 24, 64
    qubits = [0, 5, 11, 17, 23]
    q = L.create(n)
    lib.initZeroState(q)
    W.run_ops(L, q, W.c2_circuit(n=n, layers=2, seed=5))
    lib.copyStateFromGPU(q)
    times = {}
    codes = {}
    for side in ("loop", "sampler"):
        L.seed([21])
        lib.syncQuESTEnv(L.env)
        t0 = time.perf_counter()
        if side == "loop":
            got = []
            for shot in range(shots):
                if shot:
                    lib.copyStateToGPU(q)
                code = 0
                for j, t in enumerate(qubits):
                    code |= lib.measure(q, t) << j
                got.append(code)
        else:
            out = (C.c_int * shots)()
            qs = (C.c_int * len(qubits))(*qubits)
            assert lib.quest_gb300_sampleMeasurements(q, qs, len(qubits), shots, out) == 0
            got = list(out)
        lib.syncQuESTEnv(L.env)
        times[side] = (time.perf_counter() - t0) * 1e3
        codes[side] = got
        lib.copyStateToGPU(q)
    assert codes["sampler"] == codes["loop"]
    print(f"\n{n} qubits, {shots} shots of {len(qubits)} qubits: lab loop {times['loop']:.1f} ms, "
          f"sampler {times['sampler']:.2f} ms ({times['loop'] / times['sampler']:.0f}x)")
    L.destroy(q)
