"""Op-stream capture (GPU): gate calls through the QuEST API with capture on
are queued and applied through the fused FP32 engine at the first
state-reading call; the result must match the same calls run directly in
FP64 to the fused engine's bounds (1 - F <= 1e-6, max |d amp| <= 1e-5)."""
import ctypes as C

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W
from quantumlab_gb300.quest import Complex, ComplexMatrix2, ComplexMatrix4, Vector

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def no_library_errors(gpulib):
    gpulib.capture_errors()
    gpulib.errors.clear()
    yield
    errors = list(gpulib.errors)
    gpulib.errors.clear()
    assert not errors, errors


def haar(rng, k):
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    return np.linalg.qr(z)[0]


def mixed_circuit(L, q, n, seed, reads=None):
    """Every kind of gate call the capture path handles; `reads` (a list) gets
    a reduction in the middle, which must flush the queue."""
    lib = L.lib
    rng = np.random.default_rng(seed)
    for layer in range(3):
        for t in range(n):
            a, b = rng.normal(size=2) + 1j * rng.normal(size=2)
            s = np.sqrt(abs(a) ** 2 + abs(b) ** 2)
            lib.compactUnitary(q, t, Complex(a.real / s, a.imag / s), Complex(b.real / s, b.imag / s))
        for t in range(0, n - 1, 2):
            lib.controlledNot(q, t + layer % 2, t + 1 - layer % 2)
        lib.hadamard(q, 1)
        lib.pauliY(q, 2)
        lib.sGate(q, 3)
        lib.tGate(q, 4)
        lib.phaseShift(q, 5, 0.3)
        lib.rotateX(q, 6, 0.7)
        lib.rotateY(q, 7, -0.4)
        lib.rotateZ(q, 8, 1.1)
        lib.rotateAroundAxis(q, 9, 0.5, Vector(1, 2, 3))
        lib.controlledPhaseShift(q, 0, n - 1, 0.9)
        lib.controlledPhaseFlip(q, 2, 7)
        lib.controlledRotateY(q, 3, 11, 0.6)
        lib.controlledPauliY(q, 12, 1)
        lib.swapGate(q, 0, n - 2)
        lib.sqrtSwapGate(q, 4, 10)
        L.multiControlledPhaseFlip(q, [1, 5, 9])
        L.multiRotateZ(q, [2, 6, 13], 0.8)
        L.multiRotatePauli(q, [0, 3, 8], [1, 2, 3], 0.45)
        L.multiControlledMultiQubitNot(q, [4], [6, 12])
        u4 = haar(rng, 2)
        m4 = ComplexMatrix4()
        for r in range(4):
            for c in range(4):
                m4.real[r][c] = u4[r, c].real
                m4.imag[r][c] = u4[r, c].imag
        lib.twoQubitUnitary(q, 5, 14, m4)
        L.multiQubitUnitary(q, [1, 6, 11, 13], haar(rng, 4))
        u2 = haar(rng, 1)
        m2 = ComplexMatrix2()
        for r in range(2):
            for c in range(2):
                m2.real[r][c] = u2[r, c].real
                m2.imag[r][c] = u2[r, c].imag
        lib.controlledUnitary(q, 9, 3, m2)
        if reads is not None and layer == 1:
            reads.append(lib.calcProbOfOutcome(q, 3, 1))


@pytest.mark.parametrize("n", [15, 20])
def test_capture_matches_direct_fp64(gpulib, n):
    L = gpulib
    lib = L.lib
    direct = L.create(n)
    lib.initZeroState(direct)
    reads_d = []
    mixed_circuit(L, direct, n, 7, reads_d)
    cap = L.create(n)
    assert lib.quest_gb300_setCapture(cap, 1) == 0
    lib.initZeroState(cap)
    reads_c = []
    mixed_circuit(L, cap, n, 7, reads_c)
    queued = lib.quest_gb300_capturedGates(cap)
    assert queued >= n + 20                             # the last layer is still queued
    a, b = L.amps(direct), L.amps(cap)                  # amps() flushes (copyStateFromGPU)
    assert lib.quest_gb300_capturedGates(cap) == 0
    f = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    print(f"n={n}: queued {queued}, 1-F={1 - f:.2e}, max|d|={np.max(np.abs(a - b)):.2e}")
    assert 1 - f <= 1e-6 and np.max(np.abs(a - b)) <= 1e-5
    assert abs(reads_c[0] - reads_d[0]) < 1e-6         # mid-circuit read saw the flushed state
    L.destroy(direct)
    L.destroy(cap)


def test_capture_matches_oracle(gpulib, oracle):
    """Captured calls against the CPU oracle directly: the mixed circuit at
    16 qubits (every captured gate kind, a mid-circuit read), then a noisy
    7-qubit density matrix (gates and the three channels as superoperators)."""
    L = gpulib
    n = 16
    ref = oracle.create(n)
    oracle.lib.initZeroState(ref)
    reads_o = []
    mixed_circuit(oracle, ref, n, 9, reads_o)
    cap = L.create(n)
    assert L.lib.quest_gb300_setCapture(cap, 1) == 0
    L.lib.initZeroState(cap)
    reads_c = []
    mixed_circuit(L, cap, n, 9, reads_c)
    a, b = oracle.amps(ref), L.amps(cap)
    f = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    print(f"SV n={n} vs oracle: 1-F={1 - f:.2e}, max|d|={np.max(np.abs(a - b)):.2e}")
    assert 1 - f <= 1e-6 and np.max(np.abs(a - b)) <= 1e-5
    assert abs(reads_o[0] - reads_c[0]) < 1e-6
    oracle.destroy(ref)
    L.destroy(cap)

    n = 7
    ops = W.c3_circuit(nq=n, layers=2, seed=6)
    ref = oracle.create(n, density=True)
    oracle.lib.initZeroState(ref)
    W.run_ops(oracle, ref, ops)
    cap = L.create(n, density=True)
    L.lib.quest_gb300_setCapture(cap, 1)
    L.lib.initZeroState(cap)
    W.run_ops(L, cap, ops)
    a, b = oracle.amps(ref), L.amps(cap)
    po, pc = oracle.lib.calcPurity(ref), L.lib.calcPurity(cap)
    print(f"DM n={n} vs oracle: max|d rho|={np.max(np.abs(a - b)):.2e}, purity rel. diff {abs(pc / po - 1):.2e}")
    assert np.max(np.abs(a - b)) <= 1e-5 and abs(pc / po - 1) < 1e-6
    assert abs(L.lib.calcTotalProb(cap) - oracle.lib.calcTotalProb(ref)) < 1e-9
    oracle.destroy(ref)
    L.destroy(cap)


def test_capture_density_matrix_and_channels(gpulib):
    """Density matrix: gates are doubled (U on t, conj U on t + N) and queued;
    dephasing, depolarising and damping are queued too, as their 4 x 4
    superoperators on (t, t + N), and fused with the gates."""
    L = gpulib
    lib = L.lib
    n = 7
    ops = W.c3_circuit(nq=n, layers=2, seed=4)
    channels = sum(1 for op in ops if op[0] in ("deph", "depol", "damp"))
    direct = L.create(n, density=True)
    cap = L.create(n, density=True)
    lib.quest_gb300_setCapture(cap, 1)
    for q in (direct, cap):
        lib.initZeroState(q)
        W.run_ops(L, q, ops)
    assert lib.quest_gb300_capturedGates(cap) > channels      # nothing flushed the queue
    a, b = L.amps(direct), L.amps(cap)
    assert np.max(np.abs(a - b)) <= 1e-5
    # the flush restores the trace the plan started from (the FP32
    # accumulation's bias is a near-uniform shrink), which also keeps purity
    assert abs(lib.calcTotalProb(cap) - 1) < 1e-9
    pd, pc = lib.calcPurity(direct), lib.calcPurity(cap)
    print(f"DM 7 qubits: max|d rho| {np.max(np.abs(a - b)):.2e}, purity rel. diff {abs(pc / pd - 1):.2e}")
    assert abs(pc / pd - 1) < 1e-6
    L.destroy(direct)
    L.destroy(cap)


def test_capture_pauli_and_two_qubit_channels(gpulib):
    """mixPauli (a 4 x 4 superoperator on (t, t + N)) and the two-qubit
    dephasing and depolarising channels (16 x 16 on (q1, q2, q1 + N, q2 + N))
    are queued like the one-qubit channels and fused with the gates."""
    L = gpulib
    lib = L.lib
    n = 6
    rng = np.random.default_rng(9)
    direct = L.create(n, density=True)
    cap = L.create(n, density=True)
    lib.quest_gb300_setCapture(cap, 1)
    for q in (direct, cap):
        lib.initZeroState(q)
    for layer in range(3):
        angles = rng.uniform(0, 2 * np.pi, size=n)
        probs = rng.uniform(0, 0.1, size=(n, 5))
        for q in (direct, cap):
            for t in range(n):
                lib.rotateY(q, t, angles[t])
            for t in range(layer % 2, n - 1, 2):
                lib.controlledNot(q, t, t + 1)
            for t in range(n):
                lib.mixPauli(q, t, probs[t, 0], probs[t, 1], probs[t, 2])
                lib.mixTwoQubitDephasing(q, t, (t + 2) % n, probs[t, 3])
                lib.mixTwoQubitDepolarising(q, (t + 3) % n, t, probs[t, 4])
    assert lib.quest_gb300_capturedGates(cap) > 3 * n * 3
    a, b = L.amps(direct), L.amps(cap)
    assert np.max(np.abs(a - b)) <= 1e-5
    assert abs(lib.calcTotalProb(cap) - 1) < 1e-9
    assert abs(lib.calcPurity(cap) / lib.calcPurity(direct) - 1) < 1e-6
    L.destroy(direct)
    L.destroy(cap)


def test_capture_drops_queue_on_overwrite_and_off_flushes(gpulib):
    L = gpulib
    lib = L.lib
    n = 12
    q = L.create(n)
    lib.quest_gb300_setCapture(q, 1)
    lib.initZeroState(q)
    for t in range(n):
        lib.hadamard(q, t)
    assert lib.quest_gb300_capturedGates(q) == n
    lib.initZeroState(q)                                # overwrite: queue dropped
    assert lib.quest_gb300_capturedGates(q) == 0
    assert abs(lib.getRealAmp(q, 0) - 1) < 1e-12
    lib.pauliX(q, 3)
    assert lib.quest_gb300_capturedGates(q) == 1
    lib.quest_gb300_setCapture(q, 0)                    # off: flushes
    assert lib.quest_gb300_capturedGates(q) == 0
    assert abs(lib.getRealAmp(q, 1 << 3) - 1) < 1e-6
    lib.pauliX(q, 3)                                    # runs directly now
    assert abs(lib.getRealAmp(q, 0) - 1) < 1e-6
    L.destroy(q)


def test_capture_speeds_up_a_26_qubit_circuit(gpulib):
    """The 26-qubit random circuit through the QuEST API: captured (one fused
    FP32 flush; plans of 26 qubits and more take control qubits) against
    direct FP64 per-gate calls, in time and in the state."""
    L = gpulib
    lib = L.lib
    n = 26
    ops = W.c2_circuit(n=n, layers=10, seed=2)
    res = {}
    states = {}
    for mode in (0, 1):
        q = L.create(n)
        lib.quest_gb300_setCapture(q, mode)
        lib.initZeroState(q)
        W.run_ops(L, q, ops)
        lib.calcTotalProb(q)                            # warm-up (plan upload, FP32 scratch)
        lib.initZeroState(q)
        lib.quest_gb300_eventRecord(20)
        W.run_ops(L, q, ops)
        p = lib.calcTotalProb(q)
        lib.quest_gb300_eventRecord(21)
        res[mode] = (lib.quest_gb300_eventElapsedMs(20, 21), p)
        states[mode] = L.amps(q).copy()
        L.destroy(q)
    a, b = states[0], states[1]
    f = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    err = float(np.max(np.abs(a - b)))
    print(f"26q 10 layers: direct {res[0][0]:.1f} ms, captured {res[1][0]:.1f} ms, 1-F {1 - f:.2e}, max|d| {err:.2e}")
    assert abs(res[1][1] - 1) < 1e-5
    assert 1 - f <= 1e-6 and err <= 1e-5
    assert res[1][0] < res[0][0] / 3


def test_capture_takes_the_background_search(gpulib):
    """A new circuit shape is planned without lookahead; on registers of 26
    qubits a host thread then searches it again with lookahead, and a later
    flush of the same shape takes those passes when fewer: the second flush
    of the 26-qubit circuit uses no more passes than the first and gives the
    same state to FP32 precision."""
    import time
    L = gpulib
    lib = L.lib
    n = 26
    ops = W.c2_circuit(n=n, layers=12, seed=9)
    q = L.create(n)
    assert lib.quest_gb300_setCapture(q, 1) == 0
    f, g, p, ms = C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_double()
    passes, states = [], []
    for _ in range(2):
        lib.initZeroState(q)
        W.run_ops(L, q, ops)
        lib.calcTotalProb(q)
        states.append(L.amps(q).copy())
        assert lib.quest_gb300_captureStats(q, C.byref(f), C.byref(g), C.byref(p), C.byref(ms)) == 0
        passes.append(p.value - sum(passes))
        time.sleep(1.0)                                # the background search ends
    lib.quest_gb300_setCapture(q, 0)
    L.destroy(q)
    print(f"26q: passes {passes[0]} then {passes[1]}")
    assert passes[1] <= passes[0]
    assert np.max(np.abs(states[0] - states[1])) < 1e-6


def test_capture_density_matrix_with_control_qubits(gpulib):
    """A 13-qubit noisy density matrix (a 26-qubit vector, so its plans take
    control qubits): gates doubled on (t, t + N), the three channels as
    superoperators, captured against direct FP64 calls."""
    L = gpulib
    lib = L.lib
    n = 13
    ops = W.c3_circuit(nq=n, layers=2, seed=8)
    out = {}
    for mode in (0, 1):
        q = L.create(n, density=True)
        lib.quest_gb300_setCapture(q, mode)
        lib.initZeroState(q)
        W.run_ops(L, q, ops)
        out[mode] = (L.amps(q).copy(), lib.calcTotalProb(q), lib.calcPurity(q))
        L.destroy(q)
    (a, ta, pa), (b, tb, pb) = out[0], out[1]
    err = float(np.max(np.abs(a - b)))
    print(f"DM 13 qubits: max|d rho| {err:.2e}, trace {tb - ta:.1e}, purity rel. diff {abs(pb / pa - 1):.2e}")
    assert err <= 1e-5 and abs(tb - ta) < 1e-9 and abs(pb / pa - 1) < 1e-6


@pytest.mark.parametrize("n", [3, 5, 8, 11, 12, 13])
def test_capture_small_registers(gpulib, n):
    """Registers below and at the 13-qubit size from which 6-qubit passes are
    possible: random 1-, 2- and multi-qubit gates (some as wide as the
    register or six qubits) queued and fused must match direct FP64 calls."""
    L = gpulib
    lib = L.lib

    def circuit(q):
        r = np.random.default_rng(7 * n)
        for _ in range(12 * n):
            kind = r.integers(5)
            if kind == 0:
                t = int(r.integers(n))
                a, b = r.normal(size=2) + 1j * r.normal(size=2)
                s = np.sqrt(abs(a) ** 2 + abs(b) ** 2)
                lib.compactUnitary(q, t, Complex(a.real / s, a.imag / s), Complex(b.real / s, b.imag / s))
            elif kind == 1 and n > 1:
                c, t = (int(x) for x in r.choice(n, size=2, replace=False))
                lib.controlledNot(q, c, t)
            elif kind == 2 and n > 1:
                a, b = (int(x) for x in r.choice(n, size=2, replace=False))
                lib.controlledPhaseShift(q, a, b, float(r.uniform(0, 2 * np.pi)))
            elif kind == 3:
                k = int(r.integers(1, min(n, 6) + 1))
                ts = [int(x) for x in r.choice(n, size=k, replace=False)]
                L.multiQubitUnitary(q, ts, haar(r, k))
            else:
                k = int(r.integers(1, min(n, 4) + 1))
                ts = [int(x) for x in r.choice(n, size=k, replace=False)]
                L.multiRotateZ(q, ts, float(r.uniform(0, 2 * np.pi)))

    direct = L.create(n)
    lib.initZeroState(direct)
    circuit(direct)
    cap = L.create(n)
    lib.quest_gb300_setCapture(cap, 1)
    lib.initZeroState(cap)
    circuit(cap)
    a, b = L.amps(direct), L.amps(cap)
    f = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    print(f"n={n}: 1-F={1 - f:.2e}, max|d|={np.max(np.abs(a - b)):.2e}")
    assert 1 - f <= 1e-6 and np.max(np.abs(a - b)) <= 1e-5
    assert abs(lib.calcTotalProb(cap) - 1) < 1e-6
    L.destroy(direct)
    L.destroy(cap)


def test_capture_stats_count_the_flushes(gpulib):
    """quest_gb300_captureStats: -1 with capture off; after three flushes of
    a queued circuit, the flush and gate totals, at least one fused pass per
    flush and a non-negative planning time.  The later flushes take the
    first one's passes (same circuit shape): the same state."""
    L = gpulib
    lib = L.lib
    n = 14
    q = L.create(n)
    f, g, p, ms = C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_double()
    assert lib.quest_gb300_captureStats(q, C.byref(f), C.byref(g), C.byref(p), C.byref(ms)) == -1
    assert lib.quest_gb300_setCapture(q, 1) == 0
    ops = W.c2_circuit(n=n, layers=2, seed=4)
    queued = 0
    states = []
    for _ in range(3):
        lib.initZeroState(q)
        W.run_ops(L, q, ops)
        queued += lib.quest_gb300_capturedGates(q)
        lib.calcTotalProb(q)
        states.append(L.amps(q).copy())
    assert np.max(np.abs(states[0] - states[1])) < 1e-6 and np.max(np.abs(states[1] - states[2])) < 1e-6
    assert lib.quest_gb300_captureStats(q, C.byref(f), C.byref(g), C.byref(p), C.byref(ms)) == 0
    assert f.value == 3 and g.value == queued == 3 * len(ops)
    assert 2 <= p.value <= g.value and ms.value >= 0.0
    lib.quest_gb300_setCapture(q, 0)
    L.destroy(q)


def test_capture_split_fp16_takes_any_norm(gpulib):
    """With split-FP16 operands a flush's FP64 -> FP32 conversion also sums
    |x|^2, and the first tensor-core pass takes its operand scale from that
    sum (later passes from the previous pass's): a state of norm ~40 with an
    amplitude of 5 (beyond the fixed scale's 3.99) and one of norm 1e-4 both
    match the same calls run directly in FP64."""
    L = gpulib
    lib = L.lib
    n = 15
    before = lib.quest_gb300_getTensorCorePrecision()
    assert lib.quest_gb300_setTensorCorePrecision(2) == 0
    try:
        for scale in (40.0, 1e-4):
            rng = np.random.default_rng(5)
            psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
            psi *= scale / np.linalg.norm(psi)
            if scale > 1:
                psi[7] = 5.0
            direct = L.create(n)
            L.set_amps(direct, psi)
            mixed_circuit(L, direct, n, 3)
            cap = L.create(n)
            assert lib.quest_gb300_setCapture(cap, 1) == 0
            L.set_amps(cap, psi)
            mixed_circuit(L, cap, n, 3)
            assert lib.quest_gb300_capturedGates(cap) > 0
            a, b = L.amps(direct), L.amps(cap)
            f = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
            err = float(np.max(np.abs(a - b)))
            print(f"norm {np.linalg.norm(psi):.3g}: 1-F={1 - f:.2e}, max|d|={err:.2e} (max|amp| {np.abs(a).max():.3g})")
            assert 1 - f <= 1e-9 and err <= 1e-6 * np.abs(a).max()
            L.destroy(direct)
            L.destroy(cap)
    finally:
        lib.quest_gb300_setTensorCorePrecision(before)
