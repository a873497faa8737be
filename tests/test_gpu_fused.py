"""FP32 fused engine against the FP64 plain engine (GPU).

Tolerances: 1 - fidelity <= 1e-6 (the fused path's stated bound) and
max |d amp| <= 1e-5; observed errors are printed."""
import ctypes as C

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def no_library_errors(gpulib):
    """Every error the library reports through invalidQuESTInputError fails
    the test (instead of the default handler's exit)."""
    gpulib.capture_errors()
    gpulib.errors.clear()
    yield
    errors = list(gpulib.errors)
    gpulib.errors.clear()
    assert not errors, errors


def run_both(L, n, kmax, ops):
    q64 = L.create(n)
    W.run_ops(L, q64, ops)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    plan = L.plan(n, kmax, ops)
    assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
    err = C.c_double(0)
    one_minus_f = L.lib.quest_gb300_compareF32(q32, q64, C.byref(err))
    return q64, q32, plan, one_minus_f, err.value


@pytest.mark.parametrize("kmax", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [7, 16, 22])
def test_fused_matches_plain(gpulib, n, kmax):
    L = gpulib
    L.lib.quest_gb300_setTensorCores(0)
    ops = W.c2_circuit(n=n, layers=6, seed=21 + n)
    if kmax == 1:
        ops = [o for o in ops if o[0] == "cu"]
    q64, q32, plan, omf, err = run_both(L, n, kmax, ops)
    L.lib.quest_gb300_setTensorCores(1)
    print(f"n={n} k={kmax}: 1-F={omf:.2e} max|d amp|={err:.2e}")
    assert omf <= 1e-6 and err <= 1e-5
    p32 = L.lib.quest_gb300_calcTotalProbF32(q32)
    assert abs(p32 - 1) < 1e-5
    for t in (0, n // 2, n - 1):
        assert abs(L.lib.quest_gb300_calcProbOfOutcomeF32(q32, t, 1) - L.lib.calcProbOfOutcome(q64, t, 1)) < 1e-6
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


def test_fused_host_roundtrip(gpulib):
    L = gpulib
    n = 12
    rng = np.random.default_rng(5)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    re, im = np.ascontiguousarray(psi.real), np.ascontiguousarray(psi.imag)
    L.lib.quest_gb300_initStateFromAmpsF32(q32, re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)))
    back = L.amps_f32(q32, n)
    assert np.max(np.abs(back - psi)) < 1e-7
    q64 = L.create(n)
    L.set_amps(q64, psi)
    L.lib.quest_gb300_copyToQureg(q32, q64)
    assert np.max(np.abs(L.amps(q64) - back)) == 0
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


@pytest.mark.parametrize("kmax", [4, 5, 6])
@pytest.mark.parametrize("n", [13, 18])
def test_tensor_core_applier(gpulib, n, kmax):
    """tcgen05 split-TF32 passes (k = 4..6) against the FP64 plain engine and
    against the FP32 SIMT applier."""
    L = gpulib
    ops = W.c2_circuit(n=n, layers=4, seed=31 + n)
    L.lib.quest_gb300_setTensorCores(1)
    q64, q32, plan, omf, err = run_both(L, n, kmax, ops)
    print(f"TC n={n} k={kmax}: 1-F={omf:.2e} max|d amp|={err:.2e}")
    assert omf <= 1e-6 and err <= 1e-5
    if kmax <= 5:
        L.lib.quest_gb300_setTensorCores(0)
        s32 = L.lib.quest_gb300_createQuregF32(n)
        assert L.lib.quest_gb300_applyPlanF32(s32, plan) == 0
        L.lib.quest_gb300_setTensorCores(1)
        a, b = L.amps_f32(q32, n), L.amps_f32(s32, n)
        assert np.max(np.abs(a - b)) < 1e-5
        L.lib.quest_gb300_destroyQuregF32(s32)
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


def _single_gate_plan(L, n, targets, seed):
    rng = np.random.default_rng(seed)
    k = len(targets)
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    u, _ = np.linalg.qr(z)
    p = L.lib.quest_gb300_planCreate(n, k)
    re, im = np.ascontiguousarray(u.real.ravel()), np.ascontiguousarray(u.imag.ravel())
    ts = (C.c_int * k)(*targets)
    assert L.lib.quest_gb300_planAddGate(p, ts, k, re.ctypes.data_as(C.POINTER(C.c_double)),
                                         im.ctypes.data_as(C.POINTER(C.c_double))) == 0
    L.lib.quest_gb300_planCompile(p)
    return p, u


@pytest.fixture(params=[0, 1, 2], ids=["tf32", "bf16", "fp16"])
def precision(request, gpulib):
    """Operands of the pipelined kernel: 0 = 3-term split-TF32 (default),
    1 = 4-term split-BF16, 2 = 3-term split-FP16."""
    assert gpulib.lib.quest_gb300_setTensorCorePrecision(request.param) == 0
    yield request.param
    gpulib.lib.quest_gb300_setTensorCorePrecision(0)


@pytest.mark.parametrize("targets", [[0, 1, 2, 3], [0, 2, 4, 6, 8], [0, 1, 2, 3, 4, 5], [1, 3, 5, 7, 9, 11],
                                     [2, 9, 10, 14], [4, 5, 6, 7, 15, 16], [12, 13, 14, 15, 16, 17],
                                     [0, 1, 9, 17], [0, 1, 7, 12, 13], [0, 1, 5, 9, 13, 17],
                                     [0, 5, 9, 12], [0, 3, 8, 9, 15, 17]])
@pytest.mark.parametrize("version", [0, 1, 2, 3, 4, 5])
def test_tensor_core_target_layouts(gpulib, targets, version, precision):
    """One dense gate on low, interleaved and high target sets (with qubit 0,
    or qubits 0 and 1, among the targets, the pipelined kernel reads and
    writes columns as 8- or 16-byte words), every tensor-core kernel (direct-load; pipelined with 2+1, 1+1, 1+2 loader +
    epilogue warp groups, and 2+2 with the loaders splitting each chunk),
    against the FP64 engine."""
    L = gpulib
    n = 18
    rng = np.random.default_rng(3)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    q64 = L.create(n)
    L.set_amps(q64, psi)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_copyFromQureg(q32, q64)
    plan, u = _single_gate_plan(L, n, targets, 11)
    L.lib.quest_gb300_setTensorCoreKernel(version)
    assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
    L.lib.quest_gb300_setTensorCoreKernel(0)
    L.multiQubitUnitary(q64, targets, u)
    err = C.c_double(0)
    omf = L.lib.quest_gb300_compareF32(q32, q64, C.byref(err))
    print(f"TC v{version} prec={precision} targets={targets}: 1-F={omf:.2e} max|d amp|={err.value:.2e}")
    assert omf < 1e-9 and err.value < 1e-5
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


@pytest.mark.parametrize("version", [0, 2, 3, 4, 5])
def test_bulk_staging_is_bit_identical(gpulib, version, precision):
    """The pipelined kernels' TMA bulk staging (one 128-byte row per copy)
    gives the same FP32 state, bit for bit, as 16-byte cp.async staging: a
    random circuit at 18 qubits with passes of 4 to 6 qubits (qubits 0 and 1
    among the targets of some), every pipelined variant."""
    L = gpulib
    n = 18
    ops = W.c2_circuit(n=n, layers=6, seed=5)
    plan = L.plan(n, 6, ops)
    ks = [L.lib.quest_gb300_planPass(plan, i, None, None, None) for i in range(L.lib.quest_gb300_planCompile(plan))]
    assert max(ks) == 6 and min(ks) <= 5
    states = []
    L.lib.quest_gb300_setTensorCoreKernel(version)
    for staging in (0, 1):
        assert L.lib.quest_gb300_setTensorCoreStaging(staging) == 0
        assert L.lib.quest_gb300_getTensorCoreStaging() == staging
        q32 = L.lib.quest_gb300_createQuregF32(n)
        assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
        states.append(L.amps_f32(q32, n))
        L.lib.quest_gb300_destroyQuregF32(q32)
    L.lib.quest_gb300_setTensorCoreStaging(0)
    L.lib.quest_gb300_setTensorCoreKernel(0)
    assert L.lib.quest_gb300_setTensorCoreStaging(2) == -1
    L.lib.quest_gb300_planDestroy(plan)
    assert np.array_equal(states[0], states[1])
    assert abs(np.vdot(states[1], states[1]).real - 1) < 1e-5


@pytest.mark.parametrize("version", [0, 1, 3, 4, 5])
def test_non_unitary_passes_keep_their_norm(gpulib, version, precision):
    """A plan mixing non-unitary and unitary dense gates on the tensor cores:
    the drift correction must not undo a pass that changes the norm on
    purpose (only unitary passes are corrected)."""
    L = gpulib
    n = 18
    rng = np.random.default_rng(8)
    gates = []
    for i, ts in enumerate([[0, 3, 5, 9, 12], [1, 2, 6, 7, 8, 13], [4, 10, 11, 14, 15, 16], [0, 1, 2, 3, 17]]):
        k = len(ts)
        z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        m = np.linalg.qr(z)[0] if i % 2 else 0.3 * z / np.sqrt(1 << k)
        gates.append((ts, m))
    p = L.lib.quest_gb300_planCreate(n, 6)
    for ts, m in gates:
        re, im = np.ascontiguousarray(m.real.ravel()), np.ascontiguousarray(m.imag.ravel())
        assert L.lib.quest_gb300_planAddGate(p, (C.c_int * len(ts))(*ts), len(ts),
                                             re.ctypes.data_as(C.POINTER(C.c_double)),
                                             im.ctypes.data_as(C.POINTER(C.c_double))) == 0
    assert L.lib.quest_gb300_planCompile(p) == 4
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    q64 = L.create(n)
    L.set_amps(q64, psi)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_copyFromQureg(q32, q64)
    L.lib.quest_gb300_setTensorCoreKernel(version)
    assert L.lib.quest_gb300_applyPlanF32(q32, p) == 0
    L.lib.quest_gb300_setTensorCoreKernel(0)
    for ts, m in gates:
        L.applyMatrixN(q64, ts, m)
    err = C.c_double(0)
    omf = L.lib.quest_gb300_compareF32(q32, q64, C.byref(err))
    p64 = L.lib.calcTotalProb(q64)
    p32 = L.lib.quest_gb300_calcTotalProbF32(q32)
    print(f"non-unitary v{version}: norm {p64:.6e} vs {p32:.6e}, 1-F={omf:.2e}")
    assert abs(p32 / p64 - 1) < 1e-5 and omf < 1e-9
    L.lib.quest_gb300_planDestroy(p)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


@pytest.mark.parametrize("kmax,version", [(6, 0), (6, 1), (6, 2), (6, 3), (6, 4), (6, 5), (5, 0), (4, 0)])
def test_controlled_passes_match_oracle(gpulib, oracle, kmax, version, precision):
    """Passes with control qubits (up to three, the matrix chosen per control
    value; the CTAs of a launch split over the control values) on every
    pipelined kernel variant (1, the direct-load kernel, takes none and maps
    to 5): the random circuit at 20 qubits against the oracle's FP64 state."""
    L = gpulib
    n = 20
    ops = W.c2_circuit(n=n, layers=8, seed=13)
    qo = oracle.create(n)
    W.run_ops(oracle, qo, ops)
    ref = oracle.amps(qo).copy()
    oracle.destroy(qo)
    plan = L.plan(n, kmax, ops, controls=3)
    npass = L.lib.quest_gb300_planCompile(plan)
    ctl = sum(L.lib.quest_gb300_planPassControls(plan, i, None) > 0 for i in range(npass))
    assert ctl > 0
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_setTensorCoreKernel(version)
    rc = L.lib.quest_gb300_applyPlanF32(q32, plan)
    L.lib.quest_gb300_setTensorCoreKernel(0)
    assert rc == 0
    got = L.amps_f32(q32, n)
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    omf = 1 - abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    err = float(np.max(np.abs(got - ref)))
    print(f"k={kmax} v{version} prec={precision}: {npass} passes ({ctl} controlled) 1-F={omf:.2e} max|d amp|={err:.2e}")
    assert omf <= 1e-6 and err <= 1e-5


def test_controlled_pass_needs_the_tensor_cores(gpulib):
    """A plan compiled with control qubits refuses the SIMT applier (tensor
    cores switched off after compiling) with an input error."""
    L = gpulib
    n = 20
    plan = L.plan(n, 5, W.c2_circuit(n=n, layers=4, seed=3), controls=3)      # k <= 5: the SIMT applier takes the rest
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_setTensorCores(0)
    rc = L.lib.quest_gb300_applyPlanF32(q32, plan)
    L.lib.quest_gb300_setTensorCores(1)
    errors = list(L.errors)
    L.errors.clear()
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    assert rc == -1 and any("control qubits" in e[1] for e in errors), errors


@pytest.mark.parametrize("kmax", [4, 5, 6])
def test_fused_matches_oracle(gpulib, oracle, kmax, precision):
    """The fused FP32 engine against the CPU oracle directly (not through
    the plain GPU engine): the random circuit at 20 qubits, 10 layers, from
    |0..0>; 1 - F and max |d amp| against the oracle's FP64 state."""
    L = gpulib
    n = 20
    ops = W.c2_circuit(n=n, layers=10, seed=17)
    qo = oracle.create(n)
    W.run_ops(oracle, qo, ops)
    ref = oracle.amps(qo).copy()
    oracle.destroy(qo)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    plan = L.plan(n, kmax, ops)
    assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
    got = L.amps_f32(q32, n)
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    ov = np.vdot(ref, got)
    omf = 1 - abs(ov) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    err = float(np.max(np.abs(got - ref)))
    print(f"n={n} k={kmax} prec={precision} vs oracle: 1-F={omf:.2e} max|d amp|={err:.2e}")
    assert omf <= 1e-6 and err <= 1e-5


@pytest.mark.parametrize("kmax", [4, 6])
def test_fused_30q_headline_accuracy(gpulib, kmax, precision):
    """The 30-qubit, 20-layer circuit: fused FP32 vs plain FP64."""
    L = gpulib
    ops = W.c2_circuit(n=30, layers=20, seed=2)
    q64, q32, plan, omf, err = run_both(L, 30, kmax, ops)
    norm = L.lib.quest_gb300_calcTotalProbF32(q32)
    print(f"30q k={kmax} prec={precision}: 1-F={omf:.3e} max|d amp|={err:.3e} norm-1={norm - 1:.2e}")
    assert omf <= 1e-6 and abs(norm - 1) < 1e-5
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


def test_autotuned_plan_matches_and_predicts(gpulib, tmp_path, monkeypatch):
    """planCompileTuned picks a width in [4, 6], the tuned plan is still the
    circuit, and its predicted time is positive."""
    L = gpulib
    monkeypatch.setenv("QUEST_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    n = 16
    ops = W.c2_circuit(n=n, layers=4, seed=77)
    p = L.plan(n, 4, ops)
    k = L.lib.quest_gb300_planCompileTuned(p, 4, 6)
    assert 4 <= k <= 6
    assert L.lib.quest_gb300_planPredictMs(p) > 0
    q32 = L.lib.quest_gb300_createQuregF32(n)
    assert L.lib.quest_gb300_applyPlanF32(q32, p) == 0
    q64 = L.create(n)
    W.run_ops(L, q64, ops)
    omf = L.lib.quest_gb300_compareF32(q32, q64, None)
    assert omf < 1e-9
    L.lib.quest_gb300_planDestroy(p)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


def test_autotune_picks_kernel_variants(gpulib, tmp_path, monkeypatch):
    """autotune times every pipelined variant of each tensor-core pass class
    and keeps the fastest; the plan gives the same state with the tuned
    variants and with the fixed defaults; the cache records the choices."""
    L = gpulib
    lib = L.lib
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("QUEST_GB300_TUNE_CACHE", str(cache))
    n = 17
    assert lib.quest_gb300_autotune(n) == 0
    ms = C.c_double(0)
    for k in (4, 5, 6):
        for layout in (0, 1, 2):
            v = lib.quest_gb300_tunedKernel(n, k, layout, C.byref(ms))
            assert 2 <= v <= 5 and ms.value > 0, (k, layout, v)
    text = cache.read_text()
    assert f'"n{n}_p0_k6_l2_v"' in text or f'"n{n}_p1_k6_l2_v"' in text
    ops = W.c2_circuit(n=n, layers=6, seed=5)
    p = L.plan(n, 6, ops)
    states = []
    for tuning in (1, 0):
        lib.quest_gb300_setKernelTuning(tuning)
        q32 = lib.quest_gb300_createQuregF32(n)
        assert lib.quest_gb300_applyPlanF32(q32, p) == 0
        states.append(L.amps_f32(q32, n))
        lib.quest_gb300_destroyQuregF32(q32)
    lib.quest_gb300_setKernelTuning(1)
    a, b = states
    assert np.max(np.abs(a - b)) < 1e-5
    lib.quest_gb300_planDestroy(p)


def test_capture_with_autotuned_width(gpulib, tmp_path, monkeypatch):
    """setCaptureFusion(0): each searched flush plan takes the width the
    autotuner predicts fastest; the result matches the direct FP64 calls."""
    L = gpulib
    lib = L.lib
    monkeypatch.setenv("QUEST_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    n = 16
    ops = W.c2_circuit(n=n, layers=5, seed=21)
    direct, cap = L.create(n), L.create(n)
    lib.quest_gb300_setCaptureFusion(0)
    try:
        lib.quest_gb300_setCapture(cap, 1)
        for q in (direct, cap):
            lib.initZeroState(q)
            W.run_ops(L, q, ops)
        a, b = L.amps(direct), L.amps(cap)
    finally:
        lib.quest_gb300_setCaptureFusion(6)
    f = abs(np.vdot(a, b)) ** 2
    assert 1 - f <= 1e-6 and np.max(np.abs(a - b)) <= 1e-5
    L.destroy(direct)
    L.destroy(cap)


def test_pass_events_time_every_pass(gpulib):
    """setPassEvents(1): applyPlanF32 records an event pair around each pass;
    passTimesMs returns one positive duration per pass of the last
    application, summing to no more than the whole application."""
    L = gpulib
    lib = L.lib
    n = 18
    p = L.plan(n, 6, W.c2_circuit(n=n, layers=4, seed=3))
    npass = lib.quest_gb300_planCompile(p)
    q32 = lib.quest_gb300_createQuregF32(n)
    lib.quest_gb300_applyPlanF32(q32, p)                      # warm-up (upload)
    lib.quest_gb300_setPassEvents(1)
    try:
        lib.quest_gb300_eventRecord(40)
        assert lib.quest_gb300_applyPlanF32(q32, p) == 0
        lib.quest_gb300_eventRecord(41)
        whole = lib.quest_gb300_eventElapsedMs(40, 41)
        out = (C.c_double * npass)()
        assert lib.quest_gb300_passTimesMs(out, npass) == npass
        times = list(out)
        assert all(t > 0 for t in times) and sum(times) <= whole * 1.01
    finally:
        lib.quest_gb300_setPassEvents(0)
    lib.quest_gb300_destroyQuregF32(q32)
    lib.quest_gb300_planDestroy(p)


@pytest.fixture
def split_fp16(gpulib):
    assert gpulib.lib.quest_gb300_setTensorCorePrecision(2) == 0
    assert gpulib.lib.quest_gb300_getTensorCorePrecision() == 2
    yield
    gpulib.lib.quest_gb300_setTensorCorePrecision(0)


def _dense_plan(L, n, gates):
    p = L.lib.quest_gb300_planCreate(n, 6)
    for ts, m in gates:
        re, im = np.ascontiguousarray(m.real.ravel()), np.ascontiguousarray(m.imag.ravel())
        assert L.lib.quest_gb300_planAddGate(p, (C.c_int * len(ts))(*ts), len(ts),
                                             re.ctypes.data_as(C.POINTER(C.c_double)),
                                             im.ctypes.data_as(C.POINTER(C.c_double))) == 0
    assert L.lib.quest_gb300_planCompile(p) == len(gates)
    return p


@pytest.mark.parametrize("version", [0, 2, 5])
def test_split_fp16_scales_each_matrix_block(gpulib, split_fp16, version):
    """Split-FP16 with matrices far from unit size: a 5-qubit matrix of
    entries up to ~30 (60 x a unitary), then 6-qubit ones scaled by 1/60,
    1e-3 and 1e3, on a normalised 18-qubit state (the state's norm goes 60,
    1, 1e-3, 1).  Each operand block carries its own power-of-two scale, so
    every pass keeps FP16's 11-bit precision: the result matches the FP64
    engine as closely as unit-size passes do."""
    L = gpulib
    n = 18
    rng = np.random.default_rng(23)

    def haar(k):
        return np.linalg.qr(rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k)))[0]

    gates = [([0, 4, 7, 11, 16], 60.0 * haar(5)), ([1, 2, 3, 5, 6, 8], haar(6) / 60.0),
             ([9, 10, 12, 13, 14, 15], 1e-3 * haar(6)), ([0, 1, 4, 9, 16, 17], 1e3 * haar(6))]
    p = _dense_plan(L, n, gates)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    q64 = L.create(n)
    L.set_amps(q64, psi)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_copyFromQureg(q32, q64)
    L.lib.quest_gb300_setTensorCoreKernel(version)
    rc = L.lib.quest_gb300_applyPlanF32(q32, p)
    L.lib.quest_gb300_setTensorCoreKernel(0)
    assert rc == 0
    assert all(L.lib.quest_gb300_planPassUsesTensorCores(p, i) >= 2 for i in range(len(gates)))
    for ts, m in gates:
        L.applyMatrixN(q64, ts, m)
    ref, got = L.amps(q64), L.amps_f32(q32, n)
    omf = 1 - abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    err = float(np.max(np.abs(got - ref)))
    p64, p32 = np.vdot(ref, ref).real, np.vdot(got, got).real
    print(f"split-FP16 scaled blocks v{version}: norm {p64:.6e} vs {p32:.6e}, 1-F={omf:.2e}, max|d amp|={err:.2e}")
    assert abs(p32 / p64 - 1) < 1e-5 and omf < 1e-10 and err < 1e-7
    L.lib.quest_gb300_planDestroy(p)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)


def test_split_fp16_reports_out_of_range_amplitudes(gpulib, split_fp16):
    """An amplitude of modulus 5 exceeds split-FP16's range (3.99 after the
    2^14 scale): the pass's non-finite output is reported as an input error
    naming split-FP16 (the state is lost); split-TF32 takes the same state."""
    L = gpulib
    n = 14
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[3], psi[900] = 5.0, 0.5j
    q64 = L.create(n)
    L.set_amps(q64, psi)
    plan, u = _single_gate_plan(L, n, [0, 1, 2, 3, 4, 5], 5)
    q32 = L.lib.quest_gb300_createQuregF32(n)
    L.lib.quest_gb300_copyFromQureg(q32, q64)
    rc = L.lib.quest_gb300_applyPlanF32(q32, plan)
    errors = list(L.errors)
    L.errors.clear()
    assert rc == -1 and any("split-FP16" in e[1] for e in errors), errors
    L.lib.quest_gb300_setTensorCorePrecision(0)
    L.lib.quest_gb300_copyFromQureg(q32, q64)
    assert L.lib.quest_gb300_applyPlanF32(q32, plan) == 0
    L.multiQubitUnitary(q64, [0, 1, 2, 3, 4, 5], u)
    err = C.c_double(0)
    omf = L.lib.quest_gb300_compareF32(q32, q64, C.byref(err))
    assert omf < 1e-9
    L.lib.quest_gb300_planDestroy(plan)
    L.lib.quest_gb300_destroyQuregF32(q32)
    L.destroy(q64)
