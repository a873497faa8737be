"""Batched Trotter instances (GPU): several Fermi-Hubbard instances with
different U evolve together (one fusion plan, one tensor-core launch per pass
over all states, graph replay after the first run).  Each instance must match
QuEST's applyTrotterCircuit run alone in FP64 on the plain path: 1 - F <=
1e-6, max |d amp| <= 1e-5, and its energy to 1e-5 of the coefficients' total
magnitude (the fused FP32 engine's bounds)."""
import ctypes as C

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def library_errors(gpulib):
    gpulib.capture_errors()
    gpulib.errors.clear()
    yield gpulib.errors
    gpulib.errors.clear()


def plain_run(L, sites, U, time, order, reps):
    codes, coeffs, _ = W.hubbard_terms(sites, U)
    n = 2 * sites
    h = L.pauli_hamil(codes, coeffs)
    q, ws = L.create(n), L.create(n)
    L.lib.initClassicalState(q, W.neel_index(sites))
    L.lib.applyTrotterCircuit(q, h, time, order, reps)
    amps = L.amps(q).copy()
    energy = L.lib.calcExpecPauliHamil(q, h, ws)
    L.destroy(ws)
    L.destroy(q)
    L.lib.destroyPauliHamil(h)
    return amps, energy, float(np.sum(np.abs(coeffs)))


@pytest.mark.parametrize("sites,order,reps", [(6, 1, 10), (6, 2, 5), (7, 1, 4)])
def test_batch_matches_each_instance_alone(gpulib, library_errors, sites, order, reps):
    L = gpulib
    lib = L.lib
    n, time = 2 * sites, 1.0
    Us = [2.0, 4.0, 8.0]
    b = lib.quest_gb300_trotterBatchCreate(n, len(Us))
    assert b
    hams = []
    for i, U in enumerate(Us):
        codes, coeffs, _ = W.hubbard_terms(sites, U)
        hams.append(L.pauli_hamil(codes, coeffs))
        assert lib.quest_gb300_trotterBatchSetInstance(b, i, hams[-1], time, order, reps, W.neel_index(sites)) == 0
    e1 = (C.c_double * len(Us))()
    assert lib.quest_gb300_trotterBatchRun(b, e1) == 0, list(library_errors)
    passes = lib.quest_gb300_trotterBatchNumPasses(b)
    e2 = (C.c_double * len(Us))()
    assert lib.quest_gb300_trotterBatchRun(b, e2) == 0          # graph replay
    assert list(e1) == list(e2)
    q = L.create(n)
    for i, U in enumerate(Us):
        want, e_want, scale = plain_run(L, sites, U, time, order, reps)
        assert lib.quest_gb300_trotterBatchCopyState(b, i, q) == 0
        got = L.amps(q)
        f = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        err = np.max(np.abs(got - want))
        print(f"sites={sites} order={order} U={U}: {passes} passes, 1-F={1 - f:.2e}, max|d amp|={err:.2e}, "
              f"dE={e1[i] - e_want:.2e}")
        assert 1 - f <= 1e-6 and err <= 1e-5
        assert abs(e1[i] - e_want) <= 1e-5 * scale
    L.destroy(q)
    lib.quest_gb300_trotterBatchDestroy(b)
    for h in hams:
        lib.destroyPauliHamil(h)
    assert not library_errors


def test_batch_matches_oracle(gpulib, oracle, library_errors):
    """Batch instances against the CPU oracle's applyTrotterCircuit directly
    (not through the plain GPU engine): 6 sites, orders 1 and 2, U = 2, 8."""
    L = gpulib
    lib = L.lib
    sites, time = 6, 1.0
    n = 2 * sites
    inst = [(2.0, 1, 6), (8.0, 2, 3)]
    b = lib.quest_gb300_trotterBatchCreate(n, len(inst))
    hams = []
    for i, (U, order, reps) in enumerate(inst):
        codes, coeffs, _ = W.hubbard_terms(sites, U)
        hams.append(L.pauli_hamil(codes, coeffs))
        assert lib.quest_gb300_trotterBatchSetInstance(b, i, hams[-1], time, order, reps, W.neel_index(sites)) == 0
    e = (C.c_double * len(inst))()
    assert lib.quest_gb300_trotterBatchRun(b, e) == 0, list(library_errors)
    q = L.create(n)
    for i, (U, order, reps) in enumerate(inst):
        want, e_want, scale = plain_run(oracle, sites, U, time, order, reps)
        assert lib.quest_gb300_trotterBatchCopyState(b, i, q) == 0
        got = L.amps(q)
        f = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        err = np.max(np.abs(got - want))
        print(f"U={U} order={order} reps={reps} vs oracle: 1-F={1 - f:.2e}, max|d amp|={err:.2e}, dE={e[i] - e_want:.2e}")
        assert 1 - f <= 1e-6 and err <= 1e-5
        assert abs(e[i] - e_want) <= 1e-5 * scale
    L.destroy(q)
    lib.quest_gb300_trotterBatchDestroy(b)
    for h in hams:
        lib.destroyPauliHamil(h)
    assert not library_errors


def _check_instance(L, b, i, sites, U, time, order, reps, energy, q=None):
    """Instance i of the batch against applyTrotterCircuit run alone in FP64."""
    want, e_want, scale = plain_run(L, sites, U, time, order, reps)
    own = q is None
    if own:
        q = L.create(2 * sites)
    assert L.lib.quest_gb300_trotterBatchCopyState(b, i, q) == 0
    got = L.amps(q)
    if own:
        L.destroy(q)
    f = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
    err = np.max(np.abs(got - want))
    assert 1 - f <= 1e-6 and err <= 1e-5, (i, 1 - f, err)
    assert abs(energy - e_want) <= 1e-5 * scale, (i, energy, e_want)
    return 1 - f, abs(energy - e_want) / scale


def test_batch_of_uneven_instances(gpulib, library_errors):
    """Instances of different Trotter orders, step counts (repetitions),
    Hamiltonians and register sizes run in one batch: they fall into classes
    of one shape each, and every instance matches its own plain FP64 run; the
    graph replay gives the same energies."""
    L = gpulib
    lib = L.lib
    # (sites, U, time, order, reps): orders 1/2/4, 2..6 steps, 6 and 7 sites
    spec = [(6, 2.0, 1.0, 1, 2), (6, 4.0, 1.0, 2, 3), (6, 8.0, 0.5, 1, 6), (7, 2.0, 1.0, 2, 2),
            (6, 4.0, 1.0, 1, 2), (6, 2.0, 0.7, 4, 1), (7, 4.0, 1.0, 2, 2), (6, 8.0, 1.0, 2, 3)]
    b = lib.quest_gb300_trotterBatchCreate(14, len(spec))
    assert b
    hams = []
    for i, (sites, U, time, order, reps) in enumerate(spec):
        codes, coeffs, _ = W.hubbard_terms(sites, U)
        hams.append(L.pauli_hamil(codes, coeffs))
        assert lib.quest_gb300_trotterBatchSetInstance(b, i, hams[-1], time, order, reps, W.neel_index(sites)) == 0
    e1 = (C.c_double * len(spec))()
    assert lib.quest_gb300_trotterBatchRun(b, e1) == 0, list(library_errors)
    # classes: (6 sites, o1, 2 reps) x2, (6, o2, 3) x2, (6, o1, 6), (7, o2, 2) x2, (6, o4, 1)
    assert lib.quest_gb300_trotterBatchNumClasses(b) == 5
    e2 = (C.c_double * len(spec))()
    assert lib.quest_gb300_trotterBatchRun(b, e2) == 0
    assert list(e1) == list(e2)
    for i, (sites, U, time, order, reps) in enumerate(spec):
        dF, dE = _check_instance(L, b, i, sites, U, time, order, reps, e1[i])
        print(f"instance {i} {spec[i]}: 1-F={dF:.2e}, |dE|/sum|c|={dE:.2e}")
    lib.quest_gb300_trotterBatchDestroy(b)
    for h in hams:
        lib.destroyPauliHamil(h)
    assert not library_errors


def test_batch_checks_and_precision_switch(gpulib, library_errors):
    """CopyState needs a run and a register of the instance's size; changing
    the tensor-core precision between runs rebuilds the batch's operands for
    the new kernels."""
    L = gpulib
    lib = L.lib
    sites = 6
    n = 2 * sites
    b = lib.quest_gb300_trotterBatchCreate(n, 2)
    c0, k0, _ = W.hubbard_terms(sites, 2.0)
    h0 = L.pauli_hamil(c0, k0)
    assert lib.quest_gb300_trotterBatchSetInstance(b, 0, h0, 1.0, 1, 2, W.neel_index(sites)) == 0
    assert lib.quest_gb300_trotterBatchSetInstance(b, 1, h0, 1.0, 2, 2, W.neel_index(sites)) == 0
    q = L.create(n)
    assert lib.quest_gb300_trotterBatchCopyState(b, 0, q) == -1                          # nothing run yet
    assert any("run it first" in m for _, m in library_errors), list(library_errors)
    library_errors.clear()
    c1, k1, _ = W.hubbard_terms(7, 2.0)
    h1 = L.pauli_hamil(c1, k1)
    assert lib.quest_gb300_trotterBatchSetInstance(b, 0, h1, 1.0, 1, 2, 0) == -1         # wider than the batch
    library_errors.clear()
    before = lib.quest_gb300_getTensorCorePrecision()
    e = (C.c_double * 2)()
    try:
        for prec in (0, 1, 2, 0):
            assert lib.quest_gb300_setTensorCorePrecision(prec) == 0
            assert lib.quest_gb300_trotterBatchRun(b, e) == 0, list(library_errors)
            for i, order in enumerate((1, 2)):
                _check_instance(L, b, i, sites, 2.0, 1.0, order, 2, e[i], q)
    finally:
        lib.quest_gb300_setTensorCorePrecision(before)
    small = L.create(n - 2)
    assert lib.quest_gb300_trotterBatchCopyState(b, 0, small) == -1
    L.destroy(small)
    L.destroy(q)
    lib.quest_gb300_trotterBatchDestroy(b)
    lib.destroyPauliHamil(h0)
    lib.destroyPauliHamil(h1)


def _with_new_angles(ops, seed):
    """The same circuit shape (gates on the same qubits) with other angles."""
    rng = np.random.default_rng(seed)
    out = []
    for op in ops:
        if op[0] == "cu":
            v = rng.normal(size=4)
            v /= np.linalg.norm(v)
            out.append(("cu", op[1], *v))
        elif op[0] == "cp":
            out.append(("cp", op[1], op[2], float(rng.uniform(0, 2 * np.pi))))
        else:
            out.append(op)
    return out


def test_batch_of_explicit_circuits(gpulib, library_errors):
    """Explicit circuits (fusion-plan gate lists) share a batch with a Trotter
    instance: three 13-qubit circuits of one shape with other angles (one
    class), two 14-qubit ones of another shape, each measured against Pauli
    strings shared by its size with its own coefficients; every instance
    matches the same calls run directly in FP64 (state and expectation)."""
    L = gpulib
    lib = L.lib
    rng = np.random.default_rng(31)
    base13 = W.c2_circuit(n=13, layers=4, seed=40)
    base14 = W.c2_circuit(n=14, layers=3, seed=41)
    circuits = [(13, base13), (13, _with_new_angles(base13, 1)), (13, _with_new_angles(base13, 2)),
                (14, base14), (14, _with_new_angles(base14, 3))]
    sites, U = 6, 4.0
    b = lib.quest_gb300_trotterBatchCreate(14, len(circuits) + 1)
    hams, plans, sums = [], [], []
    strings = {n: rng.integers(0, 4, size=(12, n)).astype(np.int32) for n in (13, 14)}   # one set per size
    for i, (n, ops) in enumerate(circuits):
        codes = strings[n]
        coeffs = rng.normal(size=12)
        sums.append((codes, coeffs))
        hams.append(L.pauli_hamil(codes, coeffs))
        plans.append(L.plan(n, 6, ops))
        assert lib.quest_gb300_trotterBatchSetCircuit(b, i, plans[-1], hams[-1], 5 * i) == 0
    tc, tk, _ = W.hubbard_terms(sites, U)
    hams.append(L.pauli_hamil(tc, tk))
    assert lib.quest_gb300_trotterBatchSetInstance(b, len(circuits), hams[-1], 1.0, 1, 3, W.neel_index(sites)) == 0
    e = (C.c_double * (len(circuits) + 1))()
    assert lib.quest_gb300_trotterBatchRun(b, e) == 0, list(library_errors)
    assert lib.quest_gb300_trotterBatchNumClasses(b) == 3
    for i, (n, ops) in enumerate(circuits):
        q, ws = L.create(n), L.create(n)
        L.lib.initClassicalState(q, 5 * i)
        W.run_ops(L, q, ops)
        want = L.amps(q).copy()
        codes, coeffs = sums[i]
        e_want = L.calcExpecPauliSum(q, codes, coeffs, ws)
        assert lib.quest_gb300_trotterBatchCopyState(b, i, q) == 0
        got = L.amps(q)
        f = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        assert 1 - f <= 1e-6 and np.max(np.abs(got - want)) <= 1e-5, (i, 1 - f)
        assert abs(e[i] - e_want) <= 1e-5 * np.sum(np.abs(coeffs)), (i, e[i], e_want)
        L.destroy(ws)
        L.destroy(q)
    _check_instance(L, b, len(circuits), sites, U, 1.0, 1, 3, e[len(circuits)])
    lib.quest_gb300_trotterBatchDestroy(b)
    for p in plans:
        lib.quest_gb300_planDestroy(p)
    for h in hams:
        lib.destroyPauliHamil(h)
    assert not library_errors
