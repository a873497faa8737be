"""GPU library vs the reference's outputs (golden fixtures) and vs the oracle.

Every API case of the catalogue is replayed through the C ABI of
libquest_gb300.so on cuda:0 and compared amplitude by amplitude (FP64 plain
path: |d amp| <= 1e-12 x the case's largest amplitude)."""
import numpy as np
import pytest

import quest_cases as QC
from parity import check_case
from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_catalogue_against_reference(gpulib, golden):
    cases, amps, _ = golden
    failures = []
    for i, case in enumerate(cases):
        a, results, probes = QC.run_case(gpulib, case)
        try:
            check_case(case, a, results, probes, amps[f"case{i}"])
        except AssertionError as e:
            failures.append(str(e))
    assert not failures, f"{len(failures)} failing cases:\n" + "\n".join(failures[:40])


def test_circuits_against_reference(gpulib, golden):
    _, _, circ = golden
    L = gpulib
    q = L.create(12)
    W.run_ops(L, q, W.c1_circuit(n=12, layers=8, seed=11))
    assert np.max(np.abs(L.amps(q) - circ["c1_amps"])) < 1e-12
    assert abs(L.lib.calcTotalProb(q) - circ["c1_total"][0]) < 1e-13
    p1 = [L.lib.calcProbOfOutcome(q, t, 1) for t in range(12)]
    assert np.max(np.abs(np.array(p1) - circ["c1_p1"])) < 1e-13
    L.destroy(q)
    q = L.create(10)
    W.run_ops(L, q, W.c2_circuit(n=10, layers=6, seed=12))
    assert np.max(np.abs(L.amps(q) - circ["c2_amps"])) < 1e-12
    L.destroy(q)
    d = L.create(5, True)
    W.run_ops(L, d, W.c3_circuit(nq=5, layers=4, seed=13))
    assert np.max(np.abs(L.amps(d) - circ["c3_amps"])) < 1e-12
    assert abs(L.lib.calcPurity(d) - circ["c3_purity"][0]) < 1e-12
    assert abs(L.lib.calcTotalProb(d) - circ["c3_trace"][0]) < 1e-12
    L.destroy(d)


def test_hubbard_trotter_against_reference(gpulib, golden):
    _, _, circ = golden
    L = gpulib
    for k, (U, dt, order) in enumerate([(2.0, 0.1, 1), (4.0, 0.05, 2), (8.0, 0.1, 2)]):
        codes, coeffs, const = W.hubbard_terms(4, U)
        q = L.create(8)
        L.lib.initClassicalState(q, W.neel_index(4))
        h = L.pauli_hamil(codes, coeffs)
        L.lib.applyTrotterCircuit(q, h, 1.0, order, int(round(1.0 / dt)))
        ws = L.create(8)
        e = L.calcExpecPauliSum(q, codes, coeffs, ws) + const
        assert abs(e - circ["c4_energy"][k]) < 1e-11
        occ = [L.lib.calcProbOfOutcome(q, t, 1) for t in range(8)]
        assert np.max(np.abs(np.array(occ) - circ["c4_occ"][k])) < 1e-12
        L.destroy(ws)
        L.lib.destroyPauliHamil(h)
        L.destroy(q)


@pytest.mark.parametrize("n", [16, 20])
def test_plain_random_circuit_vs_oracle(gpulib, oracle, n):
    """Config-1 structure at full size (20 qubits, 40 layers): every amplitude,
    total probability and P(q=1) for every qubit against the oracle."""
    ops = W.c1_circuit(n=n, layers=40 if n == 20 else 10, seed=1)
    res = []
    for L in (gpulib, oracle):
        q = L.create(n)
        W.run_ops(L, q, ops)
        res.append((L.amps(q).copy(), L.lib.calcTotalProb(q), [L.lib.calcProbOfOutcome(q, t, 1) for t in range(n)]))
        L.destroy(q)
    (ag, tg, pg), (ao, to, po) = res
    assert np.max(np.abs(ag - ao)) < 1e-12
    assert abs(tg - to) < 1e-13 and abs(tg - 1) < 1e-10
    assert np.max(np.abs(np.array(pg) - np.array(po))) < 1e-13


def test_validation_messages_match_reference(gpulib):
    """Invalid input reaches invalidQuESTInputError with the reference's
    message; the call returns without touching the state."""
    L = gpulib
    assert L.capture_errors()
    q = L.create(3)
    before = L.amps(q).copy()
    L.errors.clear()
    L.lib.hadamard(q, 3)
    L.lib.controlledNot(q, 1, 1)
    L.lib.compactUnitary(q, 0, QC.Complex(1, 0), QC.Complex(1, 0))
    L.lib.mixDephasing(q, 0, 0.1)
    L.lib.calcProbOfOutcome(q, 0, 2)
    msgs = [m for _, m in L.errors]
    assert msgs == ["Invalid target qubit. Must be >=0 and <numQubits.",
                    "Control qubit cannot equal target qubit.",
                    "Compact matrix formed by given complex numbers is not unitary.",
                    "Operation valid only for density matrices.",
                    "Invalid measurement outcome -- must be either 0 or 1."]
    assert np.array_equal(L.amps(q), before)
    L.destroy(q)


def test_channel_validation_and_unsupported_api(gpulib):
    """The two-qubit and Pauli channels check their input as the reference
    does (QuEST_validation.c:457-461, 609-643); the API outside the
    simulation path reports "unsupported"; neither touches the state."""
    L = gpulib
    assert L.capture_errors()
    d = L.create(3, True)
    L.lib.initPlusState(d)
    before = L.amps(d).copy()
    L.errors.clear()
    L.lib.mixTwoQubitDephasing(d, 1, 1, 0.1)
    L.lib.mixTwoQubitDephasing(d, 0, 1, 0.8)
    L.lib.mixTwoQubitDepolarising(d, 0, 3, 0.1)
    L.lib.mixTwoQubitDepolarising(d, 0, 1, 0.95)
    L.lib.mixPauli(d, 0, 0.3, 0.3, 0.1)
    L.lib.mixPauli(d, 0, -0.1, 0, 0)
    L.lib.applyFullQFT(d)
    msgs = [m for _, m in L.errors]
    assert msgs[:6] == ["The target qubits must be unique.",
                        "The probability of a two-qubit qubit dephase error cannot exceed 3/4, which maximally mixes.",
                        "Invalid target qubit. Must be >=0 and <numQubits.",
                        "The probability of a two-qubit depolarising error cannot exceed 15/16, which maximally mixes.",
                        "The probability of any X, Y or Z error cannot exceed the probability of no error.",
                        "Probabilities must be in [0, 1]."]
    assert "unsupported" in msgs[6] and L.errors[6][0] == "applyFullQFT"
    assert np.array_equal(L.amps(d), before)
    q = L.create(3)
    L.errors.clear()
    L.lib.mixPauli(q, 0, 0.1, 0.1, 0.1)
    assert [m for _, m in L.errors] == ["Operation valid only for density matrices."]
    L.destroy(q)
    L.destroy(d)


def test_host_mirror_is_page_locked(gpulib):
    """createQureg page-locks its host mirror (cudaMallocHost), so that
    copyStateToGPU / copyStateFromGPU run at the host link's speed; the query
    answers -1 for a register it does not know."""
    L = gpulib
    q = L.create(10)
    assert L.lib.quest_gb300_hostMirrorPinned(q) == 1
    L.destroy(q)
    assert L.lib.quest_gb300_hostMirrorPinned(q) == -1


def _many_term_sum(n, rng):
    """181 Pauli strings: 100 diagonal (two diagonal-group chunks), 40 on one
    shared X/Y support (two pair-group chunks), 40 random (more groups than
    one batch of result slots) and the identity."""
    codes = [[3 * int(rng.integers(2)) for _ in range(n)] for _ in range(100)]
    support = [1, n // 2, n - 1]
    for _ in range(40):
        c = [3 * int(rng.integers(2)) for _ in range(n)]
        for t in support:
            c[t] = int(rng.integers(1, 3))
        codes.append(c)
    codes += [[int(rng.integers(4)) for _ in range(n)] for _ in range(40)]
    codes.append([0] * n)
    return np.array(codes, dtype=np.int32), rng.normal(size=len(codes))


@pytest.mark.parametrize("density", [False, True])
def test_many_term_pauli_sum_vs_oracle(gpulib, oracle, density):
    """calcExpecPauliSum with many terms per X/Y group and many groups, on a
    state vector (12 qubits) and a density matrix (6 qubits), against the
    oracle to 1e-10 of the sum of |coefficients|."""
    n = 6 if density else 12
    rng = np.random.default_rng(17)
    codes, coeffs = _many_term_sum(n, rng)
    vals = []
    for L in (gpulib, oracle):
        q = L.create(n, density=density)
        ws = L.create(n, density=density)
        L.lib.initPlusState(q)
        W.run_ops(L, q, W.c1_circuit(n=n, layers=3, seed=5))
        if density:
            for t in range(0, n, 2):
                L.lib.mixDepolarising(q, t, 0.05)
                L.lib.mixDamping(q, (t + 1) % n, 0.1)
        vals.append(L.calcExpecPauliSum(q, codes, coeffs, ws))
        L.destroy(ws)
        L.destroy(q)
    assert abs(vals[0] - vals[1]) < 1e-10 * np.sum(np.abs(coeffs)), vals


@pytest.fixture
def double_float(gpulib):
    """The plain path's double-float mode for the general 2 x 2 gates, reset
    to exact FP64 afterwards."""
    assert gpulib.lib.quest_gb300_setPlainArithmetic(1) == 0
    yield gpulib
    gpulib.lib.quest_gb300_setPlainArithmetic(0)


def test_double_float_mode_catalogue(double_float, golden):
    """Every catalogue case with the general 2 x 2 gates in double-float
    arithmetic against the reference's FP64 outputs, at the plain path's
    tolerance (1e-12 x the case's largest amplitude)."""
    cases, amps, _ = golden
    failures = []
    for i, case in enumerate(cases):
        a, results, probes = QC.run_case(double_float, case)
        try:
            check_case(case, a, results, probes, amps[f"case{i}"])
        except AssertionError as e:
            failures.append(str(e))
    assert not failures, f"{len(failures)} failing cases:\n" + "\n".join(failures[:40])


def test_double_float_mode_circuit_vs_oracle(double_float, oracle):
    """The 20-qubit, 40-layer plain circuit (800 compactUnitary, 380 CNOT) in
    double-float mode against the oracle's FP64: every amplitude within
    1e-12 x max|amp|, total probability and P(q = 1) within 1e-12."""
    L = double_float
    n = 20
    ops = W.c1_circuit(n=n, layers=40, seed=1)
    res = []
    for lib in (L, oracle):
        q = lib.create(n)
        W.run_ops(lib, q, ops)
        res.append((lib.amps(q).copy(), lib.lib.calcTotalProb(q), [lib.lib.calcProbOfOutcome(q, t, 1) for t in range(n)]))
        lib.destroy(q)
    (ag, tg, pg), (ao, to, po) = res
    err = float(np.max(np.abs(ag - ao)))
    print(f"double-float 20q/40 layers: max|d amp| = {err:.3e} (max|amp| {np.max(np.abs(ao)):.3e})")
    assert err <= 1e-12 * float(np.max(np.abs(ao)))
    assert abs(tg - to) < 1e-12 and np.max(np.abs(np.array(pg) - np.array(po))) < 1e-12


def test_lab_channels_on_a_larger_density_matrix(gpulib, oracle):
    """mixPauli and the two-qubit dephasing / depolarising channels on a
    7-qubit density matrix (a 14-qubit vector: the 16-byte form of the
    two-qubit kernel runs whenever the lower qubit is not 0), every ordered
    pair of a few qubits, against the oracle to 1e-12."""
    n = 7
    rng = np.random.default_rng(23)
    ops = W.c3_circuit(nq=n, layers=2, seed=8)
    res = []
    for L in (gpulib, oracle):
        d = L.create(n, True)
        L.lib.initZeroState(d)
        W.run_ops(L, d, ops)
        r = np.random.default_rng(5)
        for q1, q2 in [(0, 1), (1, 0), (2, 6), (6, 3), (4, 5), (5, 2)]:
            L.lib.mixTwoQubitDephasing(d, q1, q2, float(r.uniform(0, 0.75)))
            L.lib.mixTwoQubitDepolarising(d, q2, q1, float(r.uniform(0, 15 / 16)))
            L.lib.mixPauli(d, q1, float(r.uniform(0, 0.2)), float(r.uniform(0, 0.2)), float(r.uniform(0, 0.2)))
        res.append((L.amps(d).copy(), L.lib.calcTotalProb(d), L.lib.calcPurity(d)))
        L.destroy(d)
    (ag, tg, pg), (ao, to, po) = res
    assert np.max(np.abs(ag - ao)) <= 1e-12 * max(1.0, float(np.max(np.abs(ao))))
    assert abs(tg - to) < 1e-12 and abs(pg - po) < 1e-12
    _ = rng
