"""Catalogue of API parity cases, in the style of the reference's Catch2 suite
(Code/QuEST340/tests/test_unitaries.cpp etc.: a small register in a known
state, one API call, every amplitude compared).

A case = register kind/size + initial state + a list of API calls + probes
(reductions evaluated afterwards).  Cases are plain JSON data: the golden
generator (tests/golden/make_golden.py) runs them through the reference's own
QuEST CPU build and stores the ops with the results, and the tests replay the
stored ops through the oracle and the GPU library.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from quantumlab_gb300.quest import (Complex, ComplexMatrix2, ComplexMatrix4, Vector, _ints, _reals, matrix2,
                                    matrix4)
from quantumlab_gb300.workloads import Xoshiro

# ------------------------------------------------------------------ encoding
def cplx(z):
    return {"re": float(np.real(z)), "im": float(np.imag(z))}


def mat(m):
    m = np.asarray(m, dtype=np.complex128)
    return {"re": m.real.tolist(), "im": m.imag.tolist()}


def dec_c(d):
    return complex(d["re"], d["im"])


def dec_m(d):
    return np.asarray(d["re"]) + 1j * np.asarray(d["im"])


# ------------------------------------------------------------------ randoms
class R:
    def __init__(self, seed):
        self.x = Xoshiro(seed)

    def u(self, a=0.0, b=1.0):
        return a + (b - a) * self.x.uniform()

    def g(self):
        return self.x.gauss()

    def angle(self):
        return self.u(-2 * math.pi, 2 * math.pi)

    def unitary(self, d):
        z = np.array([[complex(self.g(), self.g()) for _ in range(d)] for _ in range(d)])
        q, r = np.linalg.qr(z)
        ph = np.diag(r) / np.abs(np.diag(r))
        return q * ph

    def pair(self):
        v = np.array([self.g() for _ in range(4)])
        v /= np.linalg.norm(v)
        return complex(v[0], v[1]), complex(v[2], v[3])

    def state(self, n):
        v = np.array([complex(self.g(), self.g()) for _ in range(1 << n)])
        return v / np.linalg.norm(v)

    def choice(self, n, k):
        return self.x.permutation(n)[:k]


# ------------------------------------------------------------------ catalogue
ONE_Q = ["hadamard", "pauliX", "pauliY", "pauliZ", "sGate", "tGate"]
ONE_Q_ANG = ["phaseShift", "rotateX", "rotateY", "rotateZ"]
TWO_Q = ["controlledNot", "controlledPauliY", "controlledPhaseFlip", "swapGate", "sqrtSwapGate"]
TWO_Q_ANG = ["controlledPhaseShift", "controlledRotateX", "controlledRotateY", "controlledRotateZ"]


def gate_ops(rng: R, n: int):
    """One list entry per case: (name, [op, ...])."""
    out = []
    for t in range(n):
        for f in ONE_Q:
            out.append((f"{f}[{t}]", [[f, t]]))
        for f in ONE_Q_ANG:
            out.append((f"{f}[{t}]", [[f, t, rng.angle()]]))
        a, b = rng.pair()
        out.append((f"compactUnitary[{t}]", [["compactUnitary", t, cplx(a), cplx(b)]]))
        out.append((f"unitary[{t}]", [["unitary", t, mat(rng.unitary(2))]]))
        out.append((f"rotateAroundAxis[{t}]", [["rotateAroundAxis", t, rng.angle(), [rng.g(), rng.g(), rng.g()]]]))
        out.append((f"applyMatrix2[{t}]", [["applyMatrix2", t, mat(rng.unitary(2) * 1.3)]]))
    pairs = [(c, t) for c in range(n) for t in range(n) if c != t]
    for c, t in pairs:
        for f in TWO_Q:
            out.append((f"{f}[{c},{t}]", [[f, c, t]]))
        for f in TWO_Q_ANG:
            out.append((f"{f}[{c},{t}]", [[f, c, t, rng.angle()]]))
        a, b = rng.pair()
        out.append((f"controlledCompactUnitary[{c},{t}]", [["controlledCompactUnitary", c, t, cplx(a), cplx(b)]]))
        out.append((f"controlledUnitary[{c},{t}]", [["controlledUnitary", c, t, mat(rng.unitary(2))]]))
        out.append((f"controlledRotateAroundAxis[{c},{t}]",
                    [["controlledRotateAroundAxis", c, t, rng.angle(), [rng.g(), rng.g(), rng.g()]]]))
        out.append((f"twoQubitUnitary[{c},{t}]", [["twoQubitUnitary", c, t, mat(rng.unitary(4))]]))
        out.append((f"applyMatrix4[{c},{t}]", [["applyMatrix4", c, t, mat(rng.unitary(4) * 0.7)]]))
    for k in range(1, n):
        for rep in range(3):
            qs = rng.choice(n, k + 1)
            ctrls, targ = qs[:k], qs[k]
            out.append((f"multiControlledUnitary[{ctrls},{targ}]", [["multiControlledUnitary", ctrls, targ, mat(rng.unitary(2))]]))
            st = [rng.x.randint(2) for _ in ctrls]
            out.append((f"multiStateControlledUnitary[{ctrls},{st},{targ}]",
                        [["multiStateControlledUnitary", ctrls, st, targ, mat(rng.unitary(2))]]))
            out.append((f"multiControlledPhaseShift[{qs}]", [["multiControlledPhaseShift", qs, rng.angle()]]))
            out.append((f"multiControlledPhaseFlip[{qs}]", [["multiControlledPhaseFlip", qs]]))
            out.append((f"multiQubitNot[{qs}]", [["multiQubitNot", qs]]))
            out.append((f"multiRotateZ[{qs}]", [["multiRotateZ", qs, rng.angle()]]))
            paulis = [1 + rng.x.randint(3) for _ in qs]
            out.append((f"multiRotatePauli[{qs},{paulis}]", [["multiRotatePauli", qs, paulis, rng.angle()]]))
            paulis_i = [rng.x.randint(4) for _ in qs]
            out.append((f"multiRotatePauliI[{qs},{paulis_i}]", [["multiRotatePauli", qs, paulis_i, rng.angle()]]))
            if k + 1 < n:
                ts = rng.choice(n, n)
                cs2, ts2 = ts[:k], ts[k:k + 1 + rep % 2]
                if len(ts2) and not set(cs2) & set(ts2):
                    out.append((f"multiControlledMultiQubitNot[{cs2},{ts2}]", [["multiControlledMultiQubitNot", cs2, ts2]]))
                    out.append((f"multiControlledMultiRotateZ[{cs2},{ts2}]",
                                [["multiControlledMultiRotateZ", cs2, ts2, rng.angle()]]))
                    pz = [1 + rng.x.randint(3) for _ in ts2]
                    out.append((f"multiControlledMultiRotatePauli[{cs2},{ts2},{pz}]",
                                [["multiControlledMultiRotatePauli", cs2, ts2, pz, rng.angle()]]))
    for k in (1, 2, 3):
        for rep in range(2):
            ts = rng.choice(n, k)
            out.append((f"multiQubitUnitary[{ts}]", [["multiQubitUnitary", ts, mat(rng.unitary(1 << k))]]))
            out.append((f"applyMatrixN[{ts}]", [["applyMatrixN", ts, mat(rng.unitary(1 << k) * 0.9)]]))
            rest = [q for q in range(n) if q not in ts]
            if rest:
                c = rest[rep % len(rest)]
                out.append((f"multiControlledMultiQubitUnitary[{c},{ts}]",
                            [["multiControlledMultiQubitUnitary", [c], ts, mat(rng.unitary(1 << k))]]))
    for c, t in [(0, 1), (1, 0), (n - 1, 0)]:
        rest = [q for q in range(n) if q not in (c, t)]
        if len(rest) >= 1:
            out.append((f"controlledTwoQubitUnitary[{rest[0]};{c},{t}]",
                        [["controlledTwoQubitUnitary", rest[0], c, t, mat(rng.unitary(4))]]))
    # Trotter: a random Hamiltonian of 4 terms, orders 1, 2, 4
    for order in (1, 2, 4):
        codes = [[rng.x.randint(4) for _ in range(n)] for _ in range(4)]
        coeffs = [rng.g() for _ in range(4)]
        out.append((f"applyTrotterCircuit[o{order}]", [["applyTrotterCircuit", codes, coeffs, rng.u(0.1, 1.5), order, 2]]))
    # initialisation calls
    out.append(("initZeroState", [["initZeroState"]]))
    out.append(("initPlusState", [["initPlusState"]]))
    out.append(("initBlankState", [["initBlankState"]]))
    out.append(("initClassicalState", [["initClassicalState", (1 << n) - 3]]))
    out.append(("initDebugState", [["initDebugState"]]))
    return out


def decoherence_ops(rng: R, n: int):
    out = []
    for t in range(n):
        out.append((f"mixDephasing[{t}]", [["mixDephasing", t, rng.u(0, 0.5)]]))
        out.append((f"mixDepolarising[{t}]", [["mixDepolarising", t, rng.u(0, 0.75)]]))
        out.append((f"mixDamping[{t}]", [["mixDamping", t, rng.u(0, 1.0)]]))
    out.append(("mixDephasing[p=0]", [["mixDephasing", 0, 0.0]]))
    out.append(("mixDamping[p=1]", [["mixDamping", n - 1, 1.0]]))
    out.append(("mixDensityMatrix", [["mixDensityMatrix", rng.u(0, 1)]]))
    out.append(("collapseToOutcome[0,1]", [["collapseToOutcome", 0, 1]]))
    return out


def channel2_ops(rng: R, n: int):
    """The channels QuantumLab's density-matrix simulator adds
    (QLSimulatorDensityMatrix.cpp:136-150): mixPauli on every qubit, and the
    two-qubit dephasing and depolarising channels on every ordered pair."""
    out = []
    for t in range(n):
        px, py = rng.u(0, 0.25), rng.u(0, 0.2)
        out.append((f"mixPauli[{t}]", [["mixPauli", t, px, py, rng.u(0, 0.2)]]))
    out.append(("mixPauli[bound]", [["mixPauli", 0, 0.25, 0.25, 0.25]]))
    for a in range(n):
        for b in range(n):
            if a != b:
                out.append((f"mixTwoQubitDephasing[{a},{b}]", [["mixTwoQubitDephasing", a, b, rng.u(0, 0.75)]]))
                out.append((f"mixTwoQubitDepolarising[{a},{b}]",
                            [["mixTwoQubitDepolarising", a, b, rng.u(0, 15 / 16)]]))
    out.append(("mixTwoQubitDepolarising[max]", [["mixTwoQubitDepolarising", 0, n - 1, 15 / 16]]))
    out.append(("mixTwoQubitDephasing[p=0]", [["mixTwoQubitDephasing", 1, 0, 0.0]]))
    return out


def probes_for(n: int, density: bool, rng: R):
    p = [["calcTotalProb"]]
    for t in range(n):
        p.append(["calcProbOfOutcome", t, 0])
        p.append(["calcProbOfOutcome", t, 1])
    p.append(["calcProbOfAllOutcomes", [0]])
    p.append(["calcProbOfAllOutcomes", rng.choice(n, min(3, n))])
    p.append(["calcProbOfAllOutcomes", list(range(n))])
    codes = [[rng.x.randint(4) for _ in range(n)] for _ in range(6)]
    codes.append([0] * n)
    coeffs = [rng.g() for _ in codes]
    p.append(["calcExpecPauliSum", codes, coeffs])
    ts = rng.choice(n, min(2, n))
    p.append(["calcExpecPauliProd", ts, [1 + rng.x.randint(3) for _ in ts]])
    if density:
        p += [["calcPurity"], ["calcFidelity"], ["calcDensityInnerProduct"], ["calcHilbertSchmidtDistance"]]
    else:
        p += [["calcInnerProduct"], ["calcFidelity"]]
    return p


def build_cases(seed: int = 20261203):
    """The full catalogue: SV of 5 qubits, DM of 3 qubits, 1-qubit edge
    registers, and measurement with fixed seeds."""
    rng = R(seed)
    cases = []
    for density, n in ((False, 5), (True, 3)):
        kind = "dm" if density else "sv"
        ops = gate_ops(rng, n) + (decoherence_ops(rng, n) if density else [])
        for name, seq in ops:
            init = "debug" if rng.x.randint(2) else "random"
            cases.append({"name": f"{kind}{n}:{name}", "density": density, "n": n, "init": init,
                          "ops": seq, "probes": []})
        # reductions on a few states
        for init in ("debug", "random", "plus"):
            cases.append({"name": f"{kind}{n}:reductions:{init}", "density": density, "n": n, "init": init,
                          "ops": [], "probes": probes_for(n, density, rng)})
    # one-qubit registers (a single amplitude pair)
    for density in (False, True):
        kind = "dm" if density else "sv"
        for name, seq in [("hadamard", [["hadamard", 0]]), ("rotateY", [["rotateY", 0, 0.7]]),
                          ("pauliY", [["pauliY", 0]]), ("phaseShift", [["phaseShift", 0, 1.1]]),
                          ("unitary", [["unitary", 0, mat(rng.unitary(2))]])]:
            cases.append({"name": f"{kind}1:{name}", "density": density, "n": 1, "init": "random",
                          "ops": seq, "probes": [["calcTotalProb"], ["calcProbOfOutcome", 0, 1]]})
    # seeded measurement (MT19937 stream must agree with the reference)
    for density, n in ((False, 5), (True, 3)):
        kind = "dm" if density else "sv"
        for s in range(3):
            cases.append({"name": f"{kind}{n}:measure:seed{s}", "density": density, "n": n, "init": "random",
                          "ops": [["seedQuEST", [1000 + s, 77]]] + [["measure", t] for t in range(n)],
                          "probes": [["calcTotalProb"]]})
    # the two-qubit and Pauli channels, on density matrices of 2, 3 and 4
    # qubits (own random stream: the cases above keep their inputs)
    rng2 = R(seed + 1)
    for n in (2, 3, 4):
        for name, seq in channel2_ops(rng2, n):
            cases.append({"name": f"dm{n}:{name}", "density": True, "n": n, "init": "random", "ops": seq,
                          "probes": [], "stream": 2})
    # random initial states are stored explicitly
    for c in cases:
        if c.get("stream") == 2:
            continue
        if c["init"] == "random":
            nsv = 2 * c["n"] if c["density"] else c["n"]
            c["state"] = [cplx(z) for z in rng.state(c["n"])]          # pure state; DM mixes it with |+><+|
            c["mix"] = rng.u(0.2, 0.8)
            _ = nsv
        c["other"] = [cplx(z) for z in rng.state(c["n"])]
    for c in cases:
        if c.get("stream") == 2:
            c["state"] = [cplx(z) for z in rng2.state(c["n"])]
            c["mix"] = rng2.u(0.2, 0.8)
            c["other"] = [cplx(z) for z in rng2.state(c["n"])]
    return cases


# ------------------------------------------------------------------ runner
def _cm2(d):
    return matrix2(dec_m(d))


def _cm4(d):
    return matrix4(dec_m(d))


def prepare(L, case):
    """Create the case's register(s) in their initial state."""
    n, density = case["n"], case["density"]
    q = L.create(n, density)
    init = case["init"]
    if init == "debug":
        L.lib.initDebugState(q)
    elif init == "plus":
        L.lib.initPlusState(q)
    elif init == "random":
        psi = np.array([dec_c(z) for z in case["state"]])
        if density:
            pure = L.create(n)
            L.set_amps(pure, psi)
            L.lib.initPureState(q, pure)
            plus = L.create(n, True)
            L.lib.initPlusState(plus)
            L.lib.mixDensityMatrix(q, case["mix"], plus)
            L.destroy(plus)
            L.destroy(pure)
        else:
            L.set_amps(q, psi)
    other = L.create(n, density)
    psi2 = np.array([dec_c(z) for z in case["other"]])
    if density:
        pure = L.create(n)
        L.set_amps(pure, psi2)
        L.lib.initPureState(other, pure)
        L.destroy(pure)
    else:
        L.set_amps(other, psi2)
    return q, other


def apply(L, q, other, op):
    f, a = op[0], op[1:]
    lib = L.lib
    if f in ONE_Q:
        getattr(lib, f)(q, a[0])
    elif f in ONE_Q_ANG:
        getattr(lib, f)(q, a[0], a[1])
    elif f in TWO_Q:
        getattr(lib, f)(q, a[0], a[1])
    elif f in TWO_Q_ANG:
        getattr(lib, f)(q, a[0], a[1], a[2])
    elif f == "compactUnitary":
        lib.compactUnitary(q, a[0], Complex(a[1]["re"], a[1]["im"]), Complex(a[2]["re"], a[2]["im"]))
    elif f == "controlledCompactUnitary":
        lib.controlledCompactUnitary(q, a[0], a[1], Complex(a[2]["re"], a[2]["im"]), Complex(a[3]["re"], a[3]["im"]))
    elif f in ("unitary", "applyMatrix2"):
        getattr(lib, f)(q, a[0], _cm2(a[1]))
    elif f == "controlledUnitary":
        lib.controlledUnitary(q, a[0], a[1], _cm2(a[2]))
    elif f == "rotateAroundAxis":
        lib.rotateAroundAxis(q, a[0], a[1], Vector(*a[2]))
    elif f == "controlledRotateAroundAxis":
        lib.controlledRotateAroundAxis(q, a[0], a[1], a[2], Vector(*a[3]))
    elif f in ("twoQubitUnitary", "applyMatrix4"):
        getattr(lib, f)(q, a[0], a[1], _cm4(a[2]))
    elif f == "controlledTwoQubitUnitary":
        lib.controlledTwoQubitUnitary(q, a[0], a[1], a[2], _cm4(a[3]))
    elif f == "multiControlledUnitary":
        L.multiControlledUnitary(q, a[0], a[1], dec_m(a[2]))
    elif f == "multiStateControlledUnitary":
        L.multiStateControlledUnitary(q, a[0], a[1], a[2], dec_m(a[3]))
    elif f == "multiControlledPhaseShift":
        L.multiControlledPhaseShift(q, a[0], a[1])
    elif f == "multiControlledPhaseFlip":
        L.multiControlledPhaseFlip(q, a[0])
    elif f == "multiQubitNot":
        L.multiQubitNot(q, a[0])
    elif f == "multiControlledMultiQubitNot":
        L.multiControlledMultiQubitNot(q, a[0], a[1])
    elif f == "multiRotateZ":
        L.multiRotateZ(q, a[0], a[1])
    elif f == "multiControlledMultiRotateZ":
        L.multiControlledMultiRotateZ(q, a[0], a[1], a[2])
    elif f == "multiRotatePauli":
        L.multiRotatePauli(q, a[0], a[1], a[2])
    elif f == "multiControlledMultiRotatePauli":
        L.multiControlledMultiRotatePauli(q, a[0], a[1], a[2], a[3])
    elif f == "multiQubitUnitary":
        L.multiQubitUnitary(q, a[0], dec_m(a[1]))
    elif f == "multiControlledMultiQubitUnitary":
        L.multiQubitUnitary(q, a[1], dec_m(a[2]), ctrls=a[0])
    elif f == "applyMatrixN":
        L.applyMatrixN(q, a[0], dec_m(a[1]))
    elif f == "applyTrotterCircuit":
        h = L.pauli_hamil(a[0], a[1])
        lib.applyTrotterCircuit(q, h, a[2], a[3], a[4])
        lib.destroyPauliHamil(h)
    elif f in ("initZeroState", "initPlusState", "initBlankState", "initDebugState"):
        getattr(lib, f)(q)
    elif f == "initClassicalState":
        lib.initClassicalState(q, a[0])
    elif f in ("mixDephasing", "mixDepolarising", "mixDamping"):
        getattr(lib, f)(q, a[0], a[1])
    elif f == "mixPauli":
        lib.mixPauli(q, a[0], a[1], a[2], a[3])
    elif f in ("mixTwoQubitDephasing", "mixTwoQubitDepolarising"):
        getattr(lib, f)(q, a[0], a[1], a[2])
    elif f == "mixDensityMatrix":
        lib.mixDensityMatrix(q, a[0], other)
    elif f == "collapseToOutcome":
        return float(lib.collapseToOutcome(q, a[0], a[1]))
    elif f == "seedQuEST":
        L.seed(a[0])
    elif f == "measure":
        return int(lib.measure(q, a[0]))
    else:
        raise ValueError(f"unknown op {f}")
    return None


def probe(L, q, other, p):
    f, a = p[0], p[1:]
    lib = L.lib
    if f == "calcTotalProb":
        return [lib.calcTotalProb(q)]
    if f == "calcProbOfOutcome":
        return [lib.calcProbOfOutcome(q, a[0], a[1])]
    if f == "calcProbOfAllOutcomes":
        return L.calcProbOfAllOutcomes(q, a[0]).tolist()
    if f == "calcExpecPauliSum":
        ws = L.create(q.numQubitsRepresented, bool(q.isDensityMatrix))
        v = L.calcExpecPauliSum(q, np.asarray(a[0]), a[1], ws)
        L.destroy(ws)
        return [v]
    if f == "calcExpecPauliProd":
        ws = L.create(q.numQubitsRepresented, bool(q.isDensityMatrix))
        v = L.calcExpecPauliProd(q, a[0], a[1], ws)
        L.destroy(ws)
        return [v]
    if f == "calcPurity":
        return [lib.calcPurity(q)]
    if f == "calcFidelity":
        n = q.numQubitsRepresented
        pure = L.create(n)
        L.set_amps(pure, np.exp(1j * np.arange(1 << n)) / math.sqrt(1 << n))
        v = lib.calcFidelity(q, pure)
        L.destroy(pure)
        return [v]
    if f == "calcInnerProduct":
        z = lib.calcInnerProduct(other, q)
        return [z.real, z.imag]
    if f == "calcDensityInnerProduct":
        return [lib.calcDensityInnerProduct(q, other)]
    if f == "calcHilbertSchmidtDistance":
        return [lib.calcHilbertSchmidtDistance(q, other)]
    raise ValueError(f"unknown probe {f}")


def run_case(L, case):
    """-> (amps complex ndarray, op results list, probe results list)"""
    q, other = prepare(L, case)
    results = []
    for op in case["ops"]:
        r = apply(L, q, other, op)
        if r is not None:
            results.append(r)
    probes = [probe(L, q, other, p) for p in case["probes"]]
    amps = L.amps(q).copy()
    L.destroy(q)
    L.destroy(other)
    return amps, results, probes
