"""ctypes binding of the QuEST C ABI declared in include/QuEST.h.

The same binding drives any shared library that exports that ABI: the GB300
library built from quantumlab_gb300/csrc (the product), and -- in tests only --
the CPU oracle and the reference's own QuEST CPU build.  Function names,
argument order and meaning follow Code/QuEST340/QuEST/include/QuEST.h of the
reference; value types are passed by value exactly as there.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

qreal = C.c_double
c_ll = C.c_longlong


class ComplexArray(C.Structure):
    _fields_ = [("real", C.POINTER(qreal)), ("imag", C.POINTER(qreal))]


class Complex(C.Structure):
    _fields_ = [("real", qreal), ("imag", qreal)]

    def __complex__(self):
        return complex(self.real, self.imag)


class ComplexMatrix2(C.Structure):
    _fields_ = [("real", (qreal * 2) * 2), ("imag", (qreal * 2) * 2)]


class ComplexMatrix4(C.Structure):
    _fields_ = [("real", (qreal * 4) * 4), ("imag", (qreal * 4) * 4)]


class ComplexMatrixN(C.Structure):
    _fields_ = [("numQubits", C.c_int), ("real", C.POINTER(C.POINTER(qreal))),
                ("imag", C.POINTER(C.POINTER(qreal)))]


class Vector(C.Structure):
    _fields_ = [("x", qreal), ("y", qreal), ("z", qreal)]


class PauliHamil(C.Structure):
    _fields_ = [("pauliCodes", C.POINTER(C.c_int)), ("termCoeffs", C.POINTER(qreal)),
                ("numSumTerms", C.c_int), ("numQubits", C.c_int)]


class Qureg(C.Structure):
    _fields_ = [("isDensityMatrix", C.c_int), ("numQubitsRepresented", C.c_int),
                ("numQubitsInStateVec", C.c_int), ("numAmpsPerChunk", c_ll),
                ("numAmpsTotal", c_ll), ("chunkId", C.c_int), ("numChunks", C.c_int),
                ("stateVec", ComplexArray), ("pairStateVec", ComplexArray),
                ("deviceStateVec", ComplexArray), ("firstLevelReduction", C.POINTER(qreal)),
                ("secondLevelReduction", C.POINTER(qreal)), ("qasmLog", C.c_void_p)]


class QuESTEnv(C.Structure):
    _fields_ = [("rank", C.c_int), ("numRanks", C.c_int),
                ("seeds", C.POINTER(C.c_ulong)), ("numSeeds", C.c_int)]


ERROR_HANDLER = C.CFUNCTYPE(None, C.c_char_p, C.c_char_p)

_I, _D, _Q, _P = C.c_int, qreal, Qureg, C.POINTER
# name -> (restype, argtypes)
SIGNATURES = {
    "createQuESTEnv": (QuESTEnv, []),
    "destroyQuESTEnv": (None, [QuESTEnv]),
    "syncQuESTEnv": (None, [QuESTEnv]),
    "seedQuEST": (None, [_P(QuESTEnv), _P(C.c_ulong), _I]),
    "getQuEST_PREC": (_I, []),
    "createQureg": (_Q, [_I, QuESTEnv]),
    "createDensityQureg": (_Q, [_I, QuESTEnv]),
    "createCloneQureg": (_Q, [_Q, QuESTEnv]),
    "destroyQureg": (None, [_Q, QuESTEnv]),
    "copyStateToGPU": (None, [_Q]),
    "copyStateFromGPU": (None, [_Q]),
    "getNumQubits": (_I, [_Q]),
    "getNumAmps": (c_ll, [_Q]),
    "createComplexMatrixN": (ComplexMatrixN, [_I]),
    "destroyComplexMatrixN": (None, [ComplexMatrixN]),
    "createPauliHamil": (PauliHamil, [_I, _I]),
    "destroyPauliHamil": (None, [PauliHamil]),
    "initPauliHamil": (None, [PauliHamil, _P(qreal), _P(C.c_int)]),
    "initBlankState": (None, [_Q]),
    "initZeroState": (None, [_Q]),
    "initPlusState": (None, [_Q]),
    "initClassicalState": (None, [_Q, c_ll]),
    "initPureState": (None, [_Q, _Q]),
    "initDebugState": (None, [_Q]),
    "initStateFromAmps": (None, [_Q, _P(qreal), _P(qreal)]),
    "setAmps": (None, [_Q, c_ll, _P(qreal), _P(qreal), c_ll]),
    "cloneQureg": (None, [_Q, _Q]),
    "setWeightedQureg": (None, [Complex, _Q, Complex, _Q, Complex, _Q]),
    "getAmp": (Complex, [_Q, c_ll]),
    "getRealAmp": (qreal, [_Q, c_ll]),
    "getImagAmp": (qreal, [_Q, c_ll]),
    "getProbAmp": (qreal, [_Q, c_ll]),
    "getDensityAmp": (Complex, [_Q, c_ll, c_ll]),
    "hadamard": (None, [_Q, _I]),
    "pauliX": (None, [_Q, _I]),
    "pauliY": (None, [_Q, _I]),
    "pauliZ": (None, [_Q, _I]),
    "sGate": (None, [_Q, _I]),
    "tGate": (None, [_Q, _I]),
    "phaseShift": (None, [_Q, _I, _D]),
    "rotateX": (None, [_Q, _I, _D]),
    "rotateY": (None, [_Q, _I, _D]),
    "rotateZ": (None, [_Q, _I, _D]),
    "rotateAroundAxis": (None, [_Q, _I, _D, Vector]),
    "compactUnitary": (None, [_Q, _I, Complex, Complex]),
    "unitary": (None, [_Q, _I, ComplexMatrix2]),
    "applyMatrix2": (None, [_Q, _I, ComplexMatrix2]),
    "controlledNot": (None, [_Q, _I, _I]),
    "controlledPauliY": (None, [_Q, _I, _I]),
    "controlledPhaseShift": (None, [_Q, _I, _I, _D]),
    "controlledPhaseFlip": (None, [_Q, _I, _I]),
    "controlledRotateX": (None, [_Q, _I, _I, _D]),
    "controlledRotateY": (None, [_Q, _I, _I, _D]),
    "controlledRotateZ": (None, [_Q, _I, _I, _D]),
    "controlledRotateAroundAxis": (None, [_Q, _I, _I, _D, Vector]),
    "controlledCompactUnitary": (None, [_Q, _I, _I, Complex, Complex]),
    "controlledUnitary": (None, [_Q, _I, _I, ComplexMatrix2]),
    "multiControlledUnitary": (None, [_Q, _P(_I), _I, _I, ComplexMatrix2]),
    "multiStateControlledUnitary": (None, [_Q, _P(_I), _P(_I), _I, _I, ComplexMatrix2]),
    "multiControlledPhaseShift": (None, [_Q, _P(_I), _I, _D]),
    "multiControlledPhaseFlip": (None, [_Q, _P(_I), _I]),
    "multiQubitNot": (None, [_Q, _P(_I), _I]),
    "multiControlledMultiQubitNot": (None, [_Q, _P(_I), _I, _P(_I), _I]),
    "swapGate": (None, [_Q, _I, _I]),
    "sqrtSwapGate": (None, [_Q, _I, _I]),
    "twoQubitUnitary": (None, [_Q, _I, _I, ComplexMatrix4]),
    "controlledTwoQubitUnitary": (None, [_Q, _I, _I, _I, ComplexMatrix4]),
    "multiControlledTwoQubitUnitary": (None, [_Q, _P(_I), _I, _I, _I, ComplexMatrix4]),
    "multiQubitUnitary": (None, [_Q, _P(_I), _I, ComplexMatrixN]),
    "controlledMultiQubitUnitary": (None, [_Q, _I, _P(_I), _I, ComplexMatrixN]),
    "multiControlledMultiQubitUnitary": (None, [_Q, _P(_I), _I, _P(_I), _I, ComplexMatrixN]),
    "applyMatrix4": (None, [_Q, _I, _I, ComplexMatrix4]),
    "applyMatrixN": (None, [_Q, _P(_I), _I, ComplexMatrixN]),
    "multiRotateZ": (None, [_Q, _P(_I), _I, _D]),
    "multiControlledMultiRotateZ": (None, [_Q, _P(_I), _I, _P(_I), _I, _D]),
    "multiRotatePauli": (None, [_Q, _P(_I), _P(_I), _I, _D]),
    "multiControlledMultiRotatePauli": (None, [_Q, _P(_I), _I, _P(_I), _P(_I), _I, _D]),
    "applyTrotterCircuit": (None, [_Q, PauliHamil, _D, _I, _I]),
    "collapseToOutcome": (qreal, [_Q, _I, _I]),
    "measure": (_I, [_Q, _I]),
    "measureWithStats": (_I, [_Q, _I, _P(qreal)]),
    "calcTotalProb": (qreal, [_Q]),
    "calcProbOfOutcome": (qreal, [_Q, _I, _I]),
    "calcProbOfAllOutcomes": (None, [_P(qreal), _Q, _P(_I), _I]),
    "calcInnerProduct": (Complex, [_Q, _Q]),
    "calcDensityInnerProduct": (qreal, [_Q, _Q]),
    "calcPurity": (qreal, [_Q]),
    "calcFidelity": (qreal, [_Q, _Q]),
    "calcHilbertSchmidtDistance": (qreal, [_Q, _Q]),
    "calcExpecPauliProd": (qreal, [_Q, _P(_I), _P(_I), _I, _Q]),
    "calcExpecPauliSum": (qreal, [_Q, _P(_I), _P(qreal), _I, _Q]),
    "calcExpecPauliHamil": (qreal, [_Q, PauliHamil, _Q]),
    "mixDephasing": (None, [_Q, _I, _D]),
    "mixDepolarising": (None, [_Q, _I, _D]),
    "mixDamping": (None, [_Q, _I, _D]),
    "mixDensityMatrix": (None, [_Q, _D, _Q]),
    "mixPauli": (None, [_Q, _I, _D, _D, _D]),
    "mixTwoQubitDephasing": (None, [_Q, _I, _I, _D]),
    "mixTwoQubitDepolarising": (None, [_Q, _I, _I, _D]),
    # extensions (include/quest_gb300.h)
    "quest_gb300_stream": (C.c_void_p, []),
    "quest_gb300_launchCount": (c_ll, []),
    "quest_gb300_eventRecord": (_I, [_I]),
    "quest_gb300_eventElapsedMs": (qreal, [_I, _I]),
    "quest_gb300_planCreate": (C.c_void_p, [_I, _I]),
    "quest_gb300_planDestroy": (None, [C.c_void_p]),
    "quest_gb300_planAddGate": (_I, [C.c_void_p, _P(_I), _I, _P(qreal), _P(qreal)]),
    "quest_gb300_planAddCompactUnitary": (_I, [C.c_void_p, _I, _D, _D, _D, _D]),
    "quest_gb300_planAddUnitary": (_I, [C.c_void_p, _I, _P(qreal), _P(qreal)]),
    "quest_gb300_planAddHadamard": (_I, [C.c_void_p, _I]),
    "quest_gb300_planAddControlledNot": (_I, [C.c_void_p, _I, _I]),
    "quest_gb300_planAddControlledPhaseShift": (_I, [C.c_void_p, _I, _I, _D]),
    "quest_gb300_planSetBeamWidth": (_I, [C.c_void_p, _I]),
    "quest_gb300_planSetMaxControls": (_I, [C.c_void_p, _I]),
    "quest_gb300_planSetLookahead": (_I, [C.c_void_p, _I]),
    "quest_gb300_planPassControls": (_I, [C.c_void_p, _I, _P(_I)]),
    "quest_gb300_planPassBlock": (_I, [C.c_void_p, _I, _I, _P(qreal), _P(qreal)]),
    "quest_gb300_setTensorCorePrecision": (_I, [_I]),
    "quest_gb300_getTensorCorePrecision": (_I, []),
    "quest_gb300_setTensorCoreStaging": (_I, [_I]),
    "quest_gb300_getTensorCoreStaging": (_I, []),
    "quest_gb300_checkTileCoverage": (_I, [_I, _P(_I), _I, _P(_I), _I]),
    "quest_gb300_checkImageLayouts": (_I, []),
    "quest_gb300_roundHalf": (_I, [_P(qreal), _P(C.c_ushort), _I]),
    "quest_gb300_checkHalfImages": (_I, []),
    "quest_gb300_planPassNorms": (_I, [C.c_void_p, _I, C.POINTER(C.c_double)]),
    "quest_gb300_planCompile": (_I, [C.c_void_p]),
    "quest_gb300_planNumGates": (_I, [C.c_void_p]),
    "quest_gb300_planPass": (_I, [C.c_void_p, _I, _P(_I), _P(qreal), _P(qreal)]),
    "quest_gb300_autotune": (_I, [_I]),
    "quest_gb300_planPredictMs": (qreal, [C.c_void_p]),
    "quest_gb300_planCompileTuned": (_I, [C.c_void_p, _I, _I]),
    "quest_gb300_tunedKernel": (_I, [_I, _I, _I, _P(qreal)]),
    "quest_gb300_setKernelTuning": (None, [_I]),
    "quest_gb300_setPlainArithmetic": (_I, [_I]),
    "quest_gb300_setPassEvents": (None, [_I]),
    "quest_gb300_passTimesMs": (_I, [_P(qreal), _I]),
    "quest_gb300_getPlainArithmetic": (_I, []),
    "quest_gb300_createQuregF32": (C.c_void_p, [_I]),
    "quest_gb300_destroyQuregF32": (None, [C.c_void_p]),
    "quest_gb300_initZeroStateF32": (None, [C.c_void_p]),
    "quest_gb300_initStateFromAmpsF32": (None, [C.c_void_p, _P(qreal), _P(qreal)]),
    "quest_gb300_copyStateToHostF32": (None, [C.c_void_p, _P(qreal), _P(qreal)]),
    "quest_gb300_copyFromQureg": (None, [C.c_void_p, _Q]),
    "quest_gb300_copyToQureg": (None, [C.c_void_p, _Q]),
    "quest_gb300_applyPlanF32": (_I, [C.c_void_p, C.c_void_p]),
    "quest_gb300_applyPlanF32Range": (_I, [C.c_void_p, C.c_void_p, _I, _I]),
    "quest_gb300_planPassUsesTensorCores": (_I, [C.c_void_p, _I]),
    "quest_gb300_setTensorCores": (None, [_I]),
    "quest_gb300_setTensorCoreKernel": (None, [_I]),
    "quest_gb300_setCapture": (_I, [_Q, _I]),
    "quest_gb300_hostMirrorPinned": (_I, [_Q]),
    "quest_gb300_planCompileLike": (_I, [C.c_void_p, C.c_void_p]),
    "quest_gb300_trotterBatchCreate": (C.c_void_p, [_I, _I]),
    "quest_gb300_trotterBatchSetInstance": (_I, [C.c_void_p, _I, PauliHamil, C.c_double, _I, _I, C.c_longlong]),
    "quest_gb300_trotterBatchRun": (_I, [C.c_void_p, _P(C.c_double)]),
    "quest_gb300_trotterBatchSetCircuit": (_I, [C.c_void_p, _I, C.c_void_p, PauliHamil, C.c_longlong]),
    "quest_gb300_trotterBatchCopyState": (_I, [C.c_void_p, _I, _Q]),
    "quest_gb300_trotterBatchNumPasses": (_I, [C.c_void_p]),
    "quest_gb300_trotterBatchNumClasses": (_I, [C.c_void_p]),
    "quest_gb300_trotterBatchDestroy": (None, [C.c_void_p]),
    "quest_gb300_captureStats": (_I, [_Q, _P(C.c_longlong), _P(C.c_longlong), _P(C.c_longlong), _P(C.c_double)]),
    "quest_gb300_sampleMeasurements": (_I, [_Q, _P(_I), _I, _I, _P(_I)]),
    "quest_gb300_initProductState": (_I, [_Q, _I, _P(_I), _P(_D), _P(_D)]),
    "quest_gb300_flushCapture": (None, [_Q]),
    "quest_gb300_capturedGates": (_I, [_Q]),
    "quest_gb300_setCaptureFusion": (None, [_I]),
    "quest_gb300_swapTestBatchCreate": (C.c_void_p, [_P(qreal), _P(c_ll), _P(_I), _I, _P(_I), _P(_I), _I]),
    "quest_gb300_swapTestBatchRun": (_I, [C.c_void_p, _P(qreal)]),
    "quest_gb300_swapTestBatchDestroy": (None, [C.c_void_p]),
    "quest_gb300_swapTestBatchTune": (_I, [C.c_void_p, _P(_I), _P(_I), _P(qreal), _P(qreal)]),
    "quest_gb300_calcTotalProbNoAlloc": (_I, [C.c_void_p, C.c_void_p, c_ll, _P(qreal), C.c_void_p]),
    "quest_gb300_calcTotalProbF32": (qreal, [C.c_void_p]),
    "quest_gb300_calcProbOfOutcomeF32": (qreal, [C.c_void_p, _I, _I]),
    "quest_gb300_compareF32": (qreal, [C.c_void_p, _Q, _P(qreal)]),
}


def _ints(xs: Sequence[int]):
    arr = (C.c_int * max(1, len(xs)))(*[int(x) for x in xs])
    return arr


def _reals(xs):
    xs = np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
    return xs, xs.ctypes.data_as(C.POINTER(qreal))


def complex_(z) -> Complex:
    z = complex(z)
    return Complex(z.real, z.imag)


def matrix2(m) -> ComplexMatrix2:
    m = np.asarray(m, dtype=np.complex128)
    out = ComplexMatrix2()
    for r in range(2):
        for c in range(2):
            out.real[r][c] = m[r, c].real
            out.imag[r][c] = m[r, c].imag
    return out


def matrix4(m) -> ComplexMatrix4:
    m = np.asarray(m, dtype=np.complex128)
    out = ComplexMatrix4()
    for r in range(4):
        for c in range(4):
            out.real[r][c] = m[r, c].real
            out.imag[r][c] = m[r, c].imag
    return out


class QuESTLibrary:
    """One loaded library exporting the QuEST C ABI."""

    def __init__(self, path: str, mode: int = C.RTLD_LOCAL):
        # RTLD_LOCAL: several ABI-identical libraries (product, oracle,
        # reference build) may share one test process without interposing.
        if not os.path.exists(path):
            raise FileNotFoundError(f"QuEST ABI library not found: {path}")
        self.path = path
        self.lib = C.CDLL(path, mode=mode)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(self.lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        self.errors: list = []
        self._handler = None
        self._env: Optional[QuESTEnv] = None

    # ---- error hook -------------------------------------------------------
    def capture_errors(self) -> bool:
        """Route invalidQuESTInputError into self.errors (returns False when
        the library has no __other_input_error hook, e.g. the reference's
        non-Windows build)."""
        try:
            slot = C.c_void_p.in_dll(self.lib, "__other_input_error")
        except ValueError:
            return False

        def handler(msg, func):
            self.errors.append((func.decode(), msg.decode()))

        self._handler = ERROR_HANDLER(handler)
        slot.value = C.cast(self._handler, C.c_void_p).value
        return True

    def has(self, name: str) -> bool:
        return getattr(self.lib, name, None) is not None

    def __getattr__(self, name):
        if name.startswith("_") or name in ("lib", "path", "errors"):
            raise AttributeError(name)
        return getattr(self.lib, name)

    # ---- conveniences ------------------------------------------------------
    @property
    def env(self) -> QuESTEnv:
        if self._env is None:
            self._env = self.lib.createQuESTEnv()
        return self._env

    def seed(self, seeds: Sequence[int]):
        arr = (C.c_ulong * len(seeds))(*seeds)
        self.lib.seedQuEST(C.byref(self.env), arr, len(seeds))

    def create(self, n: int, density: bool = False) -> Qureg:
        return (self.lib.createDensityQureg if density else self.lib.createQureg)(n, self.env)

    def destroy(self, q: Qureg):
        self.lib.destroyQureg(q, self.env)

    def amps(self, q: Qureg) -> np.ndarray:
        """All amplitudes as complex128 (syncs the host mirror first)."""
        self.lib.copyStateFromGPU(q)
        n = q.numAmpsTotal
        re = np.ctypeslib.as_array(q.stateVec.real, shape=(n,))
        im = np.ctypeslib.as_array(q.stateVec.imag, shape=(n,))
        return re + 1j * im

    def set_amps(self, q: Qureg, z):
        z = np.asarray(z, dtype=np.complex128)
        re, pre = _reals(z.real)
        im, pim = _reals(z.imag)
        self.lib.initStateFromAmps(q, pre, pim)

    # thin wrappers taking Python lists
    def multiControlledUnitary(self, q, ctrls, targ, u):
        self.lib.multiControlledUnitary(q, _ints(ctrls), len(ctrls), targ, matrix2(u))

    def multiStateControlledUnitary(self, q, ctrls, states, targ, u):
        self.lib.multiStateControlledUnitary(q, _ints(ctrls), _ints(states), len(ctrls), targ, matrix2(u))

    def multiControlledPhaseShift(self, q, qs, ang):
        self.lib.multiControlledPhaseShift(q, _ints(qs), len(qs), ang)

    def multiControlledPhaseFlip(self, q, qs):
        self.lib.multiControlledPhaseFlip(q, _ints(qs), len(qs))

    def multiQubitNot(self, q, ts):
        self.lib.multiQubitNot(q, _ints(ts), len(ts))

    def multiControlledMultiQubitNot(self, q, cs, ts):
        self.lib.multiControlledMultiQubitNot(q, _ints(cs), len(cs), _ints(ts), len(ts))

    def multiRotateZ(self, q, qs, ang):
        self.lib.multiRotateZ(q, _ints(qs), len(qs), ang)

    def multiControlledMultiRotateZ(self, q, cs, ts, ang):
        self.lib.multiControlledMultiRotateZ(q, _ints(cs), len(cs), _ints(ts), len(ts), ang)

    def multiRotatePauli(self, q, ts, ps, ang):
        self.lib.multiRotatePauli(q, _ints(ts), _ints(ps), len(ts), ang)

    def multiControlledMultiRotatePauli(self, q, cs, ts, ps, ang):
        self.lib.multiControlledMultiRotatePauli(q, _ints(cs), len(cs), _ints(ts), _ints(ps), len(ts), ang)

    def matrixN(self, u):
        u = np.asarray(u, dtype=np.complex128)
        k = int(round(np.log2(u.shape[0])))
        m = self.lib.createComplexMatrixN(k)
        for r in range(1 << k):
            for c in range(1 << k):
                m.real[r][c] = u[r, c].real
                m.imag[r][c] = u[r, c].imag
        return m

    def multiQubitUnitary(self, q, ts, u, ctrls=()):
        m = self.matrixN(u)
        if ctrls:
            self.lib.multiControlledMultiQubitUnitary(q, _ints(ctrls), len(ctrls), _ints(ts), len(ts), m)
        else:
            self.lib.multiQubitUnitary(q, _ints(ts), len(ts), m)
        self.lib.destroyComplexMatrixN(m)

    def applyMatrixN(self, q, ts, u):
        m = self.matrixN(u)
        self.lib.applyMatrixN(q, _ints(ts), len(ts), m)
        self.lib.destroyComplexMatrixN(m)

    def calcProbOfAllOutcomes(self, q, qs):
        out = np.zeros(1 << len(qs))
        self.lib.calcProbOfAllOutcomes(out.ctypes.data_as(C.POINTER(qreal)), q, _ints(qs), len(qs))
        return out

    def calcExpecPauliSum(self, q, codes, coeffs, ws):
        codes = np.ascontiguousarray(np.asarray(codes, dtype=np.int32).ravel())
        co, pco = _reals(coeffs)
        return self.lib.calcExpecPauliSum(q, codes.ctypes.data_as(C.POINTER(C.c_int)), pco, len(co), ws)

    def calcExpecPauliProd(self, q, ts, ps, ws):
        return self.lib.calcExpecPauliProd(q, _ints(ts), _ints(ps), len(ts), ws)

    # ---- fused FP32 engine (include/quest_gb300.h) ----------------------------
    def plan(self, n: int, kmax: int, ops, controls: Optional[int] = None) -> int:
        """Record workloads-style ops into a fusion plan and compile it
        (`controls`: the plan's control-qubit limit, else the library's
        default for n)."""
        p = self.lib.quest_gb300_planCreate(n, kmax)
        if not p:
            raise ValueError("invalid plan parameters")
        if controls is not None and self.lib.quest_gb300_planSetMaxControls(p, controls) != 0:
            raise ValueError("invalid control limit")
        for op in ops:
            k = op[0]
            if k == "cu":
                rc = self.lib.quest_gb300_planAddCompactUnitary(p, *op[1:])
            elif k == "cx":
                rc = self.lib.quest_gb300_planAddControlledNot(p, op[1], op[2])
            elif k == "cp":
                rc = self.lib.quest_gb300_planAddControlledPhaseShift(p, op[1], op[2], op[3])
            elif k == "h":
                rc = self.lib.quest_gb300_planAddHadamard(p, op[1])
            else:
                raise ValueError(f"op {k} cannot be fused")
            if rc != 0:
                raise ValueError(f"rejected op {op}")
        self.lib.quest_gb300_planCompile(p)
        return p

    def amps_f32(self, q32, n: int) -> np.ndarray:
        re = np.empty(1 << n)
        im = np.empty(1 << n)
        self.lib.quest_gb300_copyStateToHostF32(q32, re.ctypes.data_as(C.POINTER(qreal)), im.ctypes.data_as(C.POINTER(qreal)))
        return re + 1j * im

    def pauli_hamil(self, codes, coeffs):
        codes = np.asarray(codes, dtype=np.int32)
        nt, nq = codes.shape
        h = self.lib.createPauliHamil(nq, nt)
        flat = np.ascontiguousarray(codes.ravel())
        co, pco = _reals(coeffs)
        self.lib.initPauliHamil(h, pco, flat.ctypes.data_as(C.POINTER(C.c_int)))
        return h


__all__ = ["QuESTLibrary", "Qureg", "Complex", "ComplexMatrix2", "ComplexMatrix4",
           "Vector", "complex_", "matrix2", "matrix4", "SIGNATURES"]
