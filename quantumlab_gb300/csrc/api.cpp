// api.cpp -- the QuEST C API front-end of the GB300 library (host C++).
//
// Mirrors the reference front-end Code/QuEST340/QuEST/src/QuEST.c: validate
// the arguments (same checks, same order, same messages as
// QuEST_validation.c), then dispatch to the FP64 engine; density matrices get
// the operation on the row qubits and its conjugate on the column qubits
// (t + N), exactly as QuEST.c does.  Differences by design:
//   * calcTotalProb, calcExpecPauliSum and friends reduce on the device and
//     never copy the state back (the reference copies it to the host,
//     QuEST_gpu.cu:1626-1679) -- the host mirror is therefore NOT refreshed
//     as a side effect of those calls;
//   * multiRotatePauli / applyTrotterCircuit apply each Pauli exponential in
//     one pass instead of the basis-change sequence of QuEST_common.c:411-448;
//   * calcExpecPauliSum groups terms by X/Y support and reduces each group in
//     one read of the state; the workspace register is accepted, validated
//     and left untouched;
//   * every CUDA call is checked and failures are reported through
//     invalidQuESTInputError;
//   * an API call whose validation failed returns if the error handler
//     returns (the reference relies on the handler exiting or throwing).
#include "qg_internal.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <sys/time.h>
#include <unistd.h>
#include <vector>

using qg::idx_t;

// ============================================================ error hook
extern "C" {
pfinvalidQuESTInputError __other_input_error = nullptr;

__attribute__((weak)) void invalidQuESTInputError(const char* errMsg, const char* errFunc) {
    if (__other_input_error) {
        __other_input_error(errMsg, errFunc);
        return;
    }
    printf("!!!\nQuEST Error in function %s: %s\n!!!\nexiting..\n", errFunc, errMsg);
    exit(EXIT_FAILURE);
}
}

namespace {

// messages: identical to QuEST_validation.c:127-213 because callers match them
const char* const E_INVALID_NUM_CREATE_QUBITS = "Invalid number of qubits. Must create >0.";
const char* const E_INVALID_QUBIT_INDEX = "Invalid qubit index. Must be >=0 and <numQubits.";
const char* const E_INVALID_TARGET_QUBIT = "Invalid target qubit. Must be >=0 and <numQubits.";
const char* const E_INVALID_CONTROL_QUBIT = "Invalid control qubit. Must be >=0 and <numQubits.";
const char* const E_INVALID_STATE_INDEX = "Invalid state index. Must be >=0 and <2^numQubits.";
const char* const E_INVALID_AMP_INDEX = "Invalid amplitude index. Must be >=0 and <2^numQubits.";
const char* const E_INVALID_NUM_AMPS = "Invalid number of amplitudes. Must be >=0 and <=2^numQubits (or for density matrices, <=2^(2 numQubits)).";
const char* const E_INVALID_OFFSET_NUM_AMPS_QUREG = "More amplitudes given than exist in the state from the given starting index.";
const char* const E_TARGET_IS_CONTROL = "Control qubit cannot equal target qubit.";
const char* const E_TARGET_IN_CONTROLS = "Control qubits cannot include target qubit.";
const char* const E_CONTROL_TARGET_COLLISION = "Control and target qubits must be disjoint.";
const char* const E_QUBITS_NOT_UNIQUE = "The qubits must be unique.";
const char* const E_TARGETS_NOT_UNIQUE = "The target qubits must be unique.";
const char* const E_CONTROLS_NOT_UNIQUE = "The control qubits should be unique.";
const char* const E_INVALID_NUM_QUBITS = "Invalid number of qubits. Must be >0 and <=numQubits.";
const char* const E_INVALID_NUM_TARGETS = "Invalid number of target qubits. Must be >0 and <=numQubits.";
const char* const E_INVALID_NUM_CONTROLS = "Invalid number of control qubits. Must be >0 and <numQubits.";
const char* const E_NON_UNITARY_MATRIX = "Matrix is not unitary.";
const char* const E_NON_UNITARY_COMPLEX_PAIR = "Compact matrix formed by given complex numbers is not unitary.";
const char* const E_ZERO_VECTOR = "Invalid axis vector. Must be non-zero.";
const char* const E_COLLAPSE_STATE_ZERO_PROB = "Can't collapse to state with zero probability.";
const char* const E_INVALID_QUBIT_OUTCOME = "Invalid measurement outcome -- must be either 0 or 1.";
const char* const E_SECOND_ARG_MUST_BE_STATEVEC = "Second argument must be a state-vector.";
const char* const E_MISMATCHING_QUREG_DIMENSIONS = "Dimensions of the qubit registers don't match.";
const char* const E_MISMATCHING_QUREG_TYPES = "Registers must both be state-vectors or both be density matrices.";
const char* const E_DEFINED_ONLY_FOR_STATEVECS = "Operation valid only for state-vectors.";
const char* const E_DEFINED_ONLY_FOR_DENSMATRS = "Operation valid only for density matrices.";
const char* const E_INVALID_PROB = "Probabilities must be in [0, 1].";
const char* const E_INVALID_ONE_QUBIT_DEPHASE_PROB = "The probability of a single qubit dephase error cannot exceed 1/2, which maximally mixes.";
const char* const E_INVALID_ONE_QUBIT_DEPOL_PROB = "The probability of a single qubit depolarising error cannot exceed 3/4, which maximally mixes.";
const char* const E_INVALID_TWO_QUBIT_DEPHASE_PROB = "The probability of a two-qubit qubit dephase error cannot exceed 3/4, which maximally mixes.";
const char* const E_INVALID_TWO_QUBIT_DEPOL_PROB = "The probability of a two-qubit depolarising error cannot exceed 15/16, which maximally mixes.";
const char* const E_INVALID_ONE_QUBIT_PAULI_PROBS = "The probability of any X, Y or Z error cannot exceed the probability of no error.";
const char* const E_INVALID_CONTROLS_BIT_STATE = "The state of the control qubits must be a bit sequence (0s and 1s).";
const char* const E_INVALID_PAULI_CODE = "Invalid Pauli code. Codes must be 0 (or PAULI_I), 1 (PAULI_X), 2 (PAULI_Y) or 3 (PAULI_Z) to indicate the identity, X, Y and Z operators respectively.";
const char* const E_INVALID_NUM_SUM_TERMS = "Invalid number of terms in the Pauli sum. The number of terms must be >0.";
const char* const E_CANNOT_FIT_MULTI_QUBIT_MATRIX = "The specified matrix targets too many qubits; the batches of amplitudes to modify cannot all fit in a single distributed node's memory allocation.";
const char* const E_INVALID_UNITARY_SIZE = "The matrix size does not match the number of target qubits.";
const char* const E_COMPLEX_MATRIX_NOT_INIT = "The ComplexMatrixN was not successfully created (possibly insufficient memory available).";
const char* const E_INVALID_PAULI_HAMIL_PARAMS = "The number of qubits and terms in the PauliHamil must be strictly positive.";
const char* const E_MISMATCHING_PAULI_HAMIL_QUREG_NUM_QUBITS = "The PauliHamil must act on the same number of qubits as exist in the Qureg.";
const char* const E_INVALID_TROTTER_ORDER = "The Trotterisation order must be 1, or an even number (for higher-order Suzuki symmetrized expansions).";
const char* const E_INVALID_TROTTER_REPS = "The number of Trotter repetitions must be >=1.";
const char* const E_QUREG_NOT_ALLOCATED = "Could not allocate memory for Qureg. Possibly insufficient memory.";
const char* const E_QUREG_NOT_ALLOCATED_ON_GPU = "Could not allocate memory for Qureg on GPU. Possibly insufficient memory.";
const char* const E_NO_GPU = "Trying to run GPU code with no GPU available.";
// not in the reference: functions of the QuEST API that this library exports
// only so that programs written against the whole API link
const char* const E_UNSUPPORTED = "This QuEST function is not supported by the GB300 library (unsupported).";
// not in the reference: this library's dense-matrix kernel limit
const char* const E_MATRIX_TOO_LARGE = "Matrices on more than 10 target qubits are not supported by this library.";

bool fail(const char* msg, const char* fn) {
    invalidQuESTInputError(msg, fn);
    return false;
}
#define REQUIRE(cond, msg) ((cond) ? true : fail((msg), caller))

// ---- the checks of QuEST_validation.c:382-700 --------------------------------
bool vTarget(const Qureg& q, int t, const char* caller) { return REQUIRE(t >= 0 && t < q.numQubitsRepresented, E_INVALID_TARGET_QUBIT); }
bool vControl(const Qureg& q, int c, const char* caller) { return REQUIRE(c >= 0 && c < q.numQubitsRepresented, E_INVALID_CONTROL_QUBIT); }
bool vControlTarget(const Qureg& q, int c, int t, const char* caller) {
    return vTarget(q, t, caller) && vControl(q, c, caller) && REQUIRE(c != t, E_TARGET_IS_CONTROL);
}
bool vUniqueTargets(const Qureg& q, int a, int b, const char* caller) {
    return vTarget(q, a, caller) && vTarget(q, b, caller) && REQUIRE(a != b, E_TARGETS_NOT_UNIQUE);
}
bool unique(const int* qs, int n) {
    uint64_t m = 0;
    for (int i = 0; i < n; ++i) {
        if (qs[i] < 0 || qs[i] > 63 || (m >> qs[i] & 1ull)) return false;
        m |= 1ull << qs[i];
    }
    return true;
}
bool vMultiTargets(const Qureg& q, const int* ts, int n, const char* caller) {
    if (!REQUIRE(n > 0 && n <= q.numQubitsRepresented, E_INVALID_NUM_TARGETS)) return false;
    for (int i = 0; i < n; ++i)
        if (!vTarget(q, ts[i], caller)) return false;
    return REQUIRE(unique(ts, n), E_TARGETS_NOT_UNIQUE);
}
bool vMultiControls(const Qureg& q, const int* cs, int n, const char* caller) {
    if (!REQUIRE(n > 0 && n < q.numQubitsRepresented, E_INVALID_NUM_CONTROLS)) return false;
    for (int i = 0; i < n; ++i)
        if (!vControl(q, cs[i], caller)) return false;
    return REQUIRE(unique(cs, n), E_CONTROLS_NOT_UNIQUE);
}
bool vMultiQubits(const Qureg& q, const int* qs, int n, const char* caller) {
    if (!REQUIRE(n > 0 && n <= q.numQubitsRepresented, E_INVALID_NUM_QUBITS)) return false;
    for (int i = 0; i < n; ++i)
        if (!REQUIRE(qs[i] >= 0 && qs[i] < q.numQubitsRepresented, E_INVALID_QUBIT_INDEX)) return false;
    return REQUIRE(unique(qs, n), E_QUBITS_NOT_UNIQUE);
}
bool vMultiControlsTarget(const Qureg& q, const int* cs, int n, int t, const char* caller) {
    if (!vTarget(q, t, caller) || !vMultiControls(q, cs, n, caller)) return false;
    for (int i = 0; i < n; ++i)
        if (!REQUIRE(cs[i] != t, E_TARGET_IN_CONTROLS)) return false;
    return true;
}
uint64_t maskOf(const int* qs, int n) {
    uint64_t m = 0;
    for (int i = 0; i < n; ++i) m |= 1ull << qs[i];
    return m;
}
bool vMultiControlsMultiTargets(const Qureg& q, const int* cs, int nc, const int* ts, int nt, const char* caller) {
    if (!vMultiControls(q, cs, nc, caller) || !vMultiTargets(q, ts, nt, caller)) return false;
    return REQUIRE(!(maskOf(cs, nc) & maskOf(ts, nt)), E_CONTROL_TARGET_COLLISION);
}
bool vControlState(const int* st, int n, const char* caller) {
    for (int i = 0; i < n; ++i)
        if (!REQUIRE(st[i] == 0 || st[i] == 1, E_INVALID_CONTROLS_BIT_STATE)) return false;
    return true;
}
bool vFits(const Qureg& q, int numTargs, const char* caller) {
    return REQUIRE(q.numAmpsPerChunk >= (1LL << numTargs), E_CANNOT_FIT_MULTI_QUBIT_MATRIX);
}
template <class M>
bool isUnitary(const M& m, int dim) {                   // QuEST_validation.c:271-300
    for (int r = 0; r < dim; ++r)
        for (int c = 0; c < dim; ++c) {
            double er = 0, ei = 0;
            for (int i = 0; i < dim; ++i) {
                er += m.real[r][i] * m.real[c][i] + m.imag[r][i] * m.imag[c][i];
                ei += m.imag[r][i] * m.real[c][i] - m.real[r][i] * m.imag[c][i];
            }
            if (fabs(ei) > REAL_EPS || (r == c && fabs(er - 1) > REAL_EPS) || (r != c && fabs(er) > REAL_EPS)) return false;
        }
    return true;
}
bool vUnitary2(const ComplexMatrix2& u, const char* caller) { return REQUIRE(isUnitary(u, 2), E_NON_UNITARY_MATRIX); }
bool vUnitary4(const Qureg& q, const ComplexMatrix4& u, const char* caller) {
    return vFits(q, 2, caller) && REQUIRE(isUnitary(u, 4), E_NON_UNITARY_MATRIX);
}
bool vMatrixN(const Qureg& q, const ComplexMatrixN& u, int numTargs, const char* caller) {
    if (!REQUIRE(u.real != nullptr && u.imag != nullptr, E_COMPLEX_MATRIX_NOT_INIT)) return false;
    if (!vFits(q, numTargs, caller)) return false;
    if (!REQUIRE(numTargs == u.numQubits, E_INVALID_UNITARY_SIZE)) return false;
    return REQUIRE(numTargs <= 10, E_MATRIX_TOO_LARGE);
}
bool vUnitaryN(const Qureg& q, const ComplexMatrixN& u, int numTargs, const char* caller) {
    return vMatrixN(q, u, numTargs, caller) && REQUIRE(isUnitary(u, 1 << numTargs), E_NON_UNITARY_MATRIX);
}
bool vPair(Complex a, Complex b, const char* caller) {
    return REQUIRE(fabs(-1 + a.real * a.real + a.imag * a.imag + b.real * b.real + b.imag * b.imag) < REAL_EPS,
                   E_NON_UNITARY_COMPLEX_PAIR);
}
bool vVector(Vector v, const char* caller) { return REQUIRE(sqrt(v.x * v.x + v.y * v.y + v.z * v.z) > REAL_EPS, E_ZERO_VECTOR); }
bool vStateVec(const Qureg& q, const char* caller) { return REQUIRE(!q.isDensityMatrix, E_DEFINED_ONLY_FOR_STATEVECS); }
bool vDensity(const Qureg& q, const char* caller) { return REQUIRE(q.isDensityMatrix, E_DEFINED_ONLY_FOR_DENSMATRS); }
bool vOutcome(int o, const char* caller) { return REQUIRE(o == 0 || o == 1, E_INVALID_QUBIT_OUTCOME); }
bool vMatchDims(const Qureg& a, const Qureg& b, const char* caller) {
    return REQUIRE(a.numQubitsRepresented == b.numQubitsRepresented, E_MISMATCHING_QUREG_DIMENSIONS);
}
bool vMatchTypes(const Qureg& a, const Qureg& b, const char* caller) {
    return REQUIRE(a.isDensityMatrix == b.isDensityMatrix, E_MISMATCHING_QUREG_TYPES);
}
bool vSecondStateVec(const Qureg& b, const char* caller) { return REQUIRE(!b.isDensityMatrix, E_SECOND_ARG_MUST_BE_STATEVEC); }
bool vProb(double p, const char* caller) { return REQUIRE(p >= 0 && p <= 1, E_INVALID_PROB); }
bool vPauliCodes(const enum pauliOpType* c, idx_t n, const char* caller) {
    for (idx_t i = 0; i < n; ++i)
        if (!REQUIRE(c[i] >= PAULI_I && c[i] <= PAULI_Z, E_INVALID_PAULI_CODE)) return false;
    return true;
}
bool vAmpIndex(const Qureg& q, idx_t i, const char* caller) {
    return REQUIRE(i >= 0 && i < (1LL << q.numQubitsRepresented), E_INVALID_AMP_INDEX);
}
bool vNumAmps(const Qureg& q, idx_t start, idx_t n, const char* caller) {
    return vAmpIndex(q, start, caller) && REQUIRE(n >= 0 && n <= q.numAmpsTotal, E_INVALID_NUM_AMPS) &&
           REQUIRE(n + start <= q.numAmpsTotal, E_INVALID_OFFSET_NUM_AMPS_QUREG);
}
bool vHamil(const PauliHamil& h, const char* caller) {
    return REQUIRE(h.numQubits > 0 && h.numSumTerms > 0, E_INVALID_PAULI_HAMIL_PARAMS) &&
           vPauliCodes(h.pauliCodes, (idx_t)h.numSumTerms * h.numQubits, caller);
}

// ============================================================ runtime state
std::once_flag g_initOnce;
cudaStream_t g_stream = nullptr;
int g_numSMs = 0;
bool g_haveGPU = false;

void initRuntime() {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return;
    }
    g_haveGPU = true;
    int dev = 0;
    if (const char* e = getenv("QUEST_GB300_DEVICE")) dev = atoi(e);
    if (dev < 0 || dev >= count) dev = 0;
    cudaSetDevice(dev);
    cudaDeviceGetAttribute(&g_numSMs, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreate(&g_stream) != cudaSuccess) g_stream = nullptr;
}

// pinned-vs-pageable bookkeeping for host mirrors, keyed by the device array
std::mutex g_regMutex;
std::map<const void*, bool> g_pinnedMirror;

// ---- MT19937 (Matsumoto & Nishimura, published algorithm) for measure() ----
struct MT19937 {
    static const int N = 624, M = 397;
    unsigned long s[N];
    int pos = N + 1;
    void seed(unsigned long v) {
        s[0] = v & 0xffffffffUL;
        for (int i = 1; i < N; ++i) s[i] = (1812433253UL * (s[i - 1] ^ (s[i - 1] >> 30)) + (unsigned long)i) & 0xffffffffUL;
        pos = N;
    }
    void seedArray(const unsigned long* key, int len) {
        seed(19650218UL);
        int i = 1, j = 0;
        for (int k = (N > len ? N : len); k; --k) {
            s[i] = ((s[i] ^ ((s[i - 1] ^ (s[i - 1] >> 30)) * 1664525UL)) + key[j] + (unsigned long)j) & 0xffffffffUL;
            if (++i >= N) { s[0] = s[N - 1]; i = 1; }
            if (++j >= len) j = 0;
        }
        for (int k = N - 1; k; --k) {
            s[i] = ((s[i] ^ ((s[i - 1] ^ (s[i - 1] >> 30)) * 1566083941UL)) - (unsigned long)i) & 0xffffffffUL;
            if (++i >= N) { s[0] = s[N - 1]; i = 1; }
        }
        s[0] = 0x80000000UL;
    }
    unsigned long next() {
        const unsigned long mag[2] = {0UL, 0x9908b0dfUL};
        if (pos >= N) {
            if (pos == N + 1) seed(5489UL);
            int k = 0;
            for (; k < N - M; ++k) {
                unsigned long y = (s[k] & 0x80000000UL) | (s[k + 1] & 0x7fffffffUL);
                s[k] = s[k + M] ^ (y >> 1) ^ mag[y & 1UL];
            }
            for (; k < N - 1; ++k) {
                unsigned long y = (s[k] & 0x80000000UL) | (s[k + 1] & 0x7fffffffUL);
                s[k] = s[k + (M - N)] ^ (y >> 1) ^ mag[y & 1UL];
            }
            unsigned long y = (s[N - 1] & 0x80000000UL) | (s[0] & 0x7fffffffUL);
            s[N - 1] = s[M - 1] ^ (y >> 1) ^ mag[y & 1UL];
            pos = 0;
        }
        unsigned long y = s[pos++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680UL;
        y ^= (y << 15) & 0xefc60000UL;
        y ^= y >> 18;
        return y;
    }
    double real1() { return (double)next() * (1.0 / 4294967295.0); }
} g_mt;

// State access of every call but the gates: the register's captured gates
// (capture.cpp) are applied first.
inline qg::SV sv(const Qureg& q) {
    qg::captureFlush(q.deviceStateVec.real, q.deviceStateVec.imag);
    return qg::svOf(q);
}
// State access of the gate calls: with capture on, the launchers queue the gate.
inline qg::SV svg(const Qureg& q) {
    qg::SV s = qg::svOf(q);
    s.cap = qg::captureHandle(q.deviceStateVec.real);
    return s;
}
// A call that overwrites the whole state: queued gates are dropped unapplied.
inline qg::SV svOverwrite(const Qureg& q) {
    qg::captureDiscard(q.deviceStateVec.real);
    return qg::svOf(q);
}
inline void flushQ(const Qureg& q) { qg::captureFlush(q.deviceStateVec.real, q.deviceStateVec.imag); }
inline void discardQ(const Qureg& q) { qg::captureDiscard(q.deviceStateVec.real); }
inline bool syncStream(const char* caller) { return !QG_CUDA(cudaStreamSynchronize(qg::stream()), caller); }

qg::Mat2 toMat(const ComplexMatrix2& u, bool conj) {
    qg::Mat2 m;
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            m.r[r][c] = u.real[r][c];
            m.i[r][c] = conj ? -u.imag[r][c] : u.imag[r][c];
        }
    return m;
}

// ---- gate helpers applying the density-matrix doubling -----------------------
void applyCompact(const Qureg& q, int t, uint64_t ctrl, Complex a, Complex b) {
    qg::gateCompact(svg(q), t, ctrl, a.real, a.imag, b.real, b.imag);
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gateCompact(svg(q), t + s, ctrl << s, a.real, -a.imag, b.real, -b.imag);
    }
}
void applyMatrix2Doubled(const Qureg& q, int t, uint64_t ctrl, uint64_t flip, const ComplexMatrix2& u) {
    qg::gateMatrix2(svg(q), t, ctrl, flip, toMat(u, false));
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gateMatrix2(svg(q), t + s, ctrl << s, flip << s, toMat(u, true));
    }
}
void applyPhaseDoubled(const Qureg& q, uint64_t mask, double tr, double ti) {
    qg::gatePhase(svg(q), mask, tr, ti);
    if (q.isDensityMatrix) qg::gatePhase(svg(q), mask << q.numQubitsRepresented, tr, -ti);
}
void rotationPair(double angle, Vector axis, Complex* a, Complex* b) {  // QuEST_common.c:117-124
    const double mag = sqrt(axis.x * axis.x + axis.y * axis.y + axis.z * axis.z);
    const double x = axis.x / mag, y = axis.y / mag, z = axis.z / mag;
    a->real = cos(angle / 2.0);
    a->imag = -sin(angle / 2.0) * z;
    b->real = sin(angle / 2.0) * y;
    b->imag = -sin(angle / 2.0) * x;
}
// Pauli string masks from per-target codes
void pauliMasks(const int* ts, const enum pauliOpType* ps, int n, uint64_t* x, uint64_t* y, uint64_t* z) {
    *x = *y = *z = 0;
    for (int i = 0; i < n; ++i) {
        const uint64_t b = 1ull << ts[i];
        if (ps[i] == PAULI_X) *x |= b;
        if (ps[i] == PAULI_Y) { *x |= b; *y |= b; }
        if (ps[i] == PAULI_Z) *z |= b;
    }
}
void applyPauliRotation(const Qureg& q, uint64_t ctrl, const int* ts, const enum pauliOpType* ps, int n, double angle) {
    uint64_t x, y, z;
    pauliMasks(ts, ps, n, &x, &y, &z);
    if ((x | z) == 0) return;                 // all identity: QuEST applies nothing (QuEST_common.c:430-431)
    qg::gatePauliRotation(svg(q), ctrl, x, y, z, angle, 0);
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gatePauliRotation(svg(q), ctrl << s, x << s, y << s, z << s, angle, 1);
    }
}
void applyMatrixNDoubled(const Qureg& q, uint64_t ctrl, const int* ts, int k, qreal** ur, qreal** ui, bool doubled) {
    const int D = 1 << k;
    std::vector<double> mr((size_t)D * D), mi((size_t)D * D);
    for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) {
            mr[(size_t)r * D + c] = ur[r][c];
            mi[(size_t)r * D + c] = ui[r][c];
        }
    qg::gateMatrixN(svg(q), ctrl, ts, k, mr.data(), mi.data());
    if (doubled && q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        int sh[64];
        for (int i = 0; i < k; ++i) sh[i] = ts[i] + s;
        for (auto& v : mi) v = -v;
        qg::gateMatrixN(svg(q), ctrl << s, sh, k, mr.data(), mi.data());
    }
}

Qureg allocQureg(int nsv, int isDM, int nrep, const char* caller) {
    Qureg q;
    memset(&q, 0, sizeof q);
    std::call_once(g_initOnce, initRuntime);
    if (!g_haveGPU) { fail(E_NO_GPU, caller); return q; }
    const idx_t n = 1LL << nsv;
    q.isDensityMatrix = isDM;
    q.numQubitsRepresented = nrep;
    q.numQubitsInStateVec = nsv;
    q.numAmpsPerChunk = n;
    q.numAmpsTotal = n;
    q.chunkId = 0;
    q.numChunks = 1;
    double* dev = nullptr;
    if (cudaMalloc(&dev, 2 * (size_t)n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        fail(E_QUREG_NOT_ALLOCATED_ON_GPU, caller);
        memset(&q, 0, sizeof q);
        return q;
    }
    double* host = nullptr;
    bool pinned = true;
    if (cudaMallocHost(&host, 2 * (size_t)n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        pinned = false;
        host = (double*)malloc(2 * (size_t)n * sizeof(double));
        if (!host) {
            cudaFree(dev);
            fail(E_QUREG_NOT_ALLOCATED, caller);
            memset(&q, 0, sizeof q);
            return q;
        }
    }
    double* scratch = nullptr;
    double* slot = nullptr;
    if (cudaMalloc(&scratch, qg::kScratchDoubles * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&slot, 64 * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        fail(E_QUREG_NOT_ALLOCATED_ON_GPU, caller);
        memset(&q, 0, sizeof q);
        return q;
    }
    cudaMemsetAsync(scratch, 0, qg::kScratchDoubles * sizeof(double), qg::stream());
    q.deviceStateVec.real = dev;
    q.deviceStateVec.imag = dev + n;
    qg::captureRegister(dev, nsv, isDM ? nrep : 0);
    q.stateVec.real = host;
    q.stateVec.imag = host + n;
    q.pairStateVec.real = nullptr;
    q.pairStateVec.imag = nullptr;
    q.firstLevelReduction = scratch;
    q.secondLevelReduction = slot;
    q.qasmLog = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_regMutex);
        g_pinnedMirror[dev] = pinned;
    }
    return q;
}

double probZero(const Qureg& q, int t) {
    if (q.isDensityMatrix) return qg::reduceProbZeroDM(sv(q), t, q.numQubitsRepresented, qg::scratchOf(q));
    return qg::reduceProbZeroSV(sv(q), t, qg::scratchOf(q));
}
void collapse(const Qureg& q, int t, int outcome, double prob) {
    if (q.isDensityMatrix) qg::collapseDM(sv(q), t, q.numQubitsRepresented, outcome, 1.0 / prob);
    else qg::collapseSV(sv(q), t, outcome, 1.0 / sqrt(prob));
}

}  // namespace

// ============================================================ qg runtime glue
namespace qg {
cudaStream_t stream() {
    std::call_once(g_initOnce, initRuntime);
    return g_stream;
}
int numSMs() {
    std::call_once(g_initOnce, initRuntime);
    return g_numSMs > 0 ? g_numSMs : 1;
}
bool cudaFailed(cudaError_t e, const char* what, const char* caller) {
    if (e == cudaSuccess) return false;
    static thread_local char buf[512];
    snprintf(buf, sizeof buf, "CUDA error (%s) in %s", cudaGetErrorString(e), what);
    cudaGetLastError();
    invalidQuESTInputError(buf, caller);
    return true;
}
bool launchFailed(const char* caller) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaFailed(cudaGetLastError(), "kernel launch", caller);
}
Scratch scratchOf(const Qureg& q) {
    Scratch s;
    s.partials = q.firstLevelReduction;
    s.result = q.firstLevelReduction + 2 * kMaxReduceBlocks;
    s.counter = reinterpret_cast<unsigned int*>(q.firstLevelReduction + 2 * kMaxReduceBlocks + 64);
    s.host = q.secondLevelReduction;
    return s;
}
}  // namespace qg

// ============================================================ C API
extern "C" {

// ---- environment (QuEST_gpu.cu:447-498, QuEST.c:1649-1664) ----
void seedQuEST(QuESTEnv* env, unsigned long int* seedArray, int numSeeds) {
    if (env->seeds) free(env->seeds);
    env->seeds = (unsigned long*)malloc(sizeof(unsigned long) * (numSeeds > 0 ? numSeeds : 1));
    for (int i = 0; i < numSeeds; ++i) env->seeds[i] = seedArray[i];
    env->numSeeds = numSeeds;
    g_mt.seedArray(seedArray, numSeeds);
}
void seedQuESTDefault(QuESTEnv* env) {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    unsigned long keys[2] = {(unsigned long)(tv.tv_sec * 1000 + tv.tv_usec / 1000), (unsigned long)getpid()};
    seedQuEST(env, keys, 2);
}
void getQuESTSeeds(QuESTEnv env, unsigned long int** seeds, int* numSeeds) {
    *seeds = env.seeds;
    *numSeeds = env.numSeeds;
}
int getQuEST_PREC(void) { return (int)(sizeof(qreal) / 4); }
QuESTEnv createQuESTEnv(void) {
    QuESTEnv env;
    env.rank = 0;
    env.numRanks = 1;
    env.seeds = nullptr;
    env.numSeeds = 0;
    std::call_once(g_initOnce, initRuntime);
    const char* caller = "createQuESTEnv";
    if (!REQUIRE(g_haveGPU, E_NO_GPU)) return env;
    seedQuESTDefault(&env);
    return env;
}
void destroyQuESTEnv(QuESTEnv env) { free(env.seeds); }
void syncQuESTEnv(QuESTEnv env) {
    (void)env;
    QG_CUDA(cudaDeviceSynchronize(), "syncQuESTEnv");
}
int syncQuESTSuccess(int successCode) { return successCode; }
void reportQuESTEnv(QuESTEnv env) {
    (void)env;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, 0);
    printf("EXECUTION ENVIRONMENT:\nRunning locally on one node with GPU (%s, %d SMs)\nNumber of ranks is 1\n"
           "Precision: size of qreal is %zu bytes\n", p.name, p.multiProcessorCount, sizeof(qreal));
}
void getEnvironmentString(QuESTEnv env, char str[200]) {
    (void)env;
    snprintf(str, 200, "CUDA=1 OpenMP=0 MPI=0 threads=1 ranks=1");
}

// ---- registers (QuEST.c:42-86, QuEST_gpu.cu:277-326, 500-519) ----
Qureg createQureg(int numQubits, QuESTEnv env) {
    (void)env;
    const char* caller = "createQureg";
    Qureg q;
    memset(&q, 0, sizeof q);
    if (!REQUIRE(numQubits > 0, E_INVALID_NUM_CREATE_QUBITS)) return q;
    q = allocQureg(numQubits, 0, numQubits, caller);
    if (q.deviceStateVec.real) initZeroState(q);
    return q;
}
Qureg createDensityQureg(int numQubits, QuESTEnv env) {
    (void)env;
    const char* caller = "createDensityQureg";
    Qureg q;
    memset(&q, 0, sizeof q);
    if (!REQUIRE(numQubits > 0, E_INVALID_NUM_CREATE_QUBITS)) return q;
    q = allocQureg(2 * numQubits, 1, numQubits, caller);
    if (q.deviceStateVec.real) initZeroState(q);
    return q;
}
Qureg createCloneQureg(Qureg src, QuESTEnv env) {
    (void)env;
    Qureg q = allocQureg(src.numQubitsInStateVec, src.isDensityMatrix, src.numQubitsRepresented, "createCloneQureg");
    if (q.deviceStateVec.real) cloneQureg(q, src);
    return q;
}
void destroyQureg(Qureg q, QuESTEnv env) {
    (void)env;
    if (!q.deviceStateVec.real) return;
    qg::captureDrop(q.deviceStateVec.real);
    cudaStreamSynchronize(qg::stream());
    bool pinned = true;
    {
        std::lock_guard<std::mutex> lk(g_regMutex);
        auto it = g_pinnedMirror.find(q.deviceStateVec.real);
        if (it != g_pinnedMirror.end()) {
            pinned = it->second;
            g_pinnedMirror.erase(it);
        }
    }
    cudaFree(q.deviceStateVec.real);
    if (pinned) cudaFreeHost(q.stateVec.real);
    else free(q.stateVec.real);
    cudaFree(q.firstLevelReduction);
    cudaFreeHost(q.secondLevelReduction);
}
void copyStateToGPU(Qureg q) {
    discardQ(q);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)q.numAmpsTotal * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.real, q.stateVec.real, b, cudaMemcpyHostToDevice, st), "copyStateToGPU")) return;
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.imag, q.stateVec.imag, b, cudaMemcpyHostToDevice, st), "copyStateToGPU")) return;
    syncStream("copyStateToGPU");
}
void copyStateFromGPU(Qureg q) {
    flushQ(q);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)q.numAmpsTotal * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(q.stateVec.real, q.deviceStateVec.real, b, cudaMemcpyDeviceToHost, st), "copyStateFromGPU")) return;
    if (QG_CUDA(cudaMemcpyAsync(q.stateVec.imag, q.deviceStateVec.imag, b, cudaMemcpyDeviceToHost, st), "copyStateFromGPU")) return;
    syncStream("copyStateFromGPU");
}
void copySubstateToGPU(Qureg q, idx_t start, idx_t n) {
    const char* caller = "copySubstateToGPU";
    if (!vNumAmps(q, start, n, caller)) return;
    flushQ(q);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)n * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.real + start, q.stateVec.real + start, b, cudaMemcpyHostToDevice, st), caller)) return;
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.imag + start, q.stateVec.imag + start, b, cudaMemcpyHostToDevice, st), caller)) return;
    syncStream(caller);
}
void copySubstateFromGPU(Qureg q, idx_t start, idx_t n) {
    const char* caller = "copySubstateFromGPU";
    if (!vNumAmps(q, start, n, caller)) return;
    flushQ(q);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)n * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(q.stateVec.real + start, q.deviceStateVec.real + start, b, cudaMemcpyDeviceToHost, st), caller)) return;
    if (QG_CUDA(cudaMemcpyAsync(q.stateVec.imag + start, q.deviceStateVec.imag + start, b, cudaMemcpyDeviceToHost, st), caller)) return;
    syncStream(caller);
}
int getNumQubits(Qureg q) { return q.numQubitsRepresented; }
idx_t getNumAmps(Qureg q) {
    const char* caller = "getNumAmps";
    if (!vStateVec(q, caller)) return 0;
    return q.numAmpsTotal;
}
ComplexMatrixN createComplexMatrixN(int numQubits) {
    ComplexMatrixN m;
    memset(&m, 0, sizeof m);
    const char* caller = "createComplexMatrixN";
    if (!REQUIRE(numQubits > 0, E_INVALID_NUM_QUBITS)) return m;
    const int d = 1 << numQubits;
    m.numQubits = numQubits;
    m.real = (qreal**)malloc(sizeof(qreal*) * d);
    m.imag = (qreal**)malloc(sizeof(qreal*) * d);
    for (int i = 0; i < d; ++i) {
        m.real[i] = (qreal*)calloc(d, sizeof(qreal));
        m.imag[i] = (qreal*)calloc(d, sizeof(qreal));
    }
    return m;
}
void destroyComplexMatrixN(ComplexMatrixN m) {
    const int d = 1 << m.numQubits;
    for (int i = 0; i < d; ++i) {
        free(m.real[i]);
        free(m.imag[i]);
    }
    free(m.real);
    free(m.imag);
}
PauliHamil createPauliHamil(int numQubits, int numSumTerms) {
    PauliHamil h;
    memset(&h, 0, sizeof h);
    const char* caller = "createPauliHamil";
    if (!REQUIRE(numQubits > 0 && numSumTerms > 0, E_INVALID_PAULI_HAMIL_PARAMS)) return h;
    h.numQubits = numQubits;
    h.numSumTerms = numSumTerms;
    h.pauliCodes = (enum pauliOpType*)calloc((size_t)numQubits * numSumTerms, sizeof(enum pauliOpType));
    h.termCoeffs = (qreal*)calloc(numSumTerms, sizeof(qreal));
    return h;
}
void destroyPauliHamil(PauliHamil h) {
    free(h.pauliCodes);
    free(h.termCoeffs);
}
void initPauliHamil(PauliHamil h, qreal* coeffs, enum pauliOpType* codes) {
    const char* caller = "initPauliHamil";
    if (!REQUIRE(h.numQubits > 0 && h.numSumTerms > 0, E_INVALID_PAULI_HAMIL_PARAMS)) return;
    if (!vPauliCodes(codes, (idx_t)h.numSumTerms * h.numQubits, caller)) return;
    for (int t = 0; t < h.numSumTerms; ++t) {
        h.termCoeffs[t] = coeffs[t];
        for (int i = 0; i < h.numQubits; ++i) h.pauliCodes[t * h.numQubits + i] = codes[t * h.numQubits + i];
    }
}

// ---- initialisation (QuEST.c:119-176) ----
void initBlankState(Qureg q) { qg::stateFill(svOverwrite(q), 0.0, 0.0); }
void initZeroState(Qureg q) {
    qg::stateFill(svOverwrite(q), 0.0, 0.0);
    qg::stateSetOne(sv(q), 0, 1.0, 0.0);
}
void initPlusState(Qureg q) {
    if (q.isDensityMatrix) qg::statePlusDM(svOverwrite(q), q.numQubitsRepresented);
    else qg::stateFill(svOverwrite(q), 1.0 / sqrt((double)q.numAmpsTotal), 0.0);
}
void initClassicalState(Qureg q, idx_t ind) {
    const char* caller = "initClassicalState";
    if (!REQUIRE(ind >= 0 && ind < (1LL << q.numQubitsRepresented), E_INVALID_STATE_INDEX)) return;
    qg::stateFill(svOverwrite(q), 0.0, 0.0);
    const idx_t at = q.isDensityMatrix ? ind * ((1LL << q.numQubitsRepresented) + 1) : ind;
    qg::stateSetOne(sv(q), at, 1.0, 0.0);
}
void initPureState(Qureg q, Qureg pure) {
    const char* caller = "initPureState";
    if (!vSecondStateVec(pure, caller) || !vMatchDims(q, pure, caller)) return;
    flushQ(pure);
    if (q.isDensityMatrix) qg::statePureDM(svOverwrite(q), pure.deviceStateVec.real, pure.deviceStateVec.imag, q.numQubitsRepresented);
    else cloneQureg(q, pure);
}
void initDebugState(Qureg q) { qg::stateDebug(svOverwrite(q)); }

// ---- amplitude-encoded product states (extension) ----
// QuantumLab prepares |0>|v>|u> for its swap tests by amplitude-encoding each
// vector as a circuit of uniformly controlled rotations (AmplitudeEncodeCuda.cu:
// 691-776, FRGate.cu:181-466): device allocations and a host round trip per
// vector, then O(2^d) gates per register.  Applied to |0..0>, that circuit
// prepares v / |v| on the register's qubits.  This call writes the same
// product state directly, in one pass: register r holds its vector's
// normalised amplitudes on qubits [sum of the previous registers' sizes,
// + regQubits[r]); the qubits above the registers are |0>.  (The circuit may
// differ from it by a global phase of each register, which no measurement or
// swap test sees.)
extern "C" int quest_gb300_initProductState(Qureg q, int numRegs, const int* regQubits, const double* re,
                                            const double* im) {
    const char* caller = "initProductState";
    if (!vStateVec(q, caller)) return -1;
    if (!REQUIRE(numRegs >= 1 && numRegs <= 16 && regQubits && re, "Invalid registers. Need 1 to 16 registers and their amplitudes.")) return -1;
    int total = 0;
    size_t len = 0;
    for (int r = 0; r < numRegs; ++r) {
        if (!REQUIRE(regQubits[r] >= 1 && regQubits[r] <= q.numQubitsRepresented, E_INVALID_NUM_TARGETS)) return -1;
        total += regQubits[r];
        len += (size_t)1 << regQubits[r];
    }
    if (!REQUIRE(total <= q.numQubitsRepresented, "Invalid registers. Their qubits exceed the register's.")) return -1;
    std::vector<double> vr(re, re + len), vi(len, 0.0);
    if (im) vi.assign(im, im + len);
    size_t base = 0;
    for (int r = 0; r < numRegs; ++r) {
        const size_t L = (size_t)1 << regQubits[r];
        double nrm = 0;
        for (size_t i = base; i < base + L; ++i) nrm += vr[i] * vr[i] + vi[i] * vi[i];
        if (!REQUIRE(nrm > 0 && std::isfinite(nrm), "Invalid vector. A register's amplitudes must not all be zero.")) return -1;
        const double f = 1.0 / std::sqrt(nrm);
        for (size_t i = base; i < base + L; ++i) {
            vr[i] *= f;
            vi[i] *= f;
        }
        base += L;
    }
    qg::stateProduct(svOverwrite(q), numRegs, regQubits, vr.data(), vi.data());
    return syncStream(caller) ? 0 : -1;
}
void setAmps(Qureg q, idx_t start, qreal* re, qreal* im, idx_t n) {
    const char* caller = "setAmps";
    if (!vStateVec(q, caller) || !vNumAmps(q, start, n, caller)) return;
    flushQ(q);
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.real + start, re, n * sizeof(double), cudaMemcpyHostToDevice, st), caller)) return;
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.imag + start, im, n * sizeof(double), cudaMemcpyHostToDevice, st), caller)) return;
    syncStream(caller);
}
void initStateFromAmps(Qureg q, qreal* re, qreal* im) {                 // QuEST.c:163 (no validation there either)
    const char* caller = "initStateFromAmps";
    discardQ(q);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)q.numAmpsTotal * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.real, re, b, cudaMemcpyHostToDevice, st), caller)) return;
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.imag, im, b, cudaMemcpyHostToDevice, st), caller)) return;
    syncStream(caller);
}
void setDensityAmps(Qureg q, idx_t row, idx_t col, qreal* re, qreal* im, idx_t n) {
    const char* caller = "setDensityAmps";
    if (!vDensity(q, caller) || !vAmpIndex(q, row, caller) || !vAmpIndex(q, col, caller)) return;
    if (!REQUIRE(n >= 0 && n <= q.numAmpsTotal, E_INVALID_NUM_AMPS)) return;
    const idx_t start = row + col * (1LL << q.numQubitsRepresented);
    if (!REQUIRE(n + start <= q.numAmpsTotal, E_INVALID_OFFSET_NUM_AMPS_QUREG)) return;
    flushQ(q);
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.real + start, re, n * sizeof(double), cudaMemcpyHostToDevice, st), caller)) return;
    if (QG_CUDA(cudaMemcpyAsync(q.deviceStateVec.imag + start, im, n * sizeof(double), cudaMemcpyHostToDevice, st), caller)) return;
    syncStream(caller);
}
void cloneQureg(Qureg t, Qureg s) {
    const char* caller = "cloneQureg";
    if (!vMatchTypes(t, s, caller) || !vMatchDims(t, s, caller)) return;
    flushQ(s);
    if (t.deviceStateVec.real != s.deviceStateVec.real) discardQ(t);
    cudaStream_t st = qg::stream();
    const size_t b = (size_t)t.numAmpsTotal * sizeof(double);
    if (QG_CUDA(cudaMemcpyAsync(t.deviceStateVec.real, s.deviceStateVec.real, b, cudaMemcpyDeviceToDevice, st), caller)) return;
    QG_CUDA(cudaMemcpyAsync(t.deviceStateVec.imag, s.deviceStateVec.imag, b, cudaMemcpyDeviceToDevice, st), caller);
}
void setWeightedQureg(Complex f1, Qureg a, Complex f2, Qureg b, Complex fo, Qureg out) {
    const char* caller = "setWeightedQureg";
    if (!vMatchTypes(a, b, caller) || !vMatchTypes(a, out, caller) || !vMatchDims(a, b, caller) || !vMatchDims(a, out, caller)) return;
    qg::stateWeighted(sv(out), f1.real, f1.imag, sv(a), f2.real, f2.imag, sv(b), fo.real, fo.imag);
}

// ---- amplitude access (QuEST.c:940-970, QuEST_gpu.cu:526-582) ----
static Complex readAmp(const Qureg& q, idx_t i, const char* caller) {
    Complex c = {0, 0};
    flushQ(q);
    cudaStream_t st = qg::stream();
    double* slot = q.secondLevelReduction + 8;
    if (QG_CUDA(cudaMemcpyAsync(slot, q.deviceStateVec.real + i, sizeof(double), cudaMemcpyDeviceToHost, st), caller)) return c;
    if (QG_CUDA(cudaMemcpyAsync(slot + 1, q.deviceStateVec.imag + i, sizeof(double), cudaMemcpyDeviceToHost, st), caller)) return c;
    if (!syncStream(caller)) return c;
    c.real = slot[0];
    c.imag = slot[1];
    return c;
}
Complex getAmp(Qureg q, idx_t i) {
    const char* caller = "getAmp";
    Complex z = {0, 0};
    if (!vStateVec(q, caller) || !vAmpIndex(q, i, caller)) return z;
    return readAmp(q, i, caller);
}
qreal getRealAmp(Qureg q, idx_t i) {
    const char* caller = "getRealAmp";
    if (!vStateVec(q, caller) || !vAmpIndex(q, i, caller)) return 0;
    return readAmp(q, i, caller).real;
}
qreal getImagAmp(Qureg q, idx_t i) {
    const char* caller = "getImagAmp";
    if (!vStateVec(q, caller) || !vAmpIndex(q, i, caller)) return 0;
    return readAmp(q, i, caller).imag;
}
qreal getProbAmp(Qureg q, idx_t i) {
    const char* caller = "getProbAmp";
    if (!vStateVec(q, caller) || !vAmpIndex(q, i, caller)) return 0;
    Complex c = readAmp(q, i, caller);
    return c.real * c.real + c.imag * c.imag;
}
Complex getDensityAmp(Qureg q, idx_t r, idx_t c) {
    const char* caller = "getDensityAmp";
    Complex z = {0, 0};
    if (!vDensity(q, caller) || !vAmpIndex(q, r, caller) || !vAmpIndex(q, c, caller)) return z;
    return readAmp(q, r + c * (1LL << q.numQubitsRepresented), caller);
}

// ---- one-qubit gates ----
void hadamard(Qureg q, int t) {                                           // QuEST.c:178
    const char* caller = "hadamard";
    if (!vTarget(q, t, caller)) return;
    qg::gateHadamard(svg(q), t);
    if (q.isDensityMatrix) qg::gateHadamard(svg(q), t + q.numQubitsRepresented);
}
void pauliX(Qureg q, int t) {                                             // QuEST.c:438
    const char* caller = "pauliX";
    if (!vTarget(q, t, caller)) return;
    qg::gateNot(svg(q), 0, 1ull << t);
    if (q.isDensityMatrix) qg::gateNot(svg(q), 0, 1ull << (t + q.numQubitsRepresented));
}
void pauliY(Qureg q, int t) {                                             // QuEST.c:449
    const char* caller = "pauliY";
    if (!vTarget(q, t, caller)) return;
    qg::gatePauliY(svg(q), t, 0, 1.0);
    if (q.isDensityMatrix) qg::gatePauliY(svg(q), t + q.numQubitsRepresented, 0, -1.0);
}
void pauliZ(Qureg q, int t) {
    const char* caller = "pauliZ";
    if (!vTarget(q, t, caller)) return;
    applyPhaseDoubled(q, 1ull << t, -1.0, 0.0);
}
void sGate(Qureg q, int t) {
    const char* caller = "sGate";
    if (!vTarget(q, t, caller)) return;
    applyPhaseDoubled(q, 1ull << t, 0.0, 1.0);
}
void tGate(Qureg q, int t) {
    const char* caller = "tGate";
    if (!vTarget(q, t, caller)) return;
    applyPhaseDoubled(q, 1ull << t, 1 / sqrt(2.0), 1 / sqrt(2.0));
}
void phaseShift(Qureg q, int t, qreal a) {                                // QuEST.c:493
    const char* caller = "phaseShift";
    if (!vTarget(q, t, caller)) return;
    applyPhaseDoubled(q, 1ull << t, cos(a), sin(a));
}
void rotateAroundAxis(Qureg q, int t, qreal angle, Vector axis) {         // QuEST.c:568
    const char* caller = "rotateAroundAxis";
    if (!vTarget(q, t, caller) || !vVector(axis, caller)) return;
    Complex a, b;
    rotationPair(angle, axis, &a, &b);
    applyCompact(q, t, 0, a, b);
}
void rotateX(Qureg q, int t, qreal angle) {
    const char* caller = "rotateX";
    if (!vTarget(q, t, caller)) return;
    Vector v = {1, 0, 0};
    Complex a, b;
    rotationPair(angle, v, &a, &b);
    applyCompact(q, t, 0, a, b);
}
void rotateY(Qureg q, int t, qreal angle) {
    const char* caller = "rotateY";
    if (!vTarget(q, t, caller)) return;
    Vector v = {0, 1, 0};
    Complex a, b;
    rotationPair(angle, v, &a, &b);
    applyCompact(q, t, 0, a, b);
}
void rotateZ(Qureg q, int t, qreal angle) {
    const char* caller = "rotateZ";
    if (!vTarget(q, t, caller)) return;
    Vector v = {0, 0, 1};
    Complex a, b;
    rotationPair(angle, v, &a, &b);
    applyCompact(q, t, 0, a, b);
}
void compactUnitary(Qureg q, int t, Complex a, Complex b) {               // QuEST.c:410
    const char* caller = "compactUnitary";
    if (!vTarget(q, t, caller) || !vPair(a, b, caller)) return;
    applyCompact(q, t, 0, a, b);
}
void unitary(Qureg q, int t, ComplexMatrix2 u) {                          // QuEST.c:354
    const char* caller = "unitary";
    if (!vTarget(q, t, caller) || !vUnitary2(u, caller)) return;
    applyMatrix2Doubled(q, t, 0, 0, u);
}
void applyMatrix2(Qureg q, int t, ComplexMatrix2 u) {                     // QuEST.c:1107 (no DM doubling)
    const char* caller = "applyMatrix2";
    if (!vTarget(q, t, caller)) return;
    qg::gateMatrix2(svg(q), t, 0, 0, toMat(u, false));
}

// ---- controlled gates ----
void controlledNot(Qureg q, int c, int t) {                               // QuEST.c:530
    const char* caller = "controlledNot";
    if (!vControlTarget(q, c, t, caller)) return;
    qg::gateNot(svg(q), 1ull << c, 1ull << t);
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gateNot(svg(q), 1ull << (c + s), 1ull << (t + s));
    }
}
void controlledPauliY(Qureg q, int c, int t) {                            // QuEST.c:568
    const char* caller = "controlledPauliY";
    if (!vControlTarget(q, c, t, caller)) return;
    qg::gatePauliY(svg(q), t, 1ull << c, 1.0);
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gatePauliY(svg(q), t + s, 1ull << (c + s), -1.0);
    }
}
void controlledPhaseShift(Qureg q, int a, int b, qreal angle) {           // QuEST.c:504
    const char* caller = "controlledPhaseShift";
    if (!vControlTarget(q, a, b, caller)) return;
    applyPhaseDoubled(q, (1ull << a) | (1ull << b), cos(angle), sin(angle));
}
void controlledPhaseFlip(Qureg q, int a, int b) {                         // QuEST.c:580
    const char* caller = "controlledPhaseFlip";
    if (!vControlTarget(q, a, b, caller)) return;
    applyPhaseDoubled(q, (1ull << a) | (1ull << b), -1.0, 0.0);
}
void controlledRotateAroundAxis(Qureg q, int c, int t, qreal angle, Vector axis) {
    const char* caller = "controlledRotateAroundAxis";
    if (!vControlTarget(q, c, t, caller) || !vVector(axis, caller)) return;
    Complex a, b;
    rotationPair(angle, axis, &a, &b);
    applyCompact(q, t, 1ull << c, a, b);
}
static void controlledRot(Qureg q, int c, int t, qreal angle, Vector v, const char* caller) {
    if (!vControlTarget(q, c, t, caller)) return;
    Complex a, b;
    rotationPair(angle, v, &a, &b);
    applyCompact(q, t, 1ull << c, a, b);
}
void controlledRotateX(Qureg q, int c, int t, qreal angle) { controlledRot(q, c, t, angle, Vector{1, 0, 0}, "controlledRotateX"); }
void controlledRotateY(Qureg q, int c, int t, qreal angle) { controlledRot(q, c, t, angle, Vector{0, 1, 0}, "controlledRotateY"); }
void controlledRotateZ(Qureg q, int c, int t, qreal angle) { controlledRot(q, c, t, angle, Vector{0, 0, 1}, "controlledRotateZ"); }
void controlledCompactUnitary(Qureg q, int c, int t, Complex a, Complex b) {   // QuEST.c:424
    const char* caller = "controlledCompactUnitary";
    if (!vControlTarget(q, c, t, caller) || !vPair(a, b, caller)) return;
    applyCompact(q, t, 1ull << c, a, b);
}
void controlledUnitary(Qureg q, int c, int t, ComplexMatrix2 u) {         // QuEST.c:366
    const char* caller = "controlledUnitary";
    if (!vControlTarget(q, c, t, caller) || !vUnitary2(u, caller)) return;
    applyMatrix2Doubled(q, t, 1ull << c, 0, u);
}
void multiControlledUnitary(Qureg q, int* cs, int nc, int t, ComplexMatrix2 u) {   // QuEST.c:379
    const char* caller = "multiControlledUnitary";
    if (!vMultiControlsTarget(q, cs, nc, t, caller) || !vUnitary2(u, caller)) return;
    applyMatrix2Doubled(q, t, maskOf(cs, nc), 0, u);
}
void multiStateControlledUnitary(Qureg q, int* cs, int* st, int nc, int t, ComplexMatrix2 u) {   // QuEST.c:394
    const char* caller = "multiStateControlledUnitary";
    if (!vMultiControlsTarget(q, cs, nc, t, caller) || !vUnitary2(u, caller) || !vControlState(st, nc, caller)) return;
    uint64_t flip = 0;
    for (int i = 0; i < nc; ++i)
        if (st[i] == 0) flip |= 1ull << cs[i];
    applyMatrix2Doubled(q, t, maskOf(cs, nc), flip, u);
}
void multiControlledPhaseShift(Qureg q, int* cs, int nc, qreal angle) {   // QuEST.c:516
    const char* caller = "multiControlledPhaseShift";
    if (!vMultiQubits(q, cs, nc, caller)) return;
    applyPhaseDoubled(q, maskOf(cs, nc), cos(angle), sin(angle));
}
void multiControlledPhaseFlip(Qureg q, int* cs, int nc) {                 // QuEST.c:592
    const char* caller = "multiControlledPhaseFlip";
    if (!vMultiQubits(q, cs, nc, caller)) return;
    applyPhaseDoubled(q, maskOf(cs, nc), -1.0, 0.0);
}
void multiQubitNot(Qureg q, int* ts, int nt) {                            // QuEST.c:542
    const char* caller = "multiQubitNot";
    if (!vMultiTargets(q, ts, nt, caller)) return;
    qg::gateNot(svg(q), 0, maskOf(ts, nt));
    if (q.isDensityMatrix) qg::gateNot(svg(q), 0, maskOf(ts, nt) << q.numQubitsRepresented);
}
void multiControlledMultiQubitNot(Qureg q, int* cs, int nc, int* ts, int nt) {   // QuEST.c:555
    const char* caller = "multiControlledMultiQubitNot";
    if (!vMultiControlsMultiTargets(q, cs, nc, ts, nt, caller)) return;
    qg::gateNot(svg(q), maskOf(cs, nc), maskOf(ts, nt));
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gateNot(svg(q), maskOf(cs, nc) << s, maskOf(ts, nt) << s);
    }
}
void swapGate(Qureg q, int a, int b) {                                    // QuEST.c:629
    const char* caller = "swapGate";
    if (!vUniqueTargets(q, a, b, caller)) return;
    qg::gateSwap(svg(q), a, b);
    if (q.isDensityMatrix) qg::gateSwap(svg(q), a + q.numQubitsRepresented, b + q.numQubitsRepresented);
}
void sqrtSwapGate(Qureg q, int a, int b) {                                // QuEST.c:641, QuEST_common.c:386
    const char* caller = "sqrtSwapGate";
    if (!vUniqueTargets(q, a, b, caller) || !vFits(q, 2, caller)) return;
    ComplexMatrix4 u;
    memset(&u, 0, sizeof u);
    u.real[0][0] = 1; u.real[3][3] = 1;
    u.real[1][1] = .5; u.imag[1][1] = .5; u.real[1][2] = .5; u.imag[1][2] = -.5;
    u.real[2][1] = .5; u.imag[2][1] = -.5; u.real[2][2] = .5; u.imag[2][2] = .5;
    qreal *ur[4], *ui[4];
    for (int i = 0; i < 4; ++i) { ur[i] = u.real[i]; ui[i] = u.imag[i]; }
    int ts[2] = {a, b};
    applyMatrixNDoubled(q, 0, ts, 2, ur, ui, true);
}

// ---- multi-qubit gates ----
static void twoQubit(Qureg q, uint64_t ctrl, int t1, int t2, ComplexMatrix4& u, bool doubled) {
    qreal *ur[4], *ui[4];
    for (int i = 0; i < 4; ++i) { ur[i] = u.real[i]; ui[i] = u.imag[i]; }
    int ts[2] = {t1, t2};
    applyMatrixNDoubled(q, ctrl, ts, 2, ur, ui, doubled);
}
void twoQubitUnitary(Qureg q, int t1, int t2, ComplexMatrix4 u) {         // QuEST.c:300
    const char* caller = "twoQubitUnitary";
    int ts[2] = {t1, t2};
    if (!vMultiTargets(q, ts, 2, caller) || !vUnitary4(q, u, caller)) return;
    twoQubit(q, 0, t1, t2, u, true);
}
void controlledTwoQubitUnitary(Qureg q, int c, int t1, int t2, ComplexMatrix4 u) {   // QuEST.c:313
    const char* caller = "controlledTwoQubitUnitary";
    int ts[2] = {t1, t2};
    if (!vMultiControlsMultiTargets(q, &c, 1, ts, 2, caller) || !vUnitary4(q, u, caller)) return;
    twoQubit(q, 1ull << c, t1, t2, u, true);
}
void multiControlledTwoQubitUnitary(Qureg q, int* cs, int nc, int t1, int t2, ComplexMatrix4 u) {
    const char* caller = "multiControlledTwoQubitUnitary";
    int ts[2] = {t1, t2};
    if (!vMultiControlsMultiTargets(q, cs, nc, ts, 2, caller) || !vUnitary4(q, u, caller)) return;
    twoQubit(q, maskOf(cs, nc), t1, t2, u, true);
}
void applyMatrix4(Qureg q, int t1, int t2, ComplexMatrix4 u) {            // QuEST.c:1115 (no DM doubling)
    const char* caller = "applyMatrix4";
    int ts[2] = {t1, t2};
    if (!vMultiTargets(q, ts, 2, caller) || !vFits(q, 2, caller)) return;
    twoQubit(q, 0, t1, t2, u, false);
}
void multiQubitUnitary(Qureg q, int* ts, int k, ComplexMatrixN u) {       // QuEST.c:326
    const char* caller = "multiQubitUnitary";
    if (!vMultiTargets(q, ts, k, caller) || !vUnitaryN(q, u, k, caller)) return;
    applyMatrixNDoubled(q, 0, ts, k, u.real, u.imag, true);
}
void controlledMultiQubitUnitary(Qureg q, int c, int* ts, int k, ComplexMatrixN u) {
    const char* caller = "controlledMultiQubitUnitary";
    if (!vControl(q, c, caller) || !vMultiControlsMultiTargets(q, &c, 1, ts, k, caller) || !vUnitaryN(q, u, k, caller)) return;
    applyMatrixNDoubled(q, 1ull << c, ts, k, u.real, u.imag, true);
}
void multiControlledMultiQubitUnitary(Qureg q, int* cs, int nc, int* ts, int k, ComplexMatrixN u) {
    const char* caller = "multiControlledMultiQubitUnitary";
    if (!vMultiControlsMultiTargets(q, cs, nc, ts, k, caller) || !vUnitaryN(q, u, k, caller)) return;
    applyMatrixNDoubled(q, maskOf(cs, nc), ts, k, u.real, u.imag, true);
}
void applyMatrixN(Qureg q, int* ts, int k, ComplexMatrixN u) {            // QuEST.c:1123
    const char* caller = "applyMatrixN";
    if (!vMultiTargets(q, ts, k, caller) || !vMatrixN(q, u, k, caller)) return;
    applyMatrixNDoubled(q, 0, ts, k, u.real, u.imag, false);
}
void multiRotateZ(Qureg q, int* qs, int n, qreal angle) {                 // QuEST.c:658
    const char* caller = "multiRotateZ";
    if (!vMultiTargets(q, qs, n, caller)) return;
    const uint64_t m = maskOf(qs, n);
    qg::gateRotateZ(svg(q), 0, m, angle);
    if (q.isDensityMatrix) qg::gateRotateZ(svg(q), 0, m << q.numQubitsRepresented, -angle);
}
void multiControlledMultiRotateZ(Qureg q, int* cs, int nc, int* ts, int nt, qreal angle) {   // QuEST.c:673
    const char* caller = "multiControlledMultiRotateZ";
    if (!vMultiControlsMultiTargets(q, cs, nc, ts, nt, caller)) return;
    const uint64_t c = maskOf(cs, nc), m = maskOf(ts, nt);
    qg::gateRotateZ(svg(q), c, m, angle);
    if (q.isDensityMatrix) {
        const int s = q.numQubitsRepresented;
        qg::gateRotateZ(svg(q), c << s, m << s, -angle);
    }
}
void multiRotatePauli(Qureg q, int* ts, enum pauliOpType* ps, int n, qreal angle) {   // QuEST.c:691
    const char* caller = "multiRotatePauli";
    if (!vMultiTargets(q, ts, n, caller) || !vPauliCodes(ps, n, caller)) return;
    applyPauliRotation(q, 0, ts, ps, n, angle);
}
void multiControlledMultiRotatePauli(Qureg q, int* cs, int nc, int* ts, enum pauliOpType* ps, int n, qreal angle) {
    const char* caller = "multiControlledMultiRotatePauli";
    if (!vMultiControlsMultiTargets(q, cs, nc, ts, n, caller) || !vPauliCodes(ps, n, caller)) return;
    applyPauliRotation(q, maskOf(cs, nc), ts, ps, n, angle);
}

// Trotter (QuEST.c:1079 -> QuEST_common.c:762-844)
static void expPauliHamil(const Qureg& q, const PauliHamil& h, double fac, int reverse) {
    int ts[64];
    for (int i = 0; i < h.numQubits; ++i) ts[i] = i;
    for (int i = 0; i < h.numSumTerms; ++i) {
        const int t = reverse ? h.numSumTerms - 1 - i : i;
        applyPauliRotation(q, 0, ts, h.pauliCodes + (idx_t)t * h.numQubits, h.numQubits, 2 * fac * h.termCoeffs[t]);
    }
}
static void symTrotter(const Qureg& q, const PauliHamil& h, double time, int order) {
    if (order == 1) {
        expPauliHamil(q, h, time, 0);
    } else if (order == 2) {
        expPauliHamil(q, h, time / 2., 0);
        expPauliHamil(q, h, time / 2., 1);
    } else {
        const double p = 1. / (4 - pow(4, 1. / (order - 1)));
        const int lo = order - 2;
        symTrotter(q, h, p * time, lo);
        symTrotter(q, h, p * time, lo);
        symTrotter(q, h, (1 - 4 * p) * time, lo);
        symTrotter(q, h, p * time, lo);
        symTrotter(q, h, p * time, lo);
    }
}
void applyTrotterCircuit(Qureg q, PauliHamil h, qreal time, int order, int reps) {
    const char* caller = "applyTrotterCircuit";
    if (!REQUIRE(order == 1 || (order >= 2 && order % 2 == 0), E_INVALID_TROTTER_ORDER)) return;
    if (!REQUIRE(reps >= 1, E_INVALID_TROTTER_REPS)) return;
    if (!vHamil(h, caller)) return;
    if (!REQUIRE(h.numQubits == q.numQubitsRepresented, E_MISMATCHING_PAULI_HAMIL_QUREG_NUM_QUBITS)) return;
    if (time == 0) return;
    for (int r = 0; r < reps; ++r) symTrotter(q, h, time / reps, order);
}

// ---- measurement (QuEST.c:972-1016, QuEST_common.c:165-180, 361-375) ----
qreal collapseToOutcome(Qureg q, int t, int outcome) {
    const char* caller = "collapseToOutcome";
    if (!vTarget(q, t, caller) || !vOutcome(outcome, caller)) return 0;
    const double p0 = probZero(q, t);
    const double p = outcome == 0 ? p0 : 1 - p0;
    if (!REQUIRE(p > REAL_EPS, E_COLLAPSE_STATE_ZERO_PROB)) return 0;
    collapse(q, t, outcome, p);
    return p;
}
int measureWithStats(Qureg q, int t, qreal* outcomeProb) {
    const char* caller = "measureWithStats";
    if (!vTarget(q, t, caller)) return 0;
    const double p0 = probZero(q, t);
    int outcome;
    if (p0 < REAL_EPS) outcome = 1;
    else if (1 - p0 < REAL_EPS) outcome = 0;
    else outcome = (g_mt.real1() > p0);
    *outcomeProb = outcome == 0 ? p0 : 1 - p0;
    collapse(q, t, outcome, *outcomeProb);
    return outcome;
}
int measure(Qureg q, int t) {
    const char* caller = "measure";
    if (!vTarget(q, t, caller)) return 0;
    qreal p;
    return measureWithStats(q, t, &p);
}

// ---- repeated measurement without a state copy per shot (extension) ----
// QuantumLab samples a register by repeating, shot after shot, "measure each
// listed qubit in order" and restoring the pre-measurement state with
// copyStateToGPU before every shot but the first
// (Code/QuantumLab/Simulator/QLSimulatorMeasure.cpp:70-109): a full host ->
// device copy and k reductions per shot.  Measuring qubit j after outcomes
// o_0..o_{j-1} has P(0) = the conditional probability of 0 given those
// outcomes, and QuEST's rule (QuEST_common.c:165-180: outcome 1 if P0 <
// REAL_EPS, 0 if 1 - P0 < REAL_EPS, else genrand_real1() > P0) consumes one
// draw of the global MT19937 stream only when the outcome is not certain.
// So one histogram of the 2^k joint outcomes, reduced once on the device, and
// a tree of its partial sums give every shot's conditional probabilities on
// the host; with the same draws the outcomes are those of the loop (up to the
// rounding of P0, which can matter only for a draw within ~1e-15 of it).
extern "C" int quest_gb300_sampleMeasurements(Qureg q, const int* qubits, int numQubits, int numShots, int* outcomes) {
    const char* caller = "sampleMeasurements";
    if (!vMultiTargets(q, qubits, numQubits, caller)) return -1;
    if (!REQUIRE(numQubits <= 24, "Invalid number of measured qubits. Must be >0 and <=24.")) return -1;
    if (!REQUIRE(numShots >= 0 && (numShots == 0 || outcomes), "Invalid number of shots. Must be >=0, with an output array.")) return -1;
    const size_t M = (size_t)1 << numQubits;
    // tree[j] (offset 2^j - 1): mass of every assignment of the first j listed
    // qubits (bit i of the index = qubit i's outcome); tree level numQubits
    // is the histogram itself
    std::vector<double> tree(2 * M - 1);
    double* hist = tree.data() + (M - 1);
    qg::reduceProbAllOutcomes(sv(q), q.isDensityMatrix, q.numQubitsRepresented, qubits, numQubits, hist,
                              qg::scratchOf(q));
    for (int j = numQubits - 1; j >= 0; --j) {
        const size_t n = (size_t)1 << j;
        double* lvl = tree.data() + (n - 1);
        const double* up = tree.data() + (2 * n - 1);
        for (size_t pfx = 0; pfx < n; ++pfx) lvl[pfx] = up[pfx] + up[pfx + n];
    }
    for (int shot = 0; shot < numShots; ++shot) {
        size_t pfx = 0;
        int code = 0;
        for (int j = 0; j < numQubits; ++j) {
            const size_t n = (size_t)1 << j;
            const double mass = tree[(n - 1) + pfx];
            const double p0 = mass > 0 ? tree[(2 * n - 1) + pfx] / mass : 0.0;
            int o;
            if (p0 < REAL_EPS) o = 1;
            else if (1 - p0 < REAL_EPS) o = 0;
            else o = (g_mt.real1() > p0);
            if (o) {
                pfx |= n;
                code |= 1 << j;
            }
        }
        outcomes[shot] = code;
    }
    return 0;
}

// ---- reductions ----
qreal calcTotalProb(Qureg q) {                                            // QuEST.c:1152
    if (q.isDensityMatrix) return qg::reduceTotalProbDM(sv(q), q.numQubitsRepresented, qg::scratchOf(q));
    return qg::reduceTotalProbSV(sv(q), qg::scratchOf(q));
}
qreal calcProbOfOutcome(Qureg q, int t, int outcome) {                    // QuEST.c:1175
    const char* caller = "calcProbOfOutcome";
    if (!vTarget(q, t, caller) || !vOutcome(outcome, caller)) return 0;
    const double p0 = probZero(q, t);
    return outcome == 0 ? p0 : 1 - p0;
}
void calcProbOfAllOutcomes(qreal* out, Qureg q, int* qs, int nq) {        // QuEST.c:1185
    const char* caller = "calcProbOfAllOutcomes";
    if (!vMultiTargets(q, qs, nq, caller)) return;
    if (!REQUIRE(nq <= 30, E_INVALID_NUM_TARGETS)) return;
    qg::reduceProbAllOutcomes(sv(q), q.isDensityMatrix, q.numQubitsRepresented, qs, nq, out, qg::scratchOf(q));
}
Complex calcInnerProduct(Qureg bra, Qureg ket) {                          // QuEST.c:1159
    const char* caller = "calcInnerProduct";
    Complex z = {0, 0};
    if (!vStateVec(bra, caller) || !vStateVec(ket, caller) || !vMatchDims(bra, ket, caller)) return z;
    qg::reduceInnerProduct(sv(bra), sv(ket), qg::scratchOf(bra), &z.real, &z.imag);
    return z;
}
qreal calcDensityInnerProduct(Qureg a, Qureg b) {                         // QuEST.c:1167
    const char* caller = "calcDensityInnerProduct";
    if (!vDensity(a, caller) || !vDensity(b, caller) || !vMatchDims(a, b, caller)) return 0;
    return qg::reduceDotReal(sv(a), sv(b), qg::scratchOf(a));
}
qreal calcPurity(Qureg q) {                                               // QuEST.c:1194
    const char* caller = "calcPurity";
    if (!vDensity(q, caller)) return 0;
    return qg::reduceNormSq(sv(q), qg::scratchOf(q));
}
qreal calcFidelity(Qureg q, Qureg pure) {                                 // QuEST.c:1200
    const char* caller = "calcFidelity";
    if (!vSecondStateVec(pure, caller) || !vMatchDims(q, pure, caller)) return 0;
    if (q.isDensityMatrix) return qg::reduceFidelityDM(sv(q), sv(pure), q.numQubitsRepresented, qg::scratchOf(q));
    Complex z;
    qg::reduceInnerProduct(sv(q), sv(pure), qg::scratchOf(q), &z.real, &z.imag);
    return z.real * z.real + z.imag * z.imag;
}
qreal calcHilbertSchmidtDistance(Qureg a, Qureg b) {                      // QuEST.c:1245
    const char* caller = "calcHilbertSchmidtDistance";
    if (!vDensity(a, caller) || !vDensity(b, caller) || !vMatchDims(a, b, caller)) return 0;
    return sqrt(qg::reduceDistSq(sv(a), sv(b), qg::scratchOf(a)));
}

// Pauli expectation values: terms grouped by X/Y support, one read per group
static double expecTerms(const Qureg& q, const enum pauliOpType* codes, const qreal* coeffs, int numTerms,
                         const int* targets, int numTargets) {
    std::map<uint64_t, std::vector<qg::PauliTerm>> groups;
    double identity = 0;
    for (int t = 0; t < numTerms; ++t) {
        uint64_t x, y, z;
        pauliMasks(targets, codes + (idx_t)t * numTargets, numTargets, &x, &y, &z);
        const double c = coeffs ? coeffs[t] : 1.0;
        if ((x | z) == 0) {               // identity term: <I> = Tr(rho) or <psi|psi>
            identity += c;
            continue;
        }
        groups[x].push_back(qg::PauliTerm{y | z, __builtin_popcountll(y), c});
    }
    double total = 0;
    if (identity != 0) total += identity * calcTotalProb(q);
    std::vector<qg::PauliTermGroup> list;
    list.reserve(groups.size());
    for (auto& g : groups) list.push_back(qg::PauliTermGroup{g.first, std::move(g.second)});
    total += qg::reduceExpecPauliGroups(sv(q), q.isDensityMatrix, q.numQubitsRepresented, list, qg::scratchOf(q));
    return total;
}
qreal calcExpecPauliProd(Qureg q, int* ts, enum pauliOpType* ps, int n, Qureg ws) {   // QuEST.c:1208
    const char* caller = "calcExpecPauliProd";
    if (!vMultiTargets(q, ts, n, caller) || !vPauliCodes(ps, n, caller) || !vMatchTypes(q, ws, caller) ||
        !vMatchDims(q, ws, caller))
        return 0;
    return expecTerms(q, ps, nullptr, 1, ts, n);
}
qreal calcExpecPauliSum(Qureg q, enum pauliOpType* codes, qreal* coeffs, int nt, Qureg ws) {   // QuEST.c:1219
    const char* caller = "calcExpecPauliSum";
    if (!REQUIRE(nt > 0, E_INVALID_NUM_SUM_TERMS) || !vPauliCodes(codes, (idx_t)nt * q.numQubitsRepresented, caller) ||
        !vMatchTypes(q, ws, caller) || !vMatchDims(q, ws, caller))
        return 0;
    int ts[64];
    for (int i = 0; i < q.numQubitsRepresented; ++i) ts[i] = i;
    return expecTerms(q, codes, coeffs, nt, ts, q.numQubitsRepresented);
}
qreal calcExpecPauliHamil(Qureg q, PauliHamil h, Qureg ws) {              // QuEST.c:1230
    const char* caller = "calcExpecPauliHamil";
    if (!vMatchTypes(q, ws, caller) || !vMatchDims(q, ws, caller) || !vHamil(h, caller)) return 0;
    if (!REQUIRE(h.numQubits == q.numQubitsRepresented, E_MISMATCHING_PAULI_HAMIL_QUREG_NUM_QUBITS)) return 0;
    int ts[64];
    for (int i = 0; i < q.numQubitsRepresented; ++i) ts[i] = i;
    return expecTerms(q, h.pauliCodes, h.termCoeffs, h.numSumTerms, ts, h.numQubits);
}

// ---- decoherence (QuEST.c:1259-1298) ----
void mixDephasing(Qureg q, int t, qreal p) {
    const char* caller = "mixDephasing";
    if (!vDensity(q, caller) || !vTarget(q, t, caller) || !vProb(p, caller) ||
        !REQUIRE(p <= 1 / 2.0, E_INVALID_ONE_QUBIT_DEPHASE_PROB))
        return;
    qg::dmDephase(svg(q), t, q.numQubitsRepresented, 1 - 2 * p);
}
void mixDepolarising(Qureg q, int t, qreal p) {
    const char* caller = "mixDepolarising";
    if (!vDensity(q, caller) || !vTarget(q, t, caller) || !vProb(p, caller) ||
        !REQUIRE(p <= 3 / 4.0, E_INVALID_ONE_QUBIT_DEPOL_PROB))
        return;
    const double level = (4 * p) / 3.0;
    if (level == 0) return;                                   // QuEST_gpu.cu:3029-3030
    qg::dmDepolarise(svg(q), t, q.numQubitsRepresented, level);
}
void mixDamping(Qureg q, int t, qreal p) {
    const char* caller = "mixDamping";
    if (!vDensity(q, caller) || !vTarget(q, t, caller) || !vProb(p, caller) ||
        !REQUIRE(p <= 1.0, E_INVALID_ONE_QUBIT_DEPOL_PROB))
        return;
    if (p == 0) return;                                       // QuEST_gpu.cu:3055-3056
    qg::dmDamp(svg(q), t, q.numQubitsRepresented, p);
}
void mixPauli(Qureg q, int t, qreal pX, qreal pY, qreal pZ) {            // QuEST.c:1312
    const char* caller = "mixPauli";
    if (!vDensity(q, caller) || !vTarget(q, t, caller) || !vProb(pX, caller) || !vProb(pY, caller) ||
        !vProb(pZ, caller))
        return;
    const double none = 1 - pX - pY - pZ;                     // QuEST_validation.c:634-643
    if (!REQUIRE(pX <= none && pY <= none && pZ <= none, E_INVALID_ONE_QUBIT_PAULI_PROBS)) return;
    qg::dmPauli(svg(q), t, q.numQubitsRepresented, pX, pY, pZ);
}
void mixTwoQubitDephasing(Qureg q, int q1, int q2, qreal p) {             // QuEST.c:1269
    const char* caller = "mixTwoQubitDephasing";
    if (!vDensity(q, caller) || !vUniqueTargets(q, q1, q2, caller) || !vProb(p, caller) ||
        !REQUIRE(p <= 3 / 4.0, E_INVALID_TWO_QUBIT_DEPHASE_PROB))
        return;
    if (q1 > q2) std::swap(q1, q2);
    const double dephase = (4 * p) / 3.0;
    if (dephase == 0) return;                                 // QuEST_gpu.cu:2939-2940
    qg::dmTwoQubitDephase(svg(q), q1, q2, q.numQubitsRepresented, 1 - dephase);
}
void mixTwoQubitDepolarising(Qureg q, int q1, int q2, qreal p) {          // QuEST.c:1300
    const char* caller = "mixTwoQubitDepolarising";
    if (!vDensity(q, caller) || !vUniqueTargets(q, q1, q2, caller) || !vProb(p, caller) ||
        !REQUIRE(p <= 15 / 16.0, E_INVALID_TWO_QUBIT_DEPOL_PROB))
        return;
    if (q1 > q2) std::swap(q1, q2);
    const double level = (16 * p) / 15.0;
    if (level == 0) return;                                   // QuEST_gpu.cu:3114-3115
    qg::dmTwoQubitDepolarise(svg(q), q1, q2, q.numQubitsRepresented, level);
}
void mixDensityMatrix(Qureg a, qreal p, Qureg b) {                        // QuEST.c:1018
    const char* caller = "mixDensityMatrix";
    if (!vDensity(a, caller) || !vDensity(b, caller) || !vMatchDims(a, b, caller) || !vProb(p, caller)) return;
    qg::stateMixDM(sv(a), p, sv(b));
}

int quest_gb300_hostMirrorPinned(Qureg q) {
    std::lock_guard<std::mutex> lk(g_regMutex);
    auto it = g_pinnedMirror.find(q.deviceStateVec.real);
    return it == g_pinnedMirror.end() ? -1 : (it->second ? 1 : 0);
}

// ---- QASM: recording is not supported; calls are accepted and ignored ----
void startRecordingQASM(Qureg q) { (void)q; }
void stopRecordingQASM(Qureg q) { (void)q; }
void clearRecordedQASM(Qureg q) { (void)q; }
void printRecordedQASM(Qureg q) { (void)q; }
void writeRecordedQASMToFile(Qureg q, char* filename) { (void)q; (void)filename; }

// ---- reports (QuEST.c:1605-1640; plain text, this library's own layout) ----
void reportQuregParams(Qureg q) {
    printf("QUBITS:\nNumber of qubits is %d.\nNumber of amps is %lld.\nNumber of amps per rank is %lld.\n",
           q.numQubitsRepresented, q.numAmpsTotal, q.numAmpsPerChunk);
}
void reportStateToScreen(Qureg q, QuESTEnv env, int reportRank) {
    (void)env; (void)reportRank;
    copyStateFromGPU(q);
    printf("Reporting state [\n");
    for (idx_t i = 0; i < q.numAmpsTotal; ++i) printf("%.14f, %.14f\n", q.stateVec.real[i], q.stateVec.imag[i]);
    printf("]\n");
}
void reportState(Qureg q) {
    copyStateFromGPU(q);
    FILE* f = fopen("state_rank_0.csv", "w");
    if (!f) return;
    fprintf(f, "real, imag\n");
    for (idx_t i = 0; i < q.numAmpsTotal; ++i) fprintf(f, "%.14f, %.14f\n", q.stateVec.real[i], q.stateVec.imag[i]);
    fclose(f);
}
void reportPauliHamil(PauliHamil h) {
    for (int t = 0; t < h.numSumTerms; ++t) {
        printf("%.14f\t", h.termCoeffs[t]);
        for (int k = 0; k < h.numQubits; ++k) printf("%d ", (int)h.pauliCodes[(idx_t)t * h.numQubits + k]);
        printf("\n");
    }
}

// ---- the rest of the QuEST 3.4 API (reference QuEST.h): not on the
// simulation path this library serves; each reports E_UNSUPPORTED through
// invalidQuESTInputError and leaves its arguments untouched ----
#define QG_UNSUPPORTED() invalidQuESTInputError(E_UNSUPPORTED, __func__)
void mixKrausMap(Qureg, int, ComplexMatrix2*, int) { QG_UNSUPPORTED(); }
void mixTwoQubitKrausMap(Qureg, int, int, ComplexMatrix4*, int) { QG_UNSUPPORTED(); }
void mixMultiQubitKrausMap(Qureg, int*, int, ComplexMatrixN*, int) { QG_UNSUPPORTED(); }
void mixNonTPKrausMap(Qureg, int, ComplexMatrix2*, int) { QG_UNSUPPORTED(); }
void mixNonTPTwoQubitKrausMap(Qureg, int, int, ComplexMatrix4*, int) { QG_UNSUPPORTED(); }
void mixNonTPMultiQubitKrausMap(Qureg, int*, int, ComplexMatrixN*, int) { QG_UNSUPPORTED(); }
void applyPauliSum(Qureg, enum pauliOpType*, qreal*, int, Qureg) { QG_UNSUPPORTED(); }
void applyPauliHamil(Qureg, PauliHamil, Qureg) { QG_UNSUPPORTED(); }
void applyMultiControlledMatrixN(Qureg, int*, int, int*, int, ComplexMatrixN) { QG_UNSUPPORTED(); }
void applyProjector(Qureg, int, int) { QG_UNSUPPORTED(); }
void applyQFT(Qureg, int*, int) { QG_UNSUPPORTED(); }
void applyFullQFT(Qureg) { QG_UNSUPPORTED(); }
void applyPhaseFunc(Qureg, int*, int, enum bitEncoding, qreal*, qreal*, int) { QG_UNSUPPORTED(); }
void applyPhaseFuncOverrides(Qureg, int*, int, enum bitEncoding, qreal*, qreal*, int, long long*, qreal*, int) {
    QG_UNSUPPORTED();
}
void applyMultiVarPhaseFunc(Qureg, int*, int*, int, enum bitEncoding, qreal*, qreal*, int*) { QG_UNSUPPORTED(); }
void applyMultiVarPhaseFuncOverrides(Qureg, int*, int*, int, enum bitEncoding, qreal*, qreal*, int*, long long*,
                                     qreal*, int) {
    QG_UNSUPPORTED();
}
void applyNamedPhaseFunc(Qureg, int*, int*, int, enum bitEncoding, enum phaseFunc) { QG_UNSUPPORTED(); }
void applyNamedPhaseFuncOverrides(Qureg, int*, int*, int, enum bitEncoding, enum phaseFunc, long long*, qreal*, int) {
    QG_UNSUPPORTED();
}
void applyParamNamedPhaseFunc(Qureg, int*, int*, int, enum bitEncoding, enum phaseFunc, qreal*, int) {
    QG_UNSUPPORTED();
}
void applyParamNamedPhaseFuncOverrides(Qureg, int*, int*, int, enum bitEncoding, enum phaseFunc, qreal*, int,
                                       long long*, qreal*, int) {
    QG_UNSUPPORTED();
}
DiagonalOp createDiagonalOp(int, QuESTEnv) {
    QG_UNSUPPORTED();
    return DiagonalOp{};
}
DiagonalOp createDiagonalOpFromPauliHamilFile(char*, QuESTEnv) {
    QG_UNSUPPORTED();
    return DiagonalOp{};
}
void destroyDiagonalOp(DiagonalOp, QuESTEnv) { QG_UNSUPPORTED(); }
void syncDiagonalOp(DiagonalOp) { QG_UNSUPPORTED(); }
void initDiagonalOp(DiagonalOp, qreal*, qreal*) { QG_UNSUPPORTED(); }
void initDiagonalOpFromPauliHamil(DiagonalOp, PauliHamil) { QG_UNSUPPORTED(); }
void setDiagonalOpElems(DiagonalOp, long long, qreal*, qreal*, long long) { QG_UNSUPPORTED(); }
void applyDiagonalOp(Qureg, DiagonalOp) { QG_UNSUPPORTED(); }
Complex calcExpecDiagonalOp(Qureg, DiagonalOp) {
    QG_UNSUPPORTED();
    return Complex{0, 0};
}
PauliHamil createPauliHamilFromFile(char*) {
    QG_UNSUPPORTED();
    return PauliHamil{};
}
// C-only helpers (their reference prototypes take variable-length 2D arrays,
// which decay to pointers to contiguous rows of 2^numQubits entries)
void initComplexMatrixN(ComplexMatrixN m, qreal* real, qreal* imag) {
    const char* caller = "initComplexMatrixN";
    if (!REQUIRE(m.real != nullptr && m.imag != nullptr, E_COMPLEX_MATRIX_NOT_INIT)) return;
    const int D = 1 << m.numQubits;
    for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) {
            m.real[r][c] = real[(size_t)r * D + c];
            m.imag[r][c] = imag[(size_t)r * D + c];
        }
}
ComplexMatrixN bindArraysToStackComplexMatrixN(int numQubits, qreal* re, qreal* im, qreal** reStorage,
                                               qreal** imStorage) {
    const int D = 1 << numQubits;
    for (int r = 0; r < D; ++r) {
        reStorage[r] = re + (size_t)r * D;
        imStorage[r] = im + (size_t)r * D;
    }
    ComplexMatrixN m;
    m.numQubits = numQubits;
    m.real = reStorage;
    m.imag = imStorage;
    return m;
}

}  // extern "C"
