/*
 * quest_oracle.c -- TEST INFRASTRUCTURE, not the product.
 *
 * A plain-C (OpenMP) restatement of the QuEST 3.4 CPU backend for the
 * functions on the simulation hot path, exported behind the same C ABI as the
 * product (include/QuEST.h).  It is the FP64 checker for the GPU library: the
 * parity tests, __graft_entry__.smoke() and bench.py's CPU baseline are the
 * only callers.  It is pinned against golden vectors produced by the
 * reference's own QuEST CPU build (tests/golden/make_golden.py).
 *
 * Each function cites the reference routine whose arithmetic it follows
 * (paths relative to Code/QuEST340/QuEST/src).  The loops enumerate the
 * touched amplitudes directly (bit insertion) instead of the reference's
 * block/offset arithmetic; the per-amplitude formulas are the reference's.
 *
 * Host arrays only: deviceStateVec aliases stateVec, and copyStateToGPU /
 * copyStateFromGPU are no-ops.
 */
#include "QuEST.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <unistd.h>

typedef long long int idx_t;

/* ------------------------------------------------------------------------ */
/* error hook (QuEST_validation.c:216-243)                                   */
/* ------------------------------------------------------------------------ */
pfinvalidQuESTInputError __other_input_error = NULL;

__attribute__((weak)) void invalidQuESTInputError(const char* errMsg, const char* errFunc) {
    if (__other_input_error) { __other_input_error(errMsg, errFunc); return; }
    printf("!!!\nQuEST Error in function %s: %s\n!!!\nexiting..\n", errFunc, errMsg);
    exit(EXIT_FAILURE);
}

static int fail(const char* msg, const char* fn) { invalidQuESTInputError(msg, fn); return 1; }
#define CHECK(cond, msg) do { if (!(cond)) { fail(msg, __func__); return; } } while (0)
#define CHECKR(cond, msg, rv) do { if (!(cond)) { fail(msg, __func__); return rv; } } while (0)

/* ------------------------------------------------------------------------ */
/* MT19937 (Matsumoto & Nishimura 1998, published algorithm): used only by  */
/* measure(), as in QuEST_common.c:165-180 + mt19937ar.c                     */
/* ------------------------------------------------------------------------ */
#define MT_N 624
#define MT_M 397
static unsigned long mt_state[MT_N];
static int mt_pos = MT_N + 1;

static void mt_seed(unsigned long s) {
    mt_state[0] = s & 0xffffffffUL;
    for (int i = 1; i < MT_N; i++) {
        mt_state[i] = (1812433253UL * (mt_state[i - 1] ^ (mt_state[i - 1] >> 30)) + (unsigned long)i);
        mt_state[i] &= 0xffffffffUL;
    }
    mt_pos = MT_N;
}

static void mt_seed_array(unsigned long* key, int len) {
    mt_seed(19650218UL);
    int i = 1, j = 0;
    for (int k = (MT_N > len ? MT_N : len); k; k--) {
        mt_state[i] = (mt_state[i] ^ ((mt_state[i - 1] ^ (mt_state[i - 1] >> 30)) * 1664525UL)) + key[j] + (unsigned long)j;
        mt_state[i] &= 0xffffffffUL;
        i++; j++;
        if (i >= MT_N) { mt_state[0] = mt_state[MT_N - 1]; i = 1; }
        if (j >= len) j = 0;
    }
    for (int k = MT_N - 1; k; k--) {
        mt_state[i] = (mt_state[i] ^ ((mt_state[i - 1] ^ (mt_state[i - 1] >> 30)) * 1566083941UL)) - (unsigned long)i;
        mt_state[i] &= 0xffffffffUL;
        i++;
        if (i >= MT_N) { mt_state[0] = mt_state[MT_N - 1]; i = 1; }
    }
    mt_state[0] = 0x80000000UL;
}

static unsigned long mt_next32(void) {
    static const unsigned long mag[2] = {0x0UL, 0x9908b0dfUL};
    if (mt_pos >= MT_N) {
        if (mt_pos == MT_N + 1) mt_seed(5489UL);
        int k;
        for (k = 0; k < MT_N - MT_M; k++) {
            unsigned long y = (mt_state[k] & 0x80000000UL) | (mt_state[k + 1] & 0x7fffffffUL);
            mt_state[k] = mt_state[k + MT_M] ^ (y >> 1) ^ mag[y & 1UL];
        }
        for (; k < MT_N - 1; k++) {
            unsigned long y = (mt_state[k] & 0x80000000UL) | (mt_state[k + 1] & 0x7fffffffUL);
            mt_state[k] = mt_state[k + (MT_M - MT_N)] ^ (y >> 1) ^ mag[y & 1UL];
        }
        unsigned long y = (mt_state[MT_N - 1] & 0x80000000UL) | (mt_state[0] & 0x7fffffffUL);
        mt_state[MT_N - 1] = mt_state[MT_M - 1] ^ (y >> 1) ^ mag[y & 1UL];
        mt_pos = 0;
    }
    unsigned long y = mt_state[mt_pos++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680UL;
    y ^= (y << 15) & 0xefc60000UL;
    y ^= (y >> 18);
    return y;
}
/* uniform on [0,1] with 32-bit resolution */
static double mt_real1(void) { return (double)mt_next32() * (1.0 / 4294967295.0); }

/* ------------------------------------------------------------------------ */
/* index helpers                                                              */
/* ------------------------------------------------------------------------ */
static inline idx_t ins0(idx_t x, int b) {           /* insert a 0 bit at position b */
    idx_t lo = x & ((1LL << b) - 1);
    return ((x >> b) << (b + 1)) | lo;
}
static idx_t maskOf(const int* qs, int n) { idx_t m = 0; for (int i = 0; i < n; i++) m |= 1LL << qs[i]; return m; }
static int parity(idx_t x) { return __builtin_parityll((unsigned long long)x); }

/* ------------------------------------------------------------------------ */
/* environment                                                                */
/* ------------------------------------------------------------------------ */
void seedQuEST(QuESTEnv* env, unsigned long int* seedArray, int numSeeds) {   /* QuEST_gpu.cu:3970-3984 */
    if (env->seeds) free(env->seeds);
    env->seeds = (unsigned long*)malloc(sizeof(unsigned long) * (numSeeds > 0 ? numSeeds : 1));
    for (int i = 0; i < numSeeds; i++) env->seeds[i] = seedArray[i];
    env->numSeeds = numSeeds;
    mt_seed_array(seedArray, numSeeds);
}
void seedQuESTDefault(QuESTEnv* env) {                                          /* QuEST.c:1653, QuEST_common.c:192-214 */
    struct timeval tv; gettimeofday(&tv, NULL);
    unsigned long keys[2] = {(unsigned long)(tv.tv_sec * 1000 + tv.tv_usec / 1000), (unsigned long)getpid()};
    seedQuEST(env, keys, 2);
}
void getQuESTSeeds(QuESTEnv env, unsigned long int** seeds, int* numSeeds) { *seeds = env.seeds; *numSeeds = env.numSeeds; }
int getQuEST_PREC(void) { return (int)(sizeof(qreal) / 4); }
QuESTEnv createQuESTEnv(void) {
    QuESTEnv env; env.rank = 0; env.numRanks = 1; env.seeds = NULL; env.numSeeds = 0;
    seedQuESTDefault(&env);
    return env;
}
void destroyQuESTEnv(QuESTEnv env) { free(env.seeds); }
void syncQuESTEnv(QuESTEnv env) { (void)env; }
int syncQuESTSuccess(int successCode) { return successCode; }
void reportQuESTEnv(QuESTEnv env) { (void)env; printf("EXECUTION ENVIRONMENT:\nRunning the CPU oracle\n"); }
void getEnvironmentString(QuESTEnv env, char str[200]) { (void)env; snprintf(str, 200, "CPU oracle, OpenMP"); }

/* ------------------------------------------------------------------------ */
/* registers                                                                  */
/* ------------------------------------------------------------------------ */
static Qureg makeQureg(int nsv, int isDM, int nrep) {                           /* QuEST_cpu.c:1297-1330 */
    Qureg q; memset(&q, 0, sizeof q);
    idx_t n = 1LL << nsv;
    q.isDensityMatrix = isDM; q.numQubitsRepresented = nrep; q.numQubitsInStateVec = nsv;
    q.numAmpsPerChunk = n; q.numAmpsTotal = n; q.chunkId = 0; q.numChunks = 1;
    q.stateVec.real = (qreal*)malloc(sizeof(qreal) * n);
    q.stateVec.imag = (qreal*)malloc(sizeof(qreal) * n);
    q.deviceStateVec = q.stateVec;
    return q;
}
void initZeroState(Qureg q);
Qureg createQureg(int numQubits, QuESTEnv env) {                                /* QuEST.c:42-54 */
    (void)env;
    Qureg q; memset(&q, 0, sizeof q);
    CHECKR(numQubits > 0, "Invalid number of qubits. Must create >0.", q);
    q = makeQureg(numQubits, 0, numQubits);
    initZeroState(q);
    return q;
}
Qureg createDensityQureg(int numQubits, QuESTEnv env) {                         /* QuEST.c:56-68 */
    (void)env;
    Qureg q; memset(&q, 0, sizeof q);
    CHECKR(numQubits > 0, "Invalid number of qubits. Must create >0.", q);
    q = makeQureg(2 * numQubits, 1, numQubits);
    initZeroState(q);
    return q;
}
Qureg createCloneQureg(Qureg src, QuESTEnv env) {                               /* QuEST.c:70-81 */
    (void)env;
    Qureg q = makeQureg(src.numQubitsInStateVec, src.isDensityMatrix, src.numQubitsRepresented);
    memcpy(q.stateVec.real, src.stateVec.real, sizeof(qreal) * q.numAmpsTotal);
    memcpy(q.stateVec.imag, src.stateVec.imag, sizeof(qreal) * q.numAmpsTotal);
    return q;
}
void destroyQureg(Qureg q, QuESTEnv env) { (void)env; free(q.stateVec.real); free(q.stateVec.imag); }
void copyStateToGPU(Qureg q) { (void)q; }
void copyStateFromGPU(Qureg q) { (void)q; }
void copySubstateToGPU(Qureg q, idx_t s, idx_t n) { (void)q; (void)s; (void)n; }
void copySubstateFromGPU(Qureg q, idx_t s, idx_t n) { (void)q; (void)s; (void)n; }
int getNumQubits(Qureg q) { return q.numQubitsRepresented; }
idx_t getNumAmps(Qureg q) { return q.numAmpsTotal; }

ComplexMatrixN createComplexMatrixN(int numQubits) {
    ComplexMatrixN m; int d = 1 << numQubits;
    m.numQubits = numQubits;
    m.real = (qreal**)malloc(sizeof(qreal*) * d);
    m.imag = (qreal**)malloc(sizeof(qreal*) * d);
    for (int i = 0; i < d; i++) { m.real[i] = (qreal*)calloc(d, sizeof(qreal)); m.imag[i] = (qreal*)calloc(d, sizeof(qreal)); }
    return m;
}
void destroyComplexMatrixN(ComplexMatrixN m) {
    int d = 1 << m.numQubits;
    for (int i = 0; i < d; i++) { free(m.real[i]); free(m.imag[i]); }
    free(m.real); free(m.imag);
}
PauliHamil createPauliHamil(int numQubits, int numSumTerms) {
    PauliHamil h; h.numQubits = numQubits; h.numSumTerms = numSumTerms;
    h.pauliCodes = (enum pauliOpType*)calloc((size_t)numQubits * numSumTerms, sizeof(enum pauliOpType));
    h.termCoeffs = (qreal*)calloc(numSumTerms, sizeof(qreal));
    return h;
}
void destroyPauliHamil(PauliHamil h) { free(h.pauliCodes); free(h.termCoeffs); }
void initPauliHamil(PauliHamil h, qreal* coeffs, enum pauliOpType* codes) {
    for (int t = 0; t < h.numSumTerms; t++) {
        h.termCoeffs[t] = coeffs[t];
        for (int q = 0; q < h.numQubits; q++) h.pauliCodes[t * h.numQubits + q] = codes[t * h.numQubits + q];
    }
}

/* ------------------------------------------------------------------------ */
/* initialisation (QuEST_cpu.c:1133-1680)                                    */
/* ------------------------------------------------------------------------ */
void initBlankState(Qureg q) {
    memset(q.stateVec.real, 0, sizeof(qreal) * q.numAmpsTotal);
    memset(q.stateVec.imag, 0, sizeof(qreal) * q.numAmpsTotal);
}
void initZeroState(Qureg q) { initBlankState(q); q.stateVec.real[0] = 1.0; }     /* QuEST_cpu.c:1485 */
void initPlusState(Qureg q) {                                                    /* QuEST_cpu.c:1495, 1172 */
    idx_t n = q.numAmpsTotal;
    qreal v = q.isDensityMatrix ? 1.0 / (qreal)(1LL << q.numQubitsRepresented) : 1.0 / sqrt((qreal)n);
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; i++) { q.stateVec.real[i] = v; q.stateVec.imag[i] = 0; }
}
void initClassicalState(Qureg q, idx_t ind) {                                   /* QuEST_cpu.c:1527, 1133 */
    idx_t dim = 1LL << q.numQubitsRepresented;
    CHECK(ind >= 0 && ind < dim, "Invalid state index. Must be >=0 and <2^numQubits.");
    initBlankState(q);
    q.stateVec.real[q.isDensityMatrix ? ind * (dim + 1) : ind] = 1.0;
}
void initPureState(Qureg q, Qureg pure) {                                        /* QuEST_cpu.c:1202, 1563 */
    if (!q.isDensityMatrix) {
        memcpy(q.stateVec.real, pure.stateVec.real, sizeof(qreal) * q.numAmpsTotal);
        memcpy(q.stateVec.imag, pure.stateVec.imag, sizeof(qreal) * q.numAmpsTotal);
        return;
    }
    idx_t d = pure.numAmpsTotal;
#pragma omp parallel for schedule(static)
    for (idx_t c = 0; c < d; c++)
        for (idx_t r = 0; r < d; r++) {
            qreal ar = pure.stateVec.real[r], ai = pure.stateVec.imag[r];
            qreal br = pure.stateVec.real[c], bi = -pure.stateVec.imag[c];
            q.stateVec.real[r + c * d] = ar * br - ai * bi;
            q.stateVec.imag[r + c * d] = ar * bi + ai * br;
        }
}
void initDebugState(Qureg q) {                                                   /* QuEST_cpu.c:1648 */
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        q.stateVec.real[i] = (i * 2.0) / 10.0;
        q.stateVec.imag[i] = (i * 2.0 + 1.0) / 10.0;
    }
}
void setAmps(Qureg q, idx_t start, qreal* re, qreal* im, idx_t n) {              /* QuEST_cpu.c:1255 */
    memcpy(q.stateVec.real + start, re, sizeof(qreal) * n);
    memcpy(q.stateVec.imag + start, im, sizeof(qreal) * n);
}
void initStateFromAmps(Qureg q, qreal* re, qreal* im) { setAmps(q, 0, re, im, q.numAmpsTotal); }
void setDensityAmps(Qureg q, idx_t row, idx_t col, qreal* re, qreal* im, idx_t n) {
    setAmps(q, row + col * (1LL << q.numQubitsRepresented), re, im, n);
}
void cloneQureg(Qureg t, Qureg s) { setAmps(t, 0, s.stateVec.real, s.stateVec.imag, t.numAmpsTotal); }
void setWeightedQureg(Complex f1, Qureg q1, Complex f2, Qureg q2, Complex fo, Qureg out) {   /* QuEST_cpu.c:3988 */
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < out.numAmpsTotal; i++) {
        qreal r1 = q1.stateVec.real[i], i1 = q1.stateVec.imag[i];
        qreal r2 = q2.stateVec.real[i], i2 = q2.stateVec.imag[i];
        qreal ro = out.stateVec.real[i], io = out.stateVec.imag[i];
        out.stateVec.real[i] = f1.real * r1 - f1.imag * i1 + f2.real * r2 - f2.imag * i2 + fo.real * ro - fo.imag * io;
        out.stateVec.imag[i] = f1.real * i1 + f1.imag * r1 + f2.real * i2 + f2.imag * r2 + fo.real * io + fo.imag * ro;
    }
}
Complex getAmp(Qureg q, idx_t i) { Complex c = {q.stateVec.real[i], q.stateVec.imag[i]}; return c; }
qreal getRealAmp(Qureg q, idx_t i) { return q.stateVec.real[i]; }
qreal getImagAmp(Qureg q, idx_t i) { return q.stateVec.imag[i]; }
qreal getProbAmp(Qureg q, idx_t i) { qreal r = q.stateVec.real[i], m = q.stateVec.imag[i]; return r * r + m * m; }
Complex getDensityAmp(Qureg q, idx_t r, idx_t c) { return getAmp(q, r + c * (1LL << q.numQubitsRepresented)); }

/* ------------------------------------------------------------------------ */
/* state-vector kernels                                                       */
/* ------------------------------------------------------------------------ */

/* pair update with a dense 2x2 over all pairs whose control bits match
 * ((i ^ flip) & ctrl) == ctrl; QuEST_cpu.c:2009 (unitary), 2251 (multi-controlled) */
static void sv_matrix2(Qureg q, int t, idx_t ctrl, idx_t flip, ComplexMatrix2 u) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t np = q.numAmpsTotal >> 1, tb = 1LL << t;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < np; k++) {
        idx_t i0 = ins0(k, t), i1 = i0 | tb;
        if (((i0 ^ flip) & ctrl) != ctrl) continue;
        qreal ur = re[i0], ui = im[i0], lr = re[i1], li = im[i1];
        re[i0] = u.real[0][0] * ur - u.imag[0][0] * ui + u.real[0][1] * lr - u.imag[0][1] * li;
        im[i0] = u.real[0][0] * ui + u.imag[0][0] * ur + u.real[0][1] * li + u.imag[0][1] * lr;
        re[i1] = u.real[1][0] * ur - u.imag[1][0] * ui + u.real[1][1] * lr - u.imag[1][1] * li;
        im[i1] = u.real[1][0] * ui + u.imag[1][0] * ur + u.real[1][1] * li + u.imag[1][1] * lr;
    }
}

/* [alpha, -conj(beta); beta, conj(alpha)] -- QuEST_cpu.c:1737-1795, 2179 */
static void sv_compact(Qureg q, int t, idx_t ctrl, Complex a, Complex b) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t np = q.numAmpsTotal >> 1, tb = 1LL << t;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < np; k++) {
        idx_t i0 = ins0(k, t), i1 = i0 | tb;
        if ((i0 & ctrl) != ctrl) continue;
        qreal ur = re[i0], ui = im[i0], lr = re[i1], li = im[i1];
        re[i0] = a.real * ur - a.imag * ui - b.real * lr - b.imag * li;
        im[i0] = a.real * ui + a.imag * ur - b.real * li + b.imag * lr;
        re[i1] = b.real * ur - b.imag * ui + a.real * lr + a.imag * li;
        im[i1] = b.real * ui + b.imag * ur + a.real * li - a.imag * lr;
    }
}

/* amp <-> amp ^ targ for amps whose control bits are set (QuEST_cpu.c:2576, 2662, 2761) */
static void sv_not(Qureg q, idx_t ctrl, idx_t targ) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t n = q.numAmpsTotal;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; i++) {
        idx_t j = i ^ targ;
        if ((i & ctrl) != ctrl || j < i) continue;
        qreal r = re[i], m = im[i];
        re[i] = re[j]; im[i] = im[j]; re[j] = r; im[j] = m;
    }
}

/* Y = [0,-i; i,0] (conjFac -1 gives conj(Y)); QuEST_cpu.c:2870-2926, 2965 */
static void sv_pauliY(Qureg q, int t, idx_t ctrl, int conjFac) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t np = q.numAmpsTotal >> 1, tb = 1LL << t;
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < np; k++) {
        idx_t i0 = ins0(k, t), i1 = i0 | tb;
        if ((i0 & ctrl) != ctrl) continue;
        qreal ur = re[i0], ui = im[i0];
        re[i0] = conjFac * im[i1];
        im[i0] = conjFac * -re[i1];
        re[i1] = conjFac * -ui;
        im[i1] = conjFac * ur;
    }
}

/* H; QuEST_cpu.c:3061-3120 */
static void sv_hadamard(Qureg q, int t) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t np = q.numAmpsTotal >> 1, tb = 1LL << t;
    qreal f = 1.0 / sqrt(2.0);
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < np; k++) {
        idx_t i0 = ins0(k, t), i1 = i0 | tb;
        qreal ur = re[i0], ui = im[i0], lr = re[i1], li = im[i1];
        re[i0] = f * (ur + lr); im[i0] = f * (ui + li);
        re[i1] = f * (ur - lr); im[i1] = f * (ui - li);
    }
}

/* amp *= term where all bits of mask are 1; QuEST_cpu.c:3168 (phaseShiftByTerm),
 * 3209 (controlledPhaseShift), 3249 (multiControlledPhaseShift), 3670/3701 (phase flips) */
static void sv_phaseMask(Qureg q, idx_t mask, Complex term) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t n = q.numAmpsTotal;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; i++) {
        if ((i & mask) != mask) continue;
        qreal r = re[i], m = im[i];
        re[i] = term.real * r - term.imag * m;
        im[i] = term.imag * r + term.real * m;
    }
}

/* amp *= exp(-i angle/2 * (+1 even parity, -1 odd)) over amps with ctrl bits set;
 * QuEST_cpu.c:3299-3380 */
static void sv_multiRotateZ(Qureg q, idx_t ctrl, idx_t mask, qreal angle) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t n = q.numAmpsTotal;
    qreal c = cos(angle / 2), s = sin(angle / 2);
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; i++) {
        if ((i & ctrl) != ctrl) continue;
        qreal fs = parity(i & mask) ? 1.0 : -1.0;     /* odd parity: exp(+i a/2) */
        qreal r = re[i], m = im[i];
        re[i] = c * r - fs * s * m;
        im[i] = fs * s * r + c * m;
    }
}

/* swap amps |..1..0..> <-> |..0..1..>; QuEST_cpu.c:3905 */
static void sv_swap(Qureg q, int a, int b) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    idx_t n = q.numAmpsTotal, ma = 1LL << a, mb = 1LL << b;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; i++) {
        if ((i & ma) && !(i & mb)) {
            idx_t j = (i ^ ma) | mb;
            qreal r = re[i], m = im[i];
            re[i] = re[j]; im[i] = im[j]; re[j] = r; im[j] = m;
        }
    }
}

/* dense 2^k x 2^k on targets (targs[0] is the least significant matrix bit)
 * for amps with ctrl bits set; QuEST_cpu.c:1796 (two-qubit), 1895 (N-qubit) */
static void sv_matrixN(Qureg q, idx_t ctrl, const int* targs, int k, qreal** ur, qreal** ui) {
    qreal* re = q.stateVec.real; qreal* im = q.stateVec.imag;
    int d = 1 << k;
    idx_t tmask = maskOf(targs, k);
    idx_t n = q.numAmpsTotal;
#pragma omp parallel
    {
        idx_t* ind = (idx_t*)malloc(sizeof(idx_t) * d);
        qreal* vr = (qreal*)malloc(sizeof(qreal) * d);
        qreal* vi = (qreal*)malloc(sizeof(qreal) * d);
#pragma omp for schedule(static)
        for (idx_t base = 0; base < n; base++) {
            if ((base & tmask) != 0 || (base & ctrl) != ctrl) continue;
            for (int j = 0; j < d; j++) {
                idx_t a = base;
                for (int b = 0; b < k; b++) if ((j >> b) & 1) a |= 1LL << targs[b];
                ind[j] = a; vr[j] = re[a]; vi[j] = im[a];
            }
            for (int r = 0; r < d; r++) {
                qreal sr = 0, si = 0;
                for (int c = 0; c < d; c++) {
                    sr += ur[r][c] * vr[c] - ui[r][c] * vi[c];
                    si += ur[r][c] * vi[c] + ui[r][c] * vr[c];
                }
                re[ind[r]] = sr; im[ind[r]] = si;
            }
        }
        free(ind); free(vr); free(vi);
    }
}

/* ------------------------------------------------------------------------ */
/* validation helpers (subset of QuEST_validation.c)                         */
/* ------------------------------------------------------------------------ */
static int validTarget(Qureg q, int t) { return t >= 0 && t < q.numQubitsRepresented; }
static int uniq(const int* a, int n) { idx_t m = 0; for (int i = 0; i < n; i++) { if (m & (1LL << a[i])) return 0; m |= 1LL << a[i]; } return 1; }

static ComplexMatrix2 conj2(ComplexMatrix2 u) { for (int i = 0; i < 2; i++) for (int j = 0; j < 2; j++) u.imag[i][j] = -u.imag[i][j]; return u; }
static Complex conjC(Complex c) { c.imag = -c.imag; return c; }

/* ------------------------------------------------------------------------ */
/* public gates (QuEST.c:178-760): DM registers get U on t, conj(U) on t+N   */
/* ------------------------------------------------------------------------ */
void compactUnitary(Qureg q, int t, Complex a, Complex b) {                      /* QuEST.c:410 */
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(fabs(-1 + a.real * a.real + a.imag * a.imag + b.real * b.real + b.imag * b.imag) < REAL_EPS,
          "Compact matrix formed by given complex numbers is not unitary.");
    sv_compact(q, t, 0, a, b);
    if (q.isDensityMatrix) sv_compact(q, t + q.numQubitsRepresented, 0, conjC(a), conjC(b));
}
void controlledCompactUnitary(Qureg q, int c, int t, Complex a, Complex b) {      /* QuEST.c:424 */
    sv_compact(q, t, 1LL << c, a, b);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_compact(q, t + s, 1LL << (c + s), conjC(a), conjC(b)); }
}
static void rotPair(qreal ang, Vector ax, Complex* a, Complex* b) {              /* QuEST_common.c:117-124 */
    qreal mag = sqrt(ax.x * ax.x + ax.y * ax.y + ax.z * ax.z);
    qreal x = ax.x / mag, y = ax.y / mag, z = ax.z / mag;
    a->real = cos(ang / 2.0); a->imag = -sin(ang / 2.0) * z;
    b->real = sin(ang / 2.0) * y; b->imag = -sin(ang / 2.0) * x;
}
void rotateAroundAxis(Qureg q, int t, qreal ang, Vector ax) {                     /* QuEST.c:647, QuEST_common.c:318 */
    Complex a, b; rotPair(ang, ax, &a, &b);
    sv_compact(q, t, 0, a, b);
    if (q.isDensityMatrix) sv_compact(q, t + q.numQubitsRepresented, 0, conjC(a), conjC(b));
}
void rotateX(Qureg q, int t, qreal ang) { Vector v = {1, 0, 0}; rotateAroundAxis(q, t, ang, v); }
void rotateY(Qureg q, int t, qreal ang) { Vector v = {0, 1, 0}; rotateAroundAxis(q, t, ang, v); }
void rotateZ(Qureg q, int t, qreal ang) { Vector v = {0, 0, 1}; rotateAroundAxis(q, t, ang, v); }
void controlledRotateAroundAxis(Qureg q, int c, int t, qreal ang, Vector ax) {
    Complex a, b; rotPair(ang, ax, &a, &b);
    controlledCompactUnitary(q, c, t, a, b);
}
void controlledRotateX(Qureg q, int c, int t, qreal ang) { Vector v = {1, 0, 0}; controlledRotateAroundAxis(q, c, t, ang, v); }
void controlledRotateY(Qureg q, int c, int t, qreal ang) { Vector v = {0, 1, 0}; controlledRotateAroundAxis(q, c, t, ang, v); }
void controlledRotateZ(Qureg q, int c, int t, qreal ang) { Vector v = {0, 0, 1}; controlledRotateAroundAxis(q, c, t, ang, v); }

void unitary(Qureg q, int t, ComplexMatrix2 u) {                                  /* QuEST.c:354 */
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    sv_matrix2(q, t, 0, 0, u);
    if (q.isDensityMatrix) sv_matrix2(q, t + q.numQubitsRepresented, 0, 0, conj2(u));
}
void applyMatrix2(Qureg q, int t, ComplexMatrix2 u) { sv_matrix2(q, t, 0, 0, u); }
void controlledUnitary(Qureg q, int c, int t, ComplexMatrix2 u) {                 /* QuEST.c:366 */
    sv_matrix2(q, t, 1LL << c, 0, u);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_matrix2(q, t + s, 1LL << (c + s), 0, conj2(u)); }
}
void multiStateControlledUnitary(Qureg q, int* cs, int* st, int nc, int t, ComplexMatrix2 u) {   /* QuEST.c:394 */
    idx_t m = maskOf(cs, nc), f = 0;
    for (int i = 0; i < nc; i++) if (st[i] == 0) f |= 1LL << cs[i];
    sv_matrix2(q, t, m, f, u);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_matrix2(q, t + s, m << s, f << s, conj2(u)); }
}
void multiControlledUnitary(Qureg q, int* cs, int nc, int t, ComplexMatrix2 u) {  /* QuEST.c:379 */
    idx_t m = maskOf(cs, nc);
    sv_matrix2(q, t, m, 0, u);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_matrix2(q, t + s, m << s, 0, conj2(u)); }
}
void pauliX(Qureg q, int t) {
    sv_not(q, 0, 1LL << t);
    if (q.isDensityMatrix) sv_not(q, 0, 1LL << (t + q.numQubitsRepresented));
}
void pauliY(Qureg q, int t) {
    sv_pauliY(q, t, 0, 1);
    if (q.isDensityMatrix) sv_pauliY(q, t + q.numQubitsRepresented, 0, -1);
}
static void phaseTerm(Qureg q, idx_t mask, Complex term) {
    sv_phaseMask(q, mask, term);
    if (q.isDensityMatrix) sv_phaseMask(q, mask << q.numQubitsRepresented, conjC(term));
}
void pauliZ(Qureg q, int t) { Complex z = {-1, 0}; phaseTerm(q, 1LL << t, z); }
void sGate(Qureg q, int t) { Complex z = {0, 1}; phaseTerm(q, 1LL << t, z); }
void tGate(Qureg q, int t) { Complex z = {1 / sqrt(2), 1 / sqrt(2)}; phaseTerm(q, 1LL << t, z); }
void phaseShift(Qureg q, int t, qreal a) { Complex z = {cos(a), sin(a)}; phaseTerm(q, 1LL << t, z); }
void controlledPhaseShift(Qureg q, int a, int b, qreal ang) { Complex z = {cos(ang), sin(ang)}; phaseTerm(q, (1LL << a) | (1LL << b), z); }
void multiControlledPhaseShift(Qureg q, int* cs, int nc, qreal ang) { Complex z = {cos(ang), sin(ang)}; phaseTerm(q, maskOf(cs, nc), z); }
void controlledPhaseFlip(Qureg q, int a, int b) { Complex z = {-1, 0}; phaseTerm(q, (1LL << a) | (1LL << b), z); }
void multiControlledPhaseFlip(Qureg q, int* cs, int nc) { Complex z = {-1, 0}; phaseTerm(q, maskOf(cs, nc), z); }
void hadamard(Qureg q, int t) {
    sv_hadamard(q, t);
    if (q.isDensityMatrix) sv_hadamard(q, t + q.numQubitsRepresented);
}
void controlledNot(Qureg q, int c, int t) {                                        /* QuEST.c:530 */
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(c >= 0 && c < q.numQubitsRepresented, "Invalid control qubit. Must be >=0 and <numQubits.");
    CHECK(c != t, "Control qubit cannot equal target qubit.");
    sv_not(q, 1LL << c, 1LL << t);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_not(q, 1LL << (c + s), 1LL << (t + s)); }
}
void multiQubitNot(Qureg q, int* ts, int nt) {
    sv_not(q, 0, maskOf(ts, nt));
    if (q.isDensityMatrix) sv_not(q, 0, maskOf(ts, nt) << q.numQubitsRepresented);
}
void multiControlledMultiQubitNot(Qureg q, int* cs, int nc, int* ts, int nt) {
    sv_not(q, maskOf(cs, nc), maskOf(ts, nt));
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_not(q, maskOf(cs, nc) << s, maskOf(ts, nt) << s); }
}
void controlledPauliY(Qureg q, int c, int t) {
    sv_pauliY(q, t, 1LL << c, 1);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_pauliY(q, t + s, 1LL << (c + s), -1); }
}
void swapGate(Qureg q, int a, int b) {
    sv_swap(q, a, b);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_swap(q, a + s, b + s); }
}

static void applyN(Qureg q, idx_t ctrl, const int* ts, int k, qreal** ur, qreal** ui, int conjToo) {
    sv_matrixN(q, ctrl, ts, k, ur, ui);
    if (q.isDensityMatrix && conjToo) {
        int s = q.numQubitsRepresented, d = 1 << k;
        int sh[64];
        for (int i = 0; i < k; i++) sh[i] = ts[i] + s;
        qreal** ci = (qreal**)malloc(sizeof(qreal*) * d);
        for (int r = 0; r < d; r++) { ci[r] = (qreal*)malloc(sizeof(qreal) * d); for (int c = 0; c < d; c++) ci[r][c] = -ui[r][c]; }
        sv_matrixN(q, ctrl << s, sh, k, ur, ci);
        for (int r = 0; r < d; r++) free(ci[r]);
        free(ci);
    }
}
static void m4rows(ComplexMatrix4* u, qreal** ur, qreal** ui) { for (int i = 0; i < 4; i++) { ur[i] = u->real[i]; ui[i] = u->imag[i]; } }
void twoQubitUnitary(Qureg q, int t1, int t2, ComplexMatrix4 u) {
    qreal *ur[4], *ui[4]; m4rows(&u, ur, ui); int ts[2] = {t1, t2};
    applyN(q, 0, ts, 2, ur, ui, 1);
}
void controlledTwoQubitUnitary(Qureg q, int c, int t1, int t2, ComplexMatrix4 u) {
    qreal *ur[4], *ui[4]; m4rows(&u, ur, ui); int ts[2] = {t1, t2};
    applyN(q, 1LL << c, ts, 2, ur, ui, 1);
}
void multiControlledTwoQubitUnitary(Qureg q, int* cs, int nc, int t1, int t2, ComplexMatrix4 u) {
    qreal *ur[4], *ui[4]; m4rows(&u, ur, ui); int ts[2] = {t1, t2};
    applyN(q, maskOf(cs, nc), ts, 2, ur, ui, 1);
}
void applyMatrix4(Qureg q, int t1, int t2, ComplexMatrix4 u) {
    qreal *ur[4], *ui[4]; m4rows(&u, ur, ui); int ts[2] = {t1, t2};
    applyN(q, 0, ts, 2, ur, ui, 0);
}
void sqrtSwapGate(Qureg q, int a, int b) {                                         /* QuEST_common.c:386-412 */
    ComplexMatrix4 u; memset(&u, 0, sizeof u);
    u.real[0][0] = 1; u.real[3][3] = 1;
    u.real[1][1] = .5; u.imag[1][1] = .5; u.real[1][2] = .5; u.imag[1][2] = -.5;
    u.real[2][1] = .5; u.imag[2][1] = -.5; u.real[2][2] = .5; u.imag[2][2] = .5;
    twoQubitUnitary(q, a, b, u);
}
void multiQubitUnitary(Qureg q, int* ts, int k, ComplexMatrixN u) { applyN(q, 0, ts, k, u.real, u.imag, 1); }
void controlledMultiQubitUnitary(Qureg q, int c, int* ts, int k, ComplexMatrixN u) { applyN(q, 1LL << c, ts, k, u.real, u.imag, 1); }
void multiControlledMultiQubitUnitary(Qureg q, int* cs, int nc, int* ts, int k, ComplexMatrixN u) { applyN(q, maskOf(cs, nc), ts, k, u.real, u.imag, 1); }
void applyMatrixN(Qureg q, int* ts, int k, ComplexMatrixN u) { applyN(q, 0, ts, k, u.real, u.imag, 0); }

void multiRotateZ(Qureg q, int* qs, int n, qreal ang) {                            /* QuEST.c:658 */
    idx_t m = maskOf(qs, n);
    sv_multiRotateZ(q, 0, m, ang);
    if (q.isDensityMatrix) sv_multiRotateZ(q, 0, m << q.numQubitsRepresented, -ang);
}
void multiControlledMultiRotateZ(Qureg q, int* cs, int nc, int* ts, int nt, qreal ang) {
    idx_t c = maskOf(cs, nc), m = maskOf(ts, nt);
    sv_multiRotateZ(q, c, m, ang);
    if (q.isDensityMatrix) { int s = q.numQubitsRepresented; sv_multiRotateZ(q, c << s, m << s, -ang); }
}

/* basis change + multiRotateZ + undo, QuEST_common.c:411-448 */
static void sv_multiRotatePauli(Qureg q, idx_t ctrl, const int* ts, const enum pauliOpType* ps, int n, qreal ang, int conj) {
    qreal f = 1 / sqrt(2);
    ComplexMatrix2 rx, ry;
    qreal sg = conj ? 1 : -1;
    memset(&rx, 0, sizeof rx); memset(&ry, 0, sizeof ry);
    rx.real[0][0] = f; rx.real[1][1] = f; rx.imag[0][1] = sg * f; rx.imag[1][0] = sg * f;
    ry.real[0][0] = f; ry.real[0][1] = f; ry.real[1][0] = -f; ry.real[1][1] = f;
    Complex rxa = {f, 0}, rxb = {0, conj ? f : -f}, rya = {f, 0}, ryb = {-f, 0};
    idx_t mask = maskOf(ts, n);
    for (int i = 0; i < n; i++) {
        if (ps[i] == PAULI_I) mask &= ~(1LL << ts[i]);
        if (ctrl == 0) {
            if (ps[i] == PAULI_X) sv_compact(q, ts[i], 0, rya, ryb);
            if (ps[i] == PAULI_Y) sv_compact(q, ts[i], 0, rxa, rxb);
        } else {
            if (ps[i] == PAULI_X) sv_matrix2(q, ts[i], ctrl, 0, ry);
            if (ps[i] == PAULI_Y) sv_matrix2(q, ts[i], ctrl, 0, rx);
        }
    }
    if (mask) sv_multiRotateZ(q, ctrl, mask, conj ? -ang : ang);
    rxb.imag = -rxb.imag; ryb.real = -ryb.real;
    rx.imag[0][1] = -rx.imag[0][1]; rx.imag[1][0] = -rx.imag[1][0];
    ry.real[0][1] = -ry.real[0][1]; ry.real[1][0] = -ry.real[1][0];
    for (int i = 0; i < n; i++) {
        if (ctrl == 0) {
            if (ps[i] == PAULI_X) sv_compact(q, ts[i], 0, rya, ryb);
            if (ps[i] == PAULI_Y) sv_compact(q, ts[i], 0, rxa, rxb);
        } else {
            if (ps[i] == PAULI_X) sv_matrix2(q, ts[i], ctrl, 0, ry);
            if (ps[i] == PAULI_Y) sv_matrix2(q, ts[i], ctrl, 0, rx);
        }
    }
}
void multiRotatePauli(Qureg q, int* ts, enum pauliOpType* ps, int n, qreal ang) {  /* QuEST.c:691 */
    sv_multiRotatePauli(q, 0, ts, ps, n, ang, 0);
    if (q.isDensityMatrix) {
        int sh[64]; for (int i = 0; i < n; i++) sh[i] = ts[i] + q.numQubitsRepresented;
        sv_multiRotatePauli(q, 0, sh, ps, n, ang, 1);
    }
}
void multiControlledMultiRotatePauli(Qureg q, int* cs, int nc, int* ts, enum pauliOpType* ps, int n, qreal ang) {
    idx_t c = maskOf(cs, nc);
    sv_multiRotatePauli(q, c, ts, ps, n, ang, 0);
    if (q.isDensityMatrix) {
        int s = q.numQubitsRepresented, sh[64]; for (int i = 0; i < n; i++) sh[i] = ts[i] + s;
        sv_multiRotatePauli(q, c << s, sh, ps, n, ang, 1);
    }
}

/* Trotter: QuEST_common.c:762-844 */
static void expPauliHamil(Qureg q, PauliHamil h, qreal fac, int rev) {
    int vt[64], dt[64];
    for (int i = 0; i < h.numQubits; i++) { vt[i] = i; dt[i] = i + h.numQubits; }
    for (int i = 0; i < h.numSumTerms; i++) {
        int t = rev ? h.numSumTerms - 1 - i : i;
        qreal ang = 2 * fac * h.termCoeffs[t];
        sv_multiRotatePauli(q, 0, vt, h.pauliCodes + (idx_t)t * h.numQubits, h.numQubits, ang, 0);
        if (q.isDensityMatrix) sv_multiRotatePauli(q, 0, dt, h.pauliCodes + (idx_t)t * h.numQubits, h.numQubits, ang, 1);
    }
}
static void symTrotter(Qureg q, PauliHamil h, qreal time, int order) {
    if (order == 1) { expPauliHamil(q, h, time, 0); return; }
    if (order == 2) { expPauliHamil(q, h, time / 2., 0); expPauliHamil(q, h, time / 2., 1); return; }
    qreal p = 1. / (4 - pow(4, 1. / (order - 1)));
    int lo = order - 2;
    symTrotter(q, h, p * time, lo); symTrotter(q, h, p * time, lo);
    symTrotter(q, h, (1 - 4 * p) * time, lo);
    symTrotter(q, h, p * time, lo); symTrotter(q, h, p * time, lo);
}
void applyTrotterCircuit(Qureg q, PauliHamil h, qreal time, int order, int reps) {
    if (time == 0) return;
    for (int r = 0; r < reps; r++) symTrotter(q, h, time / reps, order);
}

/* ------------------------------------------------------------------------ */
/* reductions                                                                 */
/* ------------------------------------------------------------------------ */
qreal calcTotalProb(Qureg q) {                                                    /* QuEST_cpu_local.c:144 (Kahan) */
    qreal sum = 0, c = 0, y, t;
    if (q.isDensityMatrix) {
        idx_t d = 1LL << q.numQubitsRepresented;
        for (idx_t i = 0; i < d; i++) { y = q.stateVec.real[i * (d + 1)] - c; t = sum + y; c = (t - sum) - y; sum = t; }
        return sum;
    }
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        y = q.stateVec.real[i] * q.stateVec.real[i] - c; t = sum + y; c = (t - sum) - y; sum = t;
        y = q.stateVec.imag[i] * q.stateVec.imag[i] - c; t = sum + y; c = (t - sum) - y; sum = t;
    }
    return sum;
}
static qreal probZero(Qureg q, int t) {                                          /* QuEST_cpu.c:3385, 3440 */
    qreal s = 0;
    if (q.isDensityMatrix) {
        idx_t d = 1LL << q.numQubitsRepresented;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (idx_t r = 0; r < d; r++) if (!((r >> t) & 1)) s += q.stateVec.real[r * (d + 1)];
        return s;
    }
    idx_t np = q.numAmpsTotal >> 1;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t k = 0; k < np; k++) {
        idx_t i = ins0(k, t);
        s += q.stateVec.real[i] * q.stateVec.real[i] + q.stateVec.imag[i] * q.stateVec.imag[i];
    }
    return s;
}
qreal calcProbOfOutcome(Qureg q, int t, int outcome) {                           /* QuEST.c:1175; QuEST_gpu.cu:2155-2161 */
    CHECKR(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.", 0);
    CHECKR(outcome == 0 || outcome == 1, "Invalid measurement outcome -- must be either 0 or 1.", 0);
    qreal p0 = probZero(q, t);
    return outcome == 0 ? p0 : 1 - p0;
}
void calcProbOfAllOutcomes(qreal* out, Qureg q, int* qs, int nq) {                /* QuEST_cpu.c:3532, 3599 */
    idx_t no = 1LL << nq;
    for (idx_t j = 0; j < no; j++) out[j] = 0;
    if (q.isDensityMatrix) {
        idx_t d = 1LL << q.numQubitsRepresented;
        for (idx_t r = 0; r < d; r++) {
            idx_t o = 0; for (int b = 0; b < nq; b++) o |= ((r >> qs[b]) & 1) << b;
            out[o] += q.stateVec.real[r * (d + 1)];
        }
        return;
    }
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t o = 0; for (int b = 0; b < nq; b++) o |= ((i >> qs[b]) & 1) << b;
        out[o] += q.stateVec.real[i] * q.stateVec.real[i] + q.stateVec.imag[i] * q.stateVec.imag[i];
    }
}
Complex calcInnerProduct(Qureg bra, Qureg ket) {                                  /* QuEST_cpu.c:1089 */
    qreal sr = 0, si = 0;
#pragma omp parallel for reduction(+ : sr, si) schedule(static)
    for (idx_t i = 0; i < bra.numAmpsTotal; i++) {
        qreal br = bra.stateVec.real[i], bi = bra.stateVec.imag[i], kr = ket.stateVec.real[i], ki = ket.stateVec.imag[i];
        sr += br * kr + bi * ki;
        si += br * ki - bi * kr;
    }
    Complex c = {sr, si};
    return c;
}
qreal calcDensityInnerProduct(Qureg a, Qureg b) {                                 /* QuEST_cpu.c:976 */
    qreal s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t i = 0; i < a.numAmpsTotal; i++) s += a.stateVec.real[i] * b.stateVec.real[i] + a.stateVec.imag[i] * b.stateVec.imag[i];
    return s;
}
qreal calcPurity(Qureg q) {                                                       /* QuEST_cpu.c:879 */
    qreal s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) s += q.stateVec.real[i] * q.stateVec.real[i] + q.stateVec.imag[i] * q.stateVec.imag[i];
    return s;
}
qreal calcHilbertSchmidtDistance(Qureg a, Qureg b) {                              /* QuEST_cpu.c:941 */
    qreal s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t i = 0; i < a.numAmpsTotal; i++) {
        qreal dr = a.stateVec.real[i] - b.stateVec.real[i], di = a.stateVec.imag[i] - b.stateVec.imag[i];
        s += dr * dr + di * di;
    }
    return sqrt(s);
}
qreal calcFidelity(Qureg q, Qureg pure) {                                         /* QuEST_common.c:377, QuEST_cpu.c:1008 */
    if (!q.isDensityMatrix) { Complex c = calcInnerProduct(q, pure); return c.real * c.real + c.imag * c.imag; }
    idx_t d = pure.numAmpsTotal;
    qreal s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t r = 0; r < d; r++) {
        qreal rr = 0, ri = 0;
        for (idx_t c = 0; c < d; c++) {
            qreal er = q.stateVec.real[r + d * c], ei = q.stateVec.imag[r + d * c];
            qreal vr = pure.stateVec.real[c], vi = pure.stateVec.imag[c];
            rr += er * vr - ei * vi;
            ri += er * vi + ei * vr;
        }
        s += rr * pure.stateVec.real[r] - ri * (-pure.stateVec.imag[r]);
    }
    return s;
}

/* clone + Pauli product + inner product (SV) or trace (DM); QuEST_common.c:493-533 */
qreal calcExpecPauliProd(Qureg q, int* ts, enum pauliOpType* ps, int n, Qureg ws) {
    cloneQureg(ws, q);
    for (int i = 0; i < n; i++) {
        if (ps[i] == PAULI_X) sv_not(ws, 0, 1LL << ts[i]);
        if (ps[i] == PAULI_Y) sv_pauliY(ws, ts[i], 0, 1);
        if (ps[i] == PAULI_Z) { Complex z = {-1, 0}; sv_phaseMask(ws, 1LL << ts[i], z); }
    }
    if (q.isDensityMatrix) return calcTotalProb(ws);
    return calcInnerProduct(ws, q).real;
}
qreal calcExpecPauliSum(Qureg q, enum pauliOpType* codes, qreal* coeffs, int nt, Qureg ws) {
    int nq = q.numQubitsRepresented, ts[64];
    for (int i = 0; i < nq; i++) ts[i] = i;
    qreal v = 0;
    for (int t = 0; t < nt; t++) v += coeffs[t] * calcExpecPauliProd(q, ts, codes + (idx_t)t * nq, nq, ws);
    return v;
}
qreal calcExpecPauliHamil(Qureg q, PauliHamil h, Qureg ws) { return calcExpecPauliSum(q, h.pauliCodes, h.termCoeffs, h.numSumTerms, ws); }

/* ------------------------------------------------------------------------ */
/* measurement (QuEST.c:972-1016, QuEST_common.c:165-180, QuEST_cpu.c:3750) */
/* ------------------------------------------------------------------------ */
static void collapse(Qureg q, int t, int outcome, qreal prob) {
    if (!q.isDensityMatrix) {
        qreal rn = 1 / sqrt(prob);
        idx_t tb = 1LL << t;
#pragma omp parallel for schedule(static)
        for (idx_t i = 0; i < q.numAmpsTotal; i++) {
            if ((int)((i & tb) != 0) == outcome) { q.stateVec.real[i] *= rn; q.stateVec.imag[i] *= rn; }
            else { q.stateVec.real[i] = 0; q.stateVec.imag[i] = 0; }
        }
        return;
    }
    /* DM: keep entries whose row and column bit both equal outcome, scaled by 1/prob (QuEST_cpu.c:757-878) */
    int s = q.numQubitsRepresented;
    idx_t rb = 1LL << t, cb = 1LL << (t + s);
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        int r = (i & rb) != 0, c = (i & cb) != 0;
        if (r == outcome && c == outcome) { q.stateVec.real[i] /= prob; q.stateVec.imag[i] /= prob; }
        else { q.stateVec.real[i] = 0; q.stateVec.imag[i] = 0; }
    }
}
qreal collapseToOutcome(Qureg q, int t, int outcome) {
    CHECKR(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.", 0);
    CHECKR(outcome == 0 || outcome == 1, "Invalid measurement outcome -- must be either 0 or 1.", 0);
    qreal p = calcProbOfOutcome(q, t, outcome);
    CHECKR(p >= REAL_EPS, "Can't collapse to state with zero probability.", 0);
    collapse(q, t, outcome, p);
    return p;
}
int measureWithStats(Qureg q, int t, qreal* outcomeProb) {
    qreal p0 = probZero(q, t);
    int outcome;
    if (p0 < REAL_EPS) outcome = 1;
    else if (1 - p0 < REAL_EPS) outcome = 0;
    else outcome = (mt_real1() > p0);
    *outcomeProb = outcome == 0 ? p0 : 1 - p0;
    collapse(q, t, outcome, *outcomeProb);
    return outcome;
}
int measure(Qureg q, int t) { qreal p; return measureWithStats(q, t, &p); }

/* ------------------------------------------------------------------------ */
/* decoherence (QuEST_cpu.c:61-235)                                          */
/* ------------------------------------------------------------------------ */
static void dephase(Qureg q, int t, qreal retain) {
    int s = q.numQubitsRepresented;
    idx_t inner = 1LL << t, outer = 1LL << (t + s), tot = inner | outer;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t p = i & tot;
        if (p == inner || p == outer) { q.stateVec.real[i] *= retain; q.stateVec.imag[i] *= retain; }
    }
}
void mixDephasing(Qureg q, int t, qreal prob) {                                   /* QuEST.c:1259 -> dephase 2p */
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(prob >= 0 && prob <= 1, "Probabilities must be in [0, 1].");
    CHECK(prob <= 1 / 2.0, "The probability of a single qubit dephase error cannot exceed 1/2, which maximally mixes.");
    dephase(q, t, 1 - 2 * prob);
}
void mixDepolarising(Qureg q, int t, qreal prob) {                                /* QuEST.c:1281 -> level 4p/3 */
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(prob >= 0 && prob <= 1, "Probabilities must be in [0, 1].");
    CHECK(prob <= 3 / 4.0, "The probability of a single qubit depolarising error cannot exceed 3/4, which maximally mixes.");
    qreal lvl = (4 * prob) / 3.0, retain = 1 - lvl;
    int s = q.numQubitsRepresented;
    idx_t inner = 1LL << t, outer = 1LL << (t + s), tot = inner | outer;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t p = i & tot;
        if (p == inner || p == outer) { q.stateVec.real[i] *= retain; q.stateVec.imag[i] *= retain; }
        else if (p == 0) {
            idx_t j = i | tot;
            qreal ar = (q.stateVec.real[i] + q.stateVec.real[j]) / 2, ai = (q.stateVec.imag[i] + q.stateVec.imag[j]) / 2;
            q.stateVec.real[i] = retain * q.stateVec.real[i] + lvl * ar;
            q.stateVec.imag[i] = retain * q.stateVec.imag[i] + lvl * ai;
            q.stateVec.real[j] = retain * q.stateVec.real[j] + lvl * ar;
            q.stateVec.imag[j] = retain * q.stateVec.imag[j] + lvl * ai;
        }
    }
}
void mixDamping(Qureg q, int t, qreal prob) {                                     /* QuEST.c:1292, QuEST_cpu.c:187 */
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(prob >= 0 && prob <= 1, "Probabilities must be in [0, 1].");
    qreal retain = 1 - prob, deph = sqrt(retain);
    int s = q.numQubitsRepresented;
    idx_t inner = 1LL << t, outer = 1LL << (t + s), tot = inner | outer;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t p = i & tot;
        if (p == inner || p == outer) { q.stateVec.real[i] *= deph; q.stateVec.imag[i] *= deph; }
        else if (p == 0) {
            idx_t j = i | tot;
            q.stateVec.real[i] = q.stateVec.real[i] + prob * q.stateVec.real[j];
            q.stateVec.imag[i] = q.stateVec.imag[i] + prob * q.stateVec.imag[j];
            q.stateVec.real[j] = retain * q.stateVec.real[j];
            q.stateVec.imag[j] = retain * q.stateVec.imag[j];
        }
    }
}
/* mixPauli: the Kraus map {sqrt(1-pX-pY-pZ) I, sqrt(pX) X, sqrt(pY) Y,
 * sqrt(pZ) Z} (QuEST_common.c:740-759), applied as its superoperator
 * S = sum_k conj(K_k) (x) K_k on (row qubit t, column qubit t + N)
 * (QuEST_common.c:590-640 populateKrausSuperOperator2 + the 2-qubit matrix
 * pass): local index r + 2c, out = S in. */
void mixPauli(Qureg q, int t, qreal pX, qreal pY, qreal pZ) {                    /* QuEST.c:1312 */
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, t), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(pX >= 0 && pX <= 1 && pY >= 0 && pY <= 1 && pZ >= 0 && pZ <= 1, "Probabilities must be in [0, 1].");
    qreal none = 1 - pX - pY - pZ;
    CHECK(pX <= none && pY <= none && pZ <= none,
          "The probability of any X, Y or Z error cannot exceed the probability of no error.");
    qreal f[4] = {sqrt(none), sqrt(pX), sqrt(pY), sqrt(pZ)};
    /* K[k][r][c] as complex (re, im) */
    qreal Kr[4][2][2] = {{{f[0], 0}, {0, f[0]}}, {{0, f[1]}, {f[1], 0}}, {{0, 0}, {0, 0}}, {{f[3], 0}, {0, -f[3]}}};
    qreal Ki[4][2][2] = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, {{0, -f[2]}, {f[2], 0}}, {{0, 0}, {0, 0}}};
    qreal Sr[4][4] = {{0}}, Si[4][4] = {{0}};
    for (int k = 0; k < 4; k++)
        for (int r = 0; r < 2; r++) for (int c = 0; c < 2; c++)
            for (int r2 = 0; r2 < 2; r2++) for (int c2 = 0; c2 < 2; c2++) {
                /* K[r][r2] * conj(K[c][c2]) */
                qreal ar = Kr[k][r][r2], ai = Ki[k][r][r2], br = Kr[k][c][c2], bi = -Ki[k][c][c2];
                Sr[r + 2 * c][r2 + 2 * c2] += ar * br - ai * bi;
                Si[r + 2 * c][r2 + 2 * c2] += ar * bi + ai * br;
            }
    int s = q.numQubitsRepresented;
    idx_t rb = 1LL << t, cb = 1LL << (t + s);
#pragma omp parallel for schedule(static)
    for (idx_t g = 0; g < q.numAmpsTotal / 4; g++) {
        idx_t b = ins0(ins0(g, t), t + s);
        idx_t ix[4] = {b, b | rb, b | cb, b | rb | cb};
        qreal xr[4], xi[4];
        for (int j = 0; j < 4; j++) { xr[j] = q.stateVec.real[ix[j]]; xi[j] = q.stateVec.imag[ix[j]]; }
        for (int r = 0; r < 4; r++) {
            qreal yr = 0, yi = 0;
            for (int j = 0; j < 4; j++) { yr += Sr[r][j] * xr[j] - Si[r][j] * xi[j]; yi += Sr[r][j] * xi[j] + Si[r][j] * xr[j]; }
            q.stateVec.real[ix[r]] = yr; q.stateVec.imag[ix[r]] = yi;
        }
    }
}
/* Entries whose row and column bits differ on qubit q1 or on qubit q2 are
 * scaled by 1 - 4p/3 (QuEST.c:1269 -> QuEST_cpu.c:97-136). */
void mixTwoQubitDephasing(Qureg q, int q1, int q2, qreal prob) {
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, q1) && validTarget(q, q2), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(q1 != q2, "The target qubits must be unique.");
    CHECK(prob >= 0 && prob <= 1, "Probabilities must be in [0, 1].");
    CHECK(prob <= 3 / 4.0, "The probability of a two-qubit qubit dephase error cannot exceed 3/4, which maximally mixes.");
    qreal retain = 1 - (4 * prob) / 3.0;
    int s = q.numQubitsRepresented;
    idx_t m1 = (1LL << q1) | (1LL << (q1 + s)), m2 = (1LL << q2) | (1LL << (q2 + s));
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t a = i & m1, b = i & m2;
        if ((a != 0 && a != m1) || (b != 0 && b != m2)) { q.stateVec.real[i] *= retain; q.stateVec.imag[i] *= retain; }
    }
}
/* Level l = 16p/15: every entry is scaled by 1 - l, and each of the four
 * entries whose row and column bits agree on both qubits gains l/4 times the
 * sum of the four (QuEST.c:1300 -> QuEST_gpu.cu:3080-3147: the dephasing
 * launch, then the averaging launch). */
void mixTwoQubitDepolarising(Qureg q, int q1, int q2, qreal prob) {
    CHECK(q.isDensityMatrix, "Operation valid only for density matrices.");
    CHECK(validTarget(q, q1) && validTarget(q, q2), "Invalid target qubit. Must be >=0 and <numQubits.");
    CHECK(q1 != q2, "The target qubits must be unique.");
    CHECK(prob >= 0 && prob <= 1, "Probabilities must be in [0, 1].");
    CHECK(prob <= 15 / 16.0, "The probability of a two-qubit depolarising error cannot exceed 15/16, which maximally mixes.");
    qreal lvl = (16 * prob) / 15.0, retain = 1 - lvl;
    if (lvl == 0) return;
    int s = q.numQubitsRepresented;
    idx_t c1 = (1LL << q1) | (1LL << (q1 + s)), c2 = (1LL << q2) | (1LL << (q2 + s));
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < q.numAmpsTotal; i++) {
        idx_t a = i & c1, b = i & c2;
        if ((a != 0 && a != c1) || (b != 0 && b != c2)) { q.stateVec.real[i] *= retain; q.stateVec.imag[i] *= retain; }
        else if (a == 0 && b == 0) {
            idx_t j[4] = {i, i | c1, i | c2, i | c1 | c2};
            qreal sr = lvl * 0.25 * (q.stateVec.real[j[0]] + q.stateVec.real[j[1]] + q.stateVec.real[j[2]] + q.stateVec.real[j[3]]);
            qreal si = lvl * 0.25 * (q.stateVec.imag[j[0]] + q.stateVec.imag[j[1]] + q.stateVec.imag[j[2]] + q.stateVec.imag[j[3]]);
            for (int k = 0; k < 4; k++) {
                q.stateVec.real[j[k]] = q.stateVec.real[j[k]] * retain + sr;
                q.stateVec.imag[j[k]] = q.stateVec.imag[j[k]] * retain + si;
            }
        }
    }
}
void mixDensityMatrix(Qureg a, qreal p, Qureg b) {                                /* QuEST_cpu.c:908 */
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < a.numAmpsTotal; i++) {
        a.stateVec.real[i] *= 1 - p; a.stateVec.imag[i] *= 1 - p;
        a.stateVec.real[i] += p * b.stateVec.real[i]; a.stateVec.imag[i] += p * b.stateVec.imag[i];
    }
}

void startRecordingQASM(Qureg q) { (void)q; }
void stopRecordingQASM(Qureg q) { (void)q; }
void clearRecordedQASM(Qureg q) { (void)q; }
void printRecordedQASM(Qureg q) { (void)q; }
void writeRecordedQASMToFile(Qureg q, char* f) { (void)q; (void)f; }
void reportState(Qureg q) { (void)q; }
void reportStateToScreen(Qureg q, QuESTEnv env, int r) { (void)q; (void)env; (void)r; }
void reportQuregParams(Qureg q) { (void)q; }
void reportPauliHamil(PauliHamil h) { (void)h; }

/* The rest of the API: exported so that the oracle and the product export
 * the same symbols; each reports that it is unsupported. */
#define UNSUP() fail("This QuEST function is not supported by the GB300 library (unsupported).", __func__)
void mixKrausMap(Qureg q, int t, ComplexMatrix2* o, int n) { (void)q; (void)t; (void)o; (void)n; UNSUP(); }
void mixTwoQubitKrausMap(Qureg q, int a, int b, ComplexMatrix4* o, int n) { (void)q; (void)a; (void)b; (void)o; (void)n; UNSUP(); }
void mixMultiQubitKrausMap(Qureg q, int* t, int k, ComplexMatrixN* o, int n) { (void)q; (void)t; (void)k; (void)o; (void)n; UNSUP(); }
void mixNonTPKrausMap(Qureg q, int t, ComplexMatrix2* o, int n) { (void)q; (void)t; (void)o; (void)n; UNSUP(); }
void mixNonTPTwoQubitKrausMap(Qureg q, int a, int b, ComplexMatrix4* o, int n) { (void)q; (void)a; (void)b; (void)o; (void)n; UNSUP(); }
void mixNonTPMultiQubitKrausMap(Qureg q, int* t, int k, ComplexMatrixN* o, int n) { (void)q; (void)t; (void)k; (void)o; (void)n; UNSUP(); }
void applyPauliSum(Qureg a, enum pauliOpType* c, qreal* w, int n, Qureg b) { (void)a; (void)c; (void)w; (void)n; (void)b; UNSUP(); }
void applyPauliHamil(Qureg a, PauliHamil h, Qureg b) { (void)a; (void)h; (void)b; UNSUP(); }
void applyMultiControlledMatrixN(Qureg q, int* c, int nc, int* t, int nt, ComplexMatrixN u) { (void)q; (void)c; (void)nc; (void)t; (void)nt; (void)u; UNSUP(); }
void applyProjector(Qureg q, int t, int o) { (void)q; (void)t; (void)o; UNSUP(); }
void applyQFT(Qureg q, int* t, int n) { (void)q; (void)t; (void)n; UNSUP(); }
void applyFullQFT(Qureg q) { (void)q; UNSUP(); }
void applyPhaseFunc(Qureg q, int* t, int n, enum bitEncoding e, qreal* c, qreal* x, int m) { (void)q; (void)t; (void)n; (void)e; (void)c; (void)x; (void)m; UNSUP(); }
void applyPhaseFuncOverrides(Qureg q, int* t, int n, enum bitEncoding e, qreal* c, qreal* x, int m, long long* oi, qreal* op, int no) {
    (void)q; (void)t; (void)n; (void)e; (void)c; (void)x; (void)m; (void)oi; (void)op; (void)no; UNSUP();
}
void applyMultiVarPhaseFunc(Qureg q, int* t, int* r, int nr, enum bitEncoding e, qreal* c, qreal* x, int* m) {
    (void)q; (void)t; (void)r; (void)nr; (void)e; (void)c; (void)x; (void)m; UNSUP();
}
void applyMultiVarPhaseFuncOverrides(Qureg q, int* t, int* r, int nr, enum bitEncoding e, qreal* c, qreal* x, int* m, long long* oi, qreal* op, int no) {
    (void)q; (void)t; (void)r; (void)nr; (void)e; (void)c; (void)x; (void)m; (void)oi; (void)op; (void)no; UNSUP();
}
void applyNamedPhaseFunc(Qureg q, int* t, int* r, int nr, enum bitEncoding e, enum phaseFunc f) { (void)q; (void)t; (void)r; (void)nr; (void)e; (void)f; UNSUP(); }
void applyNamedPhaseFuncOverrides(Qureg q, int* t, int* r, int nr, enum bitEncoding e, enum phaseFunc f, long long* oi, qreal* op, int no) {
    (void)q; (void)t; (void)r; (void)nr; (void)e; (void)f; (void)oi; (void)op; (void)no; UNSUP();
}
void applyParamNamedPhaseFunc(Qureg q, int* t, int* r, int nr, enum bitEncoding e, enum phaseFunc f, qreal* p, int np) {
    (void)q; (void)t; (void)r; (void)nr; (void)e; (void)f; (void)p; (void)np; UNSUP();
}
void applyParamNamedPhaseFuncOverrides(Qureg q, int* t, int* r, int nr, enum bitEncoding e, enum phaseFunc f, qreal* p, int np, long long* oi, qreal* op, int no) {
    (void)q; (void)t; (void)r; (void)nr; (void)e; (void)f; (void)p; (void)np; (void)oi; (void)op; (void)no; UNSUP();
}
DiagonalOp createDiagonalOp(int n, QuESTEnv env) { DiagonalOp d; memset(&d, 0, sizeof d); (void)n; (void)env; UNSUP(); return d; }
DiagonalOp createDiagonalOpFromPauliHamilFile(char* f, QuESTEnv env) { DiagonalOp d; memset(&d, 0, sizeof d); (void)f; (void)env; UNSUP(); return d; }
void destroyDiagonalOp(DiagonalOp d, QuESTEnv env) { (void)d; (void)env; UNSUP(); }
void syncDiagonalOp(DiagonalOp d) { (void)d; UNSUP(); }
void initDiagonalOp(DiagonalOp d, qreal* r, qreal* i) { (void)d; (void)r; (void)i; UNSUP(); }
void initDiagonalOpFromPauliHamil(DiagonalOp d, PauliHamil h) { (void)d; (void)h; UNSUP(); }
void setDiagonalOpElems(DiagonalOp d, long long s, qreal* r, qreal* i, long long n) { (void)d; (void)s; (void)r; (void)i; (void)n; UNSUP(); }
void applyDiagonalOp(Qureg q, DiagonalOp d) { (void)q; (void)d; UNSUP(); }
Complex calcExpecDiagonalOp(Qureg q, DiagonalOp d) { Complex z = {0, 0}; (void)q; (void)d; UNSUP(); return z; }
PauliHamil createPauliHamilFromFile(char* f) { PauliHamil h; memset(&h, 0, sizeof h); (void)f; UNSUP(); return h; }
void initComplexMatrixN(ComplexMatrixN m, qreal real[][1 << m.numQubits], qreal imag[][1 << m.numQubits]) {
    int D = 1 << m.numQubits;
    for (int r = 0; r < D; r++) for (int c = 0; c < D; c++) { m.real[r][c] = real[r][c]; m.imag[r][c] = imag[r][c]; }
}
ComplexMatrixN bindArraysToStackComplexMatrixN(int n, qreal re[][1 << n], qreal im[][1 << n], qreal** rs, qreal** is) {
    ComplexMatrixN m;
    for (int r = 0; r < (1 << n); r++) { rs[r] = re[r]; is[r] = im[r]; }
    m.numQubits = n; m.real = rs; m.imag = is;
    return m;
}
