// sv_gates.cu -- plain FP64 gate kernels for sm_103a.
//
// One launch per API gate, each a single streaming pass over only the
// amplitudes the gate touches (control bits are enumerated, not tested), with
// 16-byte vector loads of the SoA real/imag arrays.  Semantics follow the
// reference backend Code/QuEST340/QuEST/src/GPU/QuEST_gpu.cu (line numbers
// per launcher below); the thread->amplitude mapping is new.
//
// Thread mapping.  A gate touches pairs (i0, i0 ^ pmask) whose "inserted"
// bits (the lowest partner bit plus all control bits) are fixed: i0 =
// insertZeros(k) | setMask for k in [0, 2^(n - numInserted)).  When no
// inserted bit is bit 0, consecutive k give consecutive i0, so one thread
// takes k = 2t, 2t+1 and moves them with double2 loads (kVec).  When the
// partner bit is bit 0 the pair itself is adjacent (kAdj).  Otherwise kScalar.
#include "df64.cuh"
#include "qg_internal.h"

#include <algorithm>
#include <vector>

namespace qg {

namespace {

constexpr int kThreads = 256;

struct InsSpec {
    int n;
    int pos[63];   // ascending bit positions of the zeros to insert
};

__device__ __forceinline__ uint64_t insertZeros(uint64_t k, const InsSpec& s) {
    for (int j = 0; j < s.n; ++j) {
        const int b = s.pos[j];
        const uint64_t lo = k & ((1ull << b) - 1ull);
        k = ((k >> b) << (b + 1)) | lo;
    }
    return k;
}

InsSpec makeIns(uint64_t mask) {
    InsSpec s{};
    s.n = 0;
    for (int b = 0; b < 64; ++b)
        if (mask >> b & 1ull) s.pos[s.n++] = b;
    return s;
}

inline unsigned blocksFor(uint64_t threads) { return (unsigned)((threads + kThreads - 1) / kThreads); }

__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ void st2(double* p, double2 v) { *reinterpret_cast<double2*>(p) = v; }

// ---------------------------------------------------------------- pair ops
struct OpMatrix2 {
    Mat2 m;
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        const double a = ur, b = ui, c = lr, d = li;
        ur = m.r[0][0] * a - m.i[0][0] * b + m.r[0][1] * c - m.i[0][1] * d;
        ui = m.r[0][0] * b + m.i[0][0] * a + m.r[0][1] * d + m.i[0][1] * c;
        lr = m.r[1][0] * a - m.i[1][0] * b + m.r[1][1] * c - m.i[1][1] * d;
        li = m.r[1][0] * b + m.i[1][0] * a + m.r[1][1] * d + m.i[1][1] * c;
    }
};

// QuEST_gpu.cu:783-844: up' = a.up - conj(b).lo ; lo' = b.up + conj(a).lo
struct OpCompact {
    double ar, ai, br, bi;
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        const double a = ur, b = ui, c = lr, d = li;
        ur = ar * a - ai * b - br * c - bi * d;
        ui = ar * b + ai * a - br * d + bi * c;
        lr = br * a - bi * b + ar * c + ai * d;
        li = br * b + bi * a + ar * d - ai * c;
    }
};

// The 2 x 2 update in double-float form (df64.cuh), for the plain path's
// double-float mode (quest_gb300_setPlainArithmetic(1)): each output is a
// compensated four-term dot product of DF coefficients and the DF parts of
// the inputs, on the FP32 and integer pipes.  coef[o] holds the four
// coefficients of output o (ur, ui, lr, li) against inputs (a, b, c, d) =
// (ur, ui, lr, li) for the real outputs and (b, a, d, c) for the imaginary
// ones, signs included.
struct OpMatrix2DF {
    df::F2 coef[4][4];
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        const df::F2 a = df::fromDouble(ur), b = df::fromDouble(ui), c = df::fromDouble(lr), d = df::fromDouble(li);
        const df::F2 re4[4] = {a, b, c, d}, im4[4] = {b, a, d, c};
        ur = df::toDouble(df::dot4(coef[0], re4));
        ui = df::toDouble(df::dot4(coef[1], im4));
        lr = df::toDouble(df::dot4(coef[2], re4));
        li = df::toDouble(df::dot4(coef[3], im4));
    }
};
OpMatrix2DF matrix2DF(const Mat2& m) {
    OpMatrix2DF op;
    const double k[4][4] = {{m.r[0][0], -m.i[0][0], m.r[0][1], -m.i[0][1]},
                            {m.r[0][0], m.i[0][0], m.r[0][1], m.i[0][1]},
                            {m.r[1][0], -m.i[1][0], m.r[1][1], -m.i[1][1]},
                            {m.r[1][0], m.i[1][0], m.r[1][1], m.i[1][1]}};
    for (int o = 0; o < 4; ++o)
        for (int j = 0; j < 4; ++j) op.coef[o][j] = df::splitConst(k[o][j]);
    return op;
}
// 0: exact FP64 (the default); 1: double-float for the general 2 x 2 gates
int g_plainArith = 0;

// QuEST_gpu.cu:1771-1826
struct OpHadamard {
    double f;
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        const double a = ur, b = ui, c = lr, d = li;
        ur = f * (a + c); ui = f * (b + d);
        lr = f * (a - c); li = f * (b - d);
    }
};

struct OpSwap {
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        double t = ur; ur = lr; lr = t;
        t = ui; ui = li; li = t;
    }
};

// QuEST_gpu.cu:1362-1455: up' = c*(im_lo, -re_lo), lo' = c*(-im_up, re_up)
struct OpPauliY {
    double c;
    __device__ __forceinline__ void operator()(double& ur, double& ui, double& lr, double& li) const {
        const double a = ur, b = ui, x = lr, y = li;
        ur = c * y; ui = -c * x;
        lr = -c * b; li = c * a;
    }
};

template <class Op>
__global__ void __launch_bounds__(kThreads) kPairVec(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                     uint64_t setMask, uint64_t pmask, uint64_t nThreads, Op op) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nThreads) return;
    const uint64_t i0 = insertZeros(t << 1, ins) | setMask;
    const uint64_t i1 = i0 ^ pmask;
    double2 ur = ld2(re + i0), ui = ld2(im + i0), lr = ld2(re + i1), li = ld2(im + i1);
    op(ur.x, ui.x, lr.x, li.x);
    op(ur.y, ui.y, lr.y, li.y);
    st2(re + i0, ur); st2(im + i0, ui); st2(re + i1, lr); st2(im + i1, li);
}

// partner bit is bit 0: (re[i0], re[i0+1]) is one pair; two pairs per thread
template <class Op>
__global__ void __launch_bounds__(kThreads) kPairAdj(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                     uint64_t setMask, uint64_t nThreads, Op op) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nThreads) return;
    const uint64_t a0 = insertZeros(t << 1, ins) | setMask;
    const uint64_t a1 = insertZeros((t << 1) | 1ull, ins) | setMask;
    double2 r0 = ld2(re + a0), i0 = ld2(im + a0), r1 = ld2(re + a1), i1 = ld2(im + a1);
    op(r0.x, i0.x, r0.y, i0.y);
    op(r1.x, i1.x, r1.y, i1.y);
    st2(re + a0, r0); st2(im + a0, i0); st2(re + a1, r1); st2(im + a1, i1);
}

template <class Op>
__global__ void __launch_bounds__(kThreads) kPairScalar(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                        uint64_t setMask, uint64_t pmask, uint64_t nPairs, Op op) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nPairs) return;
    const uint64_t i0 = insertZeros(t, ins) | setMask;
    const uint64_t i1 = i0 ^ pmask;
    double ur = re[i0], ui = im[i0], lr = re[i1], li = im[i1];
    op(ur, ui, lr, li);
    re[i0] = ur; im[i0] = ui; re[i1] = lr; im[i1] = li;
}

// Launch a pair gate: partner = i0 ^ pmask, lowBit = lowest bit of pmask
// (inserted as 0 in i0), ctrl bits inserted and set according to setMask.
template <class Op>
void launchPair(SV s, uint64_t ctrl, uint64_t setMask, uint64_t pmask, const Op& op, const char* caller) {
    const uint64_t lowBit = pmask & (~pmask + 1ull);
    const uint64_t insMask = ctrl | lowBit;
    const InsSpec ins = makeIns(insMask);
    const int free = s.n - ins.n;
    if (free < 0) return;
    const uint64_t nPairs = 1ull << free;
    cudaStream_t st = stream();
    if (nPairs >= 2 && !(insMask & 1ull)) {
        kPairVec<Op><<<blocksFor(nPairs / 2), kThreads, 0, st>>>(s.re, s.im, ins, setMask, pmask, nPairs / 2, op);
    } else if (nPairs >= 2 && pmask == 1ull) {
        kPairAdj<Op><<<blocksFor(nPairs / 2), kThreads, 0, st>>>(s.re, s.im, ins, setMask, nPairs / 2, op);
    } else {
        kPairScalar<Op><<<blocksFor(nPairs), kThreads, 0, st>>>(s.re, s.im, ins, setMask, pmask, nPairs, op);
    }
    launchFailed(caller);
}

// ------------------------------------------------------- elementwise (diagonal)
struct OpPhase {           // amp *= t
    double tr, ti;
    __device__ __forceinline__ void operator()(uint64_t, double& r, double& i) const {
        const double a = r, b = i;
        r = tr * a - ti * b;
        i = ti * a + tr * b;
    }
};

// QuEST_gpu.cu:1565-1591: even parity -> exp(-i a/2), odd -> exp(+i a/2)
struct OpRotZ {
    uint64_t targ;
    double c, s;
    __device__ __forceinline__ void operator()(uint64_t idx, double& r, double& i) const {
        const double fs = (__popcll(idx & targ) & 1) ? 1.0 : -1.0;
        const double a = r, b = i;
        r = c * a - fs * s * b;
        i = fs * s * a + c * b;
    }
};

template <class Op>
__global__ void __launch_bounds__(kThreads) kDiagVec(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                     uint64_t setMask, uint64_t nThreads, Op op) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nThreads) return;
    const uint64_t i0 = insertZeros(t << 1, ins) | setMask;
    double2 r = ld2(re + i0), m = ld2(im + i0);
    op(i0, r.x, m.x);
    op(i0 + 1, r.y, m.y);
    st2(re + i0, r); st2(im + i0, m);
}

template <class Op>
__global__ void __launch_bounds__(kThreads) kDiagScalar(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                        uint64_t setMask, uint64_t nAmps, Op op) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nAmps) return;
    const uint64_t i = insertZeros(t, ins) | setMask;
    double r = re[i], m = im[i];
    op(i, r, m);
    re[i] = r; im[i] = m;
}

template <class Op>
void launchDiag(SV s, uint64_t fixedMask, uint64_t setMask, const Op& op, const char* caller) {
    const InsSpec ins = makeIns(fixedMask);
    const int free = s.n - ins.n;
    if (free < 0) return;
    const uint64_t nAmps = 1ull << free;
    cudaStream_t st = stream();
    if (nAmps >= 2 && !(fixedMask & 1ull))
        kDiagVec<Op><<<blocksFor(nAmps / 2), kThreads, 0, st>>>(s.re, s.im, ins, setMask, nAmps / 2, op);
    else
        kDiagScalar<Op><<<blocksFor(nAmps), kThreads, 0, st>>>(s.re, s.im, ins, setMask, nAmps, op);
    launchFailed(caller);
}

// ------------------------------------------------------- Pauli-string rotation
// exp(-i a/2 P) in one pass over pairs (j, j^x).  (P psi)[j] =
// (-i)^nY (-1)^popc(j & (y|z)) psi[j^x]; new[j] = c psi[j] + s g sgn_j psi[j^x]
// with g = -i (-i)^nY (conj: conj(g)).  Replaces the basis-change sequence of
// QuEST_common.c:411-448 (2*#XY + 1 passes) by one pass.
struct PauliRot {
    uint64_t xmask, yz;
    double c, s, gr, gi;
};

__device__ __forceinline__ void pauliPair(const PauliRot& p, uint64_t j, double& jr, double& ji, double& kr, double& ki) {
    const uint64_t k = j ^ p.xmask;
    const double sj = (__popcll(j & p.yz) & 1) ? -p.s : p.s;
    const double sk = (__popcll(k & p.yz) & 1) ? -p.s : p.s;
    const double ar = jr, ai = ji, br = kr, bi = ki;
    // g*b
    const double gbr = p.gr * br - p.gi * bi, gbi = p.gr * bi + p.gi * br;
    const double gar = p.gr * ar - p.gi * ai, gai = p.gr * ai + p.gi * ar;
    jr = p.c * ar + sj * gbr; ji = p.c * ai + sj * gbi;
    kr = p.c * br + sk * gar; ki = p.c * bi + sk * gai;
}

__global__ void __launch_bounds__(kThreads) kPauliRotVec(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                         uint64_t setMask, uint64_t nThreads, PauliRot p) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nThreads) return;
    const uint64_t j0 = insertZeros(t << 1, ins) | setMask;
    const uint64_t k0 = j0 ^ p.xmask;
    double2 jr = ld2(re + j0), ji = ld2(im + j0), kr = ld2(re + k0), ki = ld2(im + k0);
    pauliPair(p, j0, jr.x, ji.x, kr.x, ki.x);
    pauliPair(p, j0 + 1, jr.y, ji.y, kr.y, ki.y);
    st2(re + j0, jr); st2(im + j0, ji); st2(re + k0, kr); st2(im + k0, ki);
}

__global__ void __launch_bounds__(kThreads) kPauliRotScalar(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                            uint64_t setMask, uint64_t nPairs, PauliRot p) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nPairs) return;
    const uint64_t j = insertZeros(t, ins) | setMask;
    const uint64_t k = j ^ p.xmask;
    double jr = re[j], ji = im[j], kr = re[k], ki = im[k];
    pauliPair(p, j, jr, ji, kr, ki);
    re[j] = jr; im[j] = ji; re[k] = kr; im[k] = ki;
}

// ------------------------------------------------------- swap (QuEST_gpu.cu:1737-1769)
__global__ void __launch_bounds__(kThreads) kSwap(double* __restrict__ re, double* __restrict__ im, InsSpec ins,
                                                  uint64_t b1, uint64_t b2, uint64_t n) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    const uint64_t base = insertZeros(t, ins);
    const uint64_t a = base | b1, b = base | b2;
    const double r = re[a], m = im[a];
    re[a] = re[b]; im[a] = im[b];
    re[b] = r; im[b] = m;
}

// ------------------------------------------------------- dense k-qubit matrix
// One block handles G groups of D = 2^k amplitudes; thread (r, g) loads
// amplitude r of group g, then computes row r of M . v_g from shared memory.
// Consecutive threads take consecutive groups so the loads of one row index
// coalesce when the targets are above the low qubits.
__global__ void kMatrixN(double* __restrict__ re, double* __restrict__ im, InsSpec ins, uint64_t setMask,
                         int k, const int* __restrict__ targs, const double* __restrict__ mr,
                         const double* __restrict__ mi, uint64_t nGroups, int G) {
    extern __shared__ double sm[];
    const int D = 1 << k;
    double* vr = sm;
    double* vi = sm + (size_t)D * G;
    const int g = threadIdx.x % G;
    const int r = threadIdx.x / G;
    const uint64_t grp = (uint64_t)blockIdx.x * G + g;
    const bool live = grp < nGroups;
    uint64_t addr = 0;
    if (live) {
        addr = insertZeros(grp, ins) | setMask;
        for (int b = 0; b < k; ++b)
            if (r >> b & 1) addr |= 1ull << targs[b];
        vr[r * G + g] = re[addr];
        vi[r * G + g] = im[addr];
    }
    __syncthreads();
    if (!live) return;
    double sr = 0.0, si = 0.0;
    const double* rowr = mr + (size_t)r * D;
    const double* rowi = mi + (size_t)r * D;
    for (int c = 0; c < D; ++c) {
        const double ar = __ldg(rowr + c), ai = __ldg(rowi + c);
        const double xr = vr[c * G + g], xi = vi[c * G + g];
        sr += ar * xr - ai * xi;
        si += ar * xi + ai * xr;
    }
    re[addr] = sr;
    im[addr] = si;
}

// device staging for gateMatrixN (matrix + targets), grown on demand
double* g_matBuf = nullptr;
size_t g_matCap = 0;

}  // namespace

// --------------------------------------------------------------- launchers
void gateMatrix2(SV s, int target, uint64_t ctrl, uint64_t flip, const Mat2& u) {   // QuEST_gpu.cu:966, 1231, 1299
    if (s.cap) {
        const double ur[4] = {u.r[0][0], u.r[0][1], u.r[1][0], u.r[1][1]}, ui[4] = {u.i[0][0], u.i[0][1], u.i[1][0], u.i[1][1]};
        if (capturePair(s, target, ctrl, flip, ur, ui)) return;
    }
    if (g_plainArith == 1) launchPair(s, ctrl, ctrl & ~flip, 1ull << target, matrix2DF(u), "unitary");
    else launchPair(s, ctrl, ctrl & ~flip, 1ull << target, OpMatrix2{u}, "unitary");
}

void gateCompact(SV s, int target, uint64_t ctrl, double ar, double ai, double br, double bi) {   // QuEST_gpu.cu:838, 905
    if (s.cap) {
        const double ur[4] = {ar, -br, br, ar}, ui[4] = {ai, bi, bi, -ai};     // [alpha, -conj(beta); beta, conj(alpha)]
        if (capturePair(s, target, ctrl, 0, ur, ui)) return;
    }
    if (g_plainArith == 1) {
        Mat2 m;                                            // [alpha, -conj(beta); beta, conj(alpha)]
        m.r[0][0] = ar; m.i[0][0] = ai; m.r[0][1] = -br; m.i[0][1] = bi;
        m.r[1][0] = br; m.i[1][0] = bi; m.r[1][1] = ar; m.i[1][1] = -ai;
        launchPair(s, ctrl, ctrl, 1ull << target, matrix2DF(m), "compactUnitary");
        return;
    }
    launchPair(s, ctrl, ctrl, 1ull << target, OpCompact{ar, ai, br, bi}, "compactUnitary");
}

void gateHadamard(SV s, int target) {                                                // QuEST_gpu.cu:1820
    if (s.cap) {
        const double f = 0.70710678118654752440;
        const double ur[4] = {f, f, f, -f}, ui[4] = {0, 0, 0, 0};
        if (capturePair(s, target, 0, 0, ur, ui)) return;
    }
    if (g_plainArith == 1) {
        const double f = 0.70710678118654752440;
        Mat2 m{{{f, f}, {f, -f}}, {{0, 0}, {0, 0}}};
        launchPair(s, 0, 0, 1ull << target, matrix2DF(m), "hadamard");
        return;
    }
    launchPair(s, 0, 0, 1ull << target, OpHadamard{0.70710678118654752440}, "hadamard");
}

bool setPlainArithmetic(int mode) {
    if (mode != 0 && mode != 1) return false;
    g_plainArith = mode;
    return true;
}
int plainArithmetic() { return g_plainArith; }

void gateNot(SV s, uint64_t ctrl, uint64_t targMask) {                               // QuEST_gpu.cu:1354, 1867, 1912
    if (s.cap && captureNot(s, ctrl, targMask)) return;
    launchPair(s, ctrl, ctrl, targMask, OpSwap{}, "controlledNot");
}

void gatePauliY(SV s, int target, uint64_t ctrl, double conjFac) {                   // QuEST_gpu.cu:1387, 1439
    if (s.cap) {
        const double ur[4] = {0, 0, 0, 0}, ui[4] = {0, -conjFac, conjFac, 0};   // [0, -i; i, 0] (conjugated: conjFac = -1)
        if (capturePair(s, target, ctrl, 0, ur, ui)) return;
    }
    launchPair(s, ctrl, ctrl, 1ull << target, OpPauliY{conjFac}, "pauliY");
}

void gatePhase(SV s, uint64_t mask, double tr, double ti) {                          // QuEST_gpu.cu:1485, 1521, 1552, 1702
    if (s.cap && capturePhase(s, mask, tr, ti)) return;
    launchDiag(s, mask, mask, OpPhase{tr, ti}, "phaseShift");
}

void gateRotateZ(SV s, uint64_t ctrl, uint64_t targ, double angle) {                 // QuEST_gpu.cu:1582, 1615
    if (s.cap && captureRotateZ(s, ctrl, targ, angle)) return;
    launchDiag(s, ctrl, ctrl, OpRotZ{targ, cos(angle / 2), sin(angle / 2)}, "multiRotateZ");
}

void gatePauliRotation(SV s, uint64_t ctrl, uint64_t xmask, uint64_t ymask, uint64_t zmask, double angle, int conj) {
    if (s.cap && capturePauliRotation(s, ctrl, xmask, ymask, zmask, angle, conj)) return;
    if (xmask == 0) {                                      // diagonal: plain Z-rotation on the Y/Z-free mask
        gateRotateZ(s, ctrl, zmask, conj ? -angle : angle);
        return;
    }
    const int nY = __builtin_popcountll(ymask);
    // g = -i * (-i)^nY
    static const double pr[4] = {1, 0, -1, 0}, pi[4] = {0, -1, 0, 1};   // (-i)^m
    const int m = (nY + 1) & 3;
    PauliRot p;
    p.xmask = xmask;
    p.yz = ymask | zmask;
    p.c = cos(angle / 2);
    p.s = sin(angle / 2);
    p.gr = pr[m];
    p.gi = conj ? -pi[m] : pi[m];
    const uint64_t lowBit = xmask & (~xmask + 1ull);
    const uint64_t insMask = ctrl | lowBit;
    const InsSpec ins = makeIns(insMask);
    const int free = s.n - ins.n;
    if (free < 0) return;
    const uint64_t nPairs = 1ull << free;
    cudaStream_t st = stream();
    if (nPairs >= 2 && !(insMask & 1ull) && !(xmask & 1ull))
        kPauliRotVec<<<blocksFor(nPairs / 2), kThreads, 0, st>>>(s.re, s.im, ins, ctrl, nPairs / 2, p);
    else
        kPauliRotScalar<<<blocksFor(nPairs), kThreads, 0, st>>>(s.re, s.im, ins, ctrl, nPairs, p);
    launchFailed("multiRotatePauli");
}

void gateSwap(SV s, int q1, int q2) {
    if (s.cap && captureSwap(s, q1, q2)) return;
    const InsSpec ins = makeIns((1ull << q1) | (1ull << q2));
    const uint64_t n = 1ull << (s.n - 2);
    kSwap<<<blocksFor(n), kThreads, 0, stream()>>>(s.re, s.im, ins, 1ull << q1, 1ull << q2, n);
    launchFailed("swapGate");
}

void gateMatrixN(SV s, uint64_t ctrl, const int* targs, int k, const double* mr, const double* mi) {   // QuEST_gpu.cu:1033, 1166
    if (s.cap && captureMatrixN(s, ctrl, targs, k, mr, mi)) return;
    const int D = 1 << k;
    const size_t matDoubles = 2 * (size_t)D * D;
    const size_t need = matDoubles * sizeof(double) + 64 * sizeof(int);
    if (need > g_matCap) {
        if (g_matBuf) cudaFree(g_matBuf);
        g_matBuf = nullptr;
        g_matCap = 0;
        if (QG_CUDA(cudaMalloc(&g_matBuf, need), "multiQubitUnitary")) return;
        g_matCap = need;
    }
    // pageable sources: cudaMemcpyAsync returns once the host data is staged,
    // so the caller's arrays may be reused immediately.
    std::vector<double> host(matDoubles);
    std::copy(mr, mr + (size_t)D * D, host.begin());
    std::copy(mi, mi + (size_t)D * D, host.begin() + (size_t)D * D);
    int tg[64];
    for (int i = 0; i < k; ++i) tg[i] = targs[i];
    cudaStream_t st = stream();
    if (QG_CUDA(cudaMemcpyAsync(g_matBuf, host.data(), matDoubles * sizeof(double), cudaMemcpyHostToDevice, st), "multiQubitUnitary")) return;
    int* dT = reinterpret_cast<int*>(g_matBuf + matDoubles);
    if (QG_CUDA(cudaMemcpyAsync(dT, tg, k * sizeof(int), cudaMemcpyHostToDevice, st), "multiQubitUnitary")) return;
    uint64_t tmask = 0;
    for (int i = 0; i < k; ++i) tmask |= 1ull << targs[i];
    const InsSpec ins = makeIns(tmask | ctrl);
    const int free = s.n - ins.n;
    if (free < 0) return;
    const uint64_t nGroups = 1ull << free;
    int G = std::max(1, 256 / D);
    if ((uint64_t)G > nGroups) G = (int)nGroups;
    const int threads = G * D;
    const unsigned blocks = (unsigned)((nGroups + G - 1) / G);
    const size_t smem = 2 * (size_t)D * G * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(kMatrixN, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kMatrixN<<<blocks, threads, smem, st>>>(s.re, s.im, ins, ctrl, k, dT, g_matBuf, g_matBuf + (size_t)D * D, nGroups, G);
    launchFailed("multiQubitUnitary");
}

}  // namespace qg

extern "C" {
/* Arithmetic of the plain path's general 2 x 2 gates (compactUnitary and the
 * rotations built on it, unitary and its controlled forms, hadamard): 0 =
 * exact FP64 (the default), 1 = double-float on the FP32 and integer pipes
 * (df64.cuh).  Returns 0, or -1 for an unknown mode. */
int quest_gb300_setPlainArithmetic(int mode) { return qg::setPlainArithmetic(mode) ? 0 : -1; }
int quest_gb300_getPlainArithmetic(void) { return qg::plainArithmetic(); }
}
