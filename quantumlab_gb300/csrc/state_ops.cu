// state_ops.cu -- initialisation, elementwise combinations, measurement
// collapse and the density-matrix channels (FP64, sm_103a).
//
// Channel semantics follow Code/QuEST340/QuEST/src/QuEST.c:1259-1298 and the
// GPU kernels of QuEST_gpu.cu:2868-3078: the reference runs depolarising and
// damping as two launches (an off-diagonal pass, then a diagonal pass); here
// each channel is one pass over groups of the four entries
// {rho[.0..0.], rho[.0..1.], rho[.1..0.], rho[.1..1.]} (row bit t, column bit
// t+N), with the same per-entry arithmetic.
#include "qg_internal.h"

#include <type_traits>

namespace qg {
namespace {

constexpr int kThreads = 256;
inline unsigned blocksFor(uint64_t threads) { return (unsigned)((threads + kThreads - 1) / kThreads); }

__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ void st2(double* p, double2 v) { *reinterpret_cast<double2*>(p) = v; }
__device__ __forceinline__ uint64_t ins2(uint64_t k, int lo, int hi) {     // insert zeros at lo < hi
    k = ((k >> lo) << (lo + 1)) | (k & ((1ull << lo) - 1ull));
    k = ((k >> hi) << (hi + 1)) | (k & ((1ull << hi) - 1ull));
    return k;
}

// ---------------------------------------------------------------- fills
__global__ void kFill(double* __restrict__ re, double* __restrict__ im, uint64_t n2, double vr, double vi) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n2) return;
    st2(re + 2 * t, make_double2(vr, vr));
    st2(im + 2 * t, make_double2(vi, vi));
}

// Product state of registers on consecutive qubit ranges (register r on
// qubits [off_r, off_r + bits_r), its vector at base_r in vr/vi); qubits above
// the registers are |0>.  No counterpart in the reference.
constexpr int kMaxProductRegs = 16;
struct ProductSpec {
    int numRegs;
    int off[kMaxProductRegs], bits[kMaxProductRegs];
    uint64_t base[kMaxProductRegs];
};
__global__ void kProduct(double* __restrict__ re, double* __restrict__ im, const double* __restrict__ vr,
                         const double* __restrict__ vi, const ProductSpec ps, uint64_t used, uint64_t n) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    double ar = 0.0, ai = 0.0;
    if (t < used) {
        ar = 1.0;
        for (int r = 0; r < ps.numRegs; ++r) {
            const uint64_t f = ps.base[r] + ((t >> ps.off[r]) & ((1ull << ps.bits[r]) - 1ull));
            const double br = vr[f], bi = vi[f];
            const double nr = ar * br - ai * bi;
            ai = ar * bi + ai * br;
            ar = nr;
        }
    }
    re[t] = ar;
    im[t] = ai;
}

// QuEST_gpu.cu:659-684 (initDebugState): amp_k = (2k + i(2k+1)) / 10
__global__ void kDebug(double* __restrict__ re, double* __restrict__ im, uint64_t n) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    re[t] = (t * 2.0) / 10.0;
    im[t] = (t * 2.0 + 1.0) / 10.0;
}

// rho[r + c D] = psi_r conj(psi_c)  (QuEST_gpu.cu:188-228)
__global__ void kPureDM(double* __restrict__ re, double* __restrict__ im, const double* __restrict__ pr,
                        const double* __restrict__ pi, int nRep, uint64_t n) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    const uint64_t D = 1ull << nRep;
    const uint64_t r = t & (D - 1), c = t >> nRep;
    const double ar = pr[r], ai = pi[r], br = pr[c], bi = -pi[c];
    re[t] = ar * br - ai * bi;
    im[t] = ar * bi + ai * br;
}

// out = f1 a + f2 b + fo out  (QuEST_gpu.cu:3148-3190)
__global__ void kWeighted(double* __restrict__ oR, double* __restrict__ oI, const double* __restrict__ aR,
                          const double* __restrict__ aI, const double* __restrict__ bR, const double* __restrict__ bI,
                          double f1r, double f1i, double f2r, double f2i, double for_, double foi, uint64_t n) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    const double ar = aR[t], ai = aI[t], br = bR[t], bi = bI[t], xr = oR[t], xi = oI[t];
    oR[t] = f1r * ar - f1i * ai + f2r * br - f2i * bi + for_ * xr - foi * xi;
    oI[t] = f1r * ai + f1i * ar + f2r * bi + f2i * br + for_ * xi + foi * xr;
}

// a = (1-p) a + p b  (QuEST_gpu.cu:2839-2866)
__global__ void kMixDM(double* __restrict__ aR, double* __restrict__ aI, const double* __restrict__ bR,
                       const double* __restrict__ bI, double p, uint64_t n2) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n2) return;
    double2 ar = ld2(aR + 2 * t), ai = ld2(aI + 2 * t);
    const double2 br = ld2(bR + 2 * t), bi = ld2(bI + 2 * t);
    const double q = 1 - p;
    ar.x = ar.x * q + p * br.x; ar.y = ar.y * q + p * br.y;
    ai.x = ai.x * q + p * bi.x; ai.y = ai.y * q + p * bi.y;
    st2(aR + 2 * t, ar); st2(aI + 2 * t, ai);
}

// ---------------------------------------------------------------- collapse
// keep amps whose bit t == outcome (scaled), zero the rest (QuEST_gpu.cu:2718-2781)
__global__ void kCollapseSV(double* __restrict__ re, double* __restrict__ im, uint64_t n2, uint64_t tbit,
                            int outcome, double renorm) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n2) return;
    const uint64_t i = 2 * t;
    double2 r = ld2(re + i), m = ld2(im + i);
    const double f0 = (((i & tbit) != 0) == (outcome != 0)) ? renorm : 0.0;
    const double f1 = ((((i + 1) & tbit) != 0) == (outcome != 0)) ? renorm : 0.0;
    r.x *= f0; m.x *= f0; r.y *= f1; m.y *= f1;
    st2(re + i, r); st2(im + i, m);
}

// DM: keep entries whose row and column bits both equal outcome, / prob
// (QuEST_gpu.cu:2784-2837; 64-bit bit tests here, the reference uses int)
__global__ void kCollapseDM(double* __restrict__ re, double* __restrict__ im, uint64_t n2, uint64_t rbit,
                            uint64_t cbit, int outcome, double renorm) {
    const uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (t >= n2) return;
    const uint64_t i = 2 * t;
    double2 r = ld2(re + i), m = ld2(im + i);
    const uint64_t want = outcome ? (rbit | cbit) : 0;
    const double f0 = ((i & (rbit | cbit)) == want) ? renorm : 0.0;
    const double f1 = (((i + 1) & (rbit | cbit)) == want) ? renorm : 0.0;
    r.x *= f0; m.x *= f0; r.y *= f1; m.y *= f1;
    st2(re + i, r); st2(im + i, m);
}

// ---------------------------------------------------------------- channels
// The four entries of one group: e00 = base, e01 = base|row, e10 = base|col,
// e11 = base|row|col.  Off-diagonal-in-t entries are e01, e10.
struct Dephase {
    double retain;
    __device__ __forceinline__ void operator()(double&, double&, double& r01, double& i01, double& r10, double& i10,
                                               double&, double&) const {
        r01 *= retain; i01 *= retain; r10 *= retain; i10 *= retain;
    }
};
// QuEST_gpu.cu:2980-3004 (after the 1-level dephase): both diagonal entries
// become (1-l) x + l (x+y)/2
struct Depolarise {
    double level;
    __device__ __forceinline__ void operator()(double& r00, double& i00, double& r01, double& i01, double& r10,
                                               double& i10, double& r11, double& i11) const {
        const double retain = 1 - level;
        r01 *= retain; i01 *= retain; r10 *= retain; i10 *= retain;
        const double avr = level * 0.5 * (r00 + r11), avi = level * 0.5 * (i00 + i11);
        r00 = r00 * retain + avr; i00 = i00 * retain + avi;
        r11 = r11 * retain + avr; i11 = i11 * retain + avi;
    }
};
// QuEST_gpu.cu:3006-3078: off-diagonals * sqrt(1-p); rho00 += p rho11; rho11 *= 1-p
struct Damp {
    double p, dephase;
    __device__ __forceinline__ void operator()(double& r00, double& i00, double& r01, double& i01, double& r10,
                                               double& i10, double& r11, double& i11) const {
        r01 *= dephase; i01 *= dephase; r10 *= dephase; i10 *= dephase;
        const double tr = p * r11, ti = p * i11;
        r11 *= 1 - p; i11 *= 1 - p;
        r00 += tr; i00 += ti;
    }
};

// Pauli channel (1 - pX - pY - pZ) rho + pX X rho X + pY Y rho Y + pZ Z rho Z
// (QuEST.c:1312, QuEST_common.c:740-759, which applies it as the Kraus
// superoperator of those four operators): the diagonal pair exchanges weight
// pX + pY, the off-diagonal pair keeps 1 - pX - pY - 2 pZ and exchanges pX - pY.
struct PauliMix {
    double diagKeep, diagSwap, offKeep, offSwap;
    __device__ __forceinline__ void operator()(double& r00, double& i00, double& r01, double& i01, double& r10,
                                               double& i10, double& r11, double& i11) const {
        const double a = r00, b = i00, c = r01, d = i01;
        r00 = diagKeep * a + diagSwap * r11; i00 = diagKeep * b + diagSwap * i11;
        r11 = diagKeep * r11 + diagSwap * a; i11 = diagKeep * i11 + diagSwap * b;
        r01 = offKeep * c + offSwap * r10; i01 = offKeep * d + offSwap * i10;
        r10 = offKeep * r10 + offSwap * c; i10 = offKeep * i10 + offSwap * d;
    }
};

// row bit t >= 1: two consecutive groups per thread with double2 loads
template <class Op>
__global__ void __launch_bounds__(kThreads) kChannelVec(double* __restrict__ re, double* __restrict__ im, int t, int N,
                                                        uint64_t nThreads, Op op) {
    const uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (k >= nThreads) return;
    const uint64_t rb = 1ull << t, cb = 1ull << (t + N);
    const uint64_t b = ins2(k << 1, t, t + N);
    double2 r00 = ld2(re + b), i00 = ld2(im + b);
    double2 r01 = ld2(re + (b | rb)), i01 = ld2(im + (b | rb));
    double2 r10 = ld2(re + (b | cb)), i10 = ld2(im + (b | cb));
    double2 r11 = ld2(re + (b | rb | cb)), i11 = ld2(im + (b | rb | cb));
    op(r00.x, i00.x, r01.x, i01.x, r10.x, i10.x, r11.x, i11.x);
    op(r00.y, i00.y, r01.y, i01.y, r10.y, i10.y, r11.y, i11.y);
    st2(re + b, r00); st2(im + b, i00);
    st2(re + (b | rb), r01); st2(im + (b | rb), i01);
    st2(re + (b | cb), r10); st2(im + (b | cb), i10);
    st2(re + (b | rb | cb), r11); st2(im + (b | rb | cb), i11);
}

// row bit t == 0: (e00, e01) and (e10, e11) are adjacent pairs
template <class Op>
__global__ void __launch_bounds__(kThreads) kChannelT0(double* __restrict__ re, double* __restrict__ im, int N,
                                                       uint64_t nGroups, Op op) {
    const uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (k >= nGroups) return;
    const uint64_t cb = 1ull << N;
    const uint64_t b = ins2(k, 0, N);
    double2 rA = ld2(re + b), iA = ld2(im + b), rB = ld2(re + (b | cb)), iB = ld2(im + (b | cb));
    op(rA.x, iA.x, rA.y, iA.y, rB.x, iB.x, rB.y, iB.y);
    st2(re + b, rA); st2(im + b, iA); st2(re + (b | cb), rB); st2(im + (b | cb), iB);
}

template <class Op>
void launchChannel(SV s, int t, int N, const Op& op, const char* caller) {
    const uint64_t nGroups = 1ull << (s.n - 2);
    if (t >= 1 && nGroups >= 2)
        kChannelVec<Op><<<blocksFor(nGroups / 2), kThreads, 0, stream()>>>(s.re, s.im, t, N, nGroups / 2, op);
    else
        kChannelT0<Op><<<blocksFor(nGroups), kThreads, 0, stream()>>>(s.re, s.im, N, nGroups, op);
    launchFailed(caller);
}

// Two-qubit channels on a density matrix (QuEST_gpu.cu:2912-2978, 3080-3147).
// A group is the 16 entries that differ only in the bits b[0] < b[1] < b[2] <
// b[3] = (q1, q2, q1 + N, q2 + N); local index j has bit i = bit b[i].  The
// four entries whose row and column bits agree on both qubits (j = 0, 5, 10,
// 15) become diagRetain x + mix (sum of the four); the other twelve are
// scaled by retain.  Dephasing: retain = 1 - 4p/3, diagRetain = 1, no mix.
// Depolarising: retain = diagRetain = 1 - l, mix = l/4, l = 16p/15 (the
// reference's dephase launch followed by its averaging launch, in one pass).
// V = 2: two consecutive groups per thread with 16-byte accesses (b[0] >= 1).
struct TwoQubitBits {
    int b[4];
};
template <int V, bool MIX>
__global__ void __launch_bounds__(kThreads) kTwoQubitChannel(double* __restrict__ re, double* __restrict__ im,
                                                             const TwoQubitBits tb, uint64_t nThreads, double retain,
                                                             double diagRetain, double mix) {
    typedef typename std::conditional<V == 2, double2, double>::type vec;
    const uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (k >= nThreads) return;
    uint64_t base = k * V;
#pragma unroll
    for (int i = 0; i < 4; ++i) base = ((base >> tb.b[i]) << (tb.b[i] + 1)) | (base & ((1ull << tb.b[i]) - 1ull));
    auto at = [&](int j) {
        uint64_t o = base;
#pragma unroll
        for (int i = 0; i < 4; ++i) o |= (uint64_t)((j >> i) & 1) << tb.b[i];
        return o;
    };
    if (MIX) {
        const int dj[4] = {0, 5, 10, 15};
        vec r[4], m[4];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            r[d] = *reinterpret_cast<const vec*>(re + at(dj[d]));
            m[d] = *reinterpret_cast<const vec*>(im + at(dj[d]));
        }
        if constexpr (V == 2) {
            const double sx = mix * (r[0].x + r[1].x + r[2].x + r[3].x), sy = mix * (r[0].y + r[1].y + r[2].y + r[3].y);
            const double tx = mix * (m[0].x + m[1].x + m[2].x + m[3].x), ty = mix * (m[0].y + m[1].y + m[2].y + m[3].y);
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                r[d].x = r[d].x * diagRetain + sx; r[d].y = r[d].y * diagRetain + sy;
                m[d].x = m[d].x * diagRetain + tx; m[d].y = m[d].y * diagRetain + ty;
            }
        } else {
            const double sx = mix * (r[0] + r[1] + r[2] + r[3]), tx = mix * (m[0] + m[1] + m[2] + m[3]);
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                r[d] = r[d] * diagRetain + sx;
                m[d] = m[d] * diagRetain + tx;
            }
        }
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            *reinterpret_cast<vec*>(re + at(dj[d])) = r[d];
            *reinterpret_cast<vec*>(im + at(dj[d])) = m[d];
        }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        if (j == 0 || j == 5 || j == 10 || j == 15) continue;
        const uint64_t o = at(j);
        vec r = *reinterpret_cast<const vec*>(re + o), m = *reinterpret_cast<const vec*>(im + o);
        if constexpr (V == 2) {
            r.x *= retain; r.y *= retain; m.x *= retain; m.y *= retain;
        } else {
            r *= retain; m *= retain;
        }
        *reinterpret_cast<vec*>(re + o) = r;
        *reinterpret_cast<vec*>(im + o) = m;
    }
}

template <bool MIX>
void launchTwoQubitChannel(SV s, int q1, int q2, int N, double retain, double diagRetain, double mix,
                           const char* caller) {
    const TwoQubitBits tb{{q1, q2, q1 + N, q2 + N}};
    const uint64_t nGroups = 1ull << (s.n - 4);
    if (q1 >= 1)
        kTwoQubitChannel<2, MIX><<<blocksFor(nGroups / 2), kThreads, 0, stream()>>>(s.re, s.im, tb, nGroups / 2,
                                                                                  retain, diagRetain, mix);
    else
        kTwoQubitChannel<1, MIX><<<blocksFor(nGroups), kThreads, 0, stream()>>>(s.re, s.im, tb, nGroups, retain,
                                                                               diagRetain, mix);
    launchFailed(caller);
}

// the 16 x 16 superoperator of a two-qubit channel on the local qubits
// (q1, q2, q1 + N, q2 + N), for the op-stream capture
void twoQubitSuperop(double retain, double diagRetain, double mix, double S[256]) {
    for (int i = 0; i < 256; ++i) S[i] = 0;
    for (int j = 0; j < 16; ++j) {
        const bool diag = (j == 0 || j == 5 || j == 10 || j == 15);
        if (!diag) {
            S[17 * j] = retain;
            continue;
        }
        for (int c : {0, 5, 10, 15}) S[16 * j + c] = mix;
        S[17 * j] += diagRetain;
    }
}

}  // namespace

// vectors (host, unit norm), regBits per register, concatenated in vr / vi
void stateProduct(SV s, int numRegs, const int* regBits, const double* vr, const double* vi) {
    static double* buf = nullptr;          // grow-only device copy of the vectors
    static size_t cap = 0;
    ProductSpec ps{};
    ps.numRegs = numRegs;
    uint64_t len = 0;
    int off = 0;
    for (int r = 0; r < numRegs; ++r) {
        ps.off[r] = off;
        ps.bits[r] = regBits[r];
        ps.base[r] = len;
        off += regBits[r];
        len += 1ull << regBits[r];
    }
    cudaStream_t st = stream();
    if (2 * len > cap) {
        if (buf) {
            cudaStreamSynchronize(st);
            cudaFree(buf);
        }
        buf = nullptr;
        cap = 0;
        if (QG_CUDA(cudaMalloc(&buf, 2 * len * sizeof(double)), "initProductState")) return;
        cap = 2 * len;
    }
    // pageable sources: the copies return once the host data is staged
    if (QG_CUDA(cudaMemcpyAsync(buf, vr, len * sizeof(double), cudaMemcpyHostToDevice, st), "initProductState")) return;
    if (QG_CUDA(cudaMemcpyAsync(buf + len, vi, len * sizeof(double), cudaMemcpyHostToDevice, st), "initProductState")) return;
    const uint64_t n = 1ull << s.n;
    kProduct<<<blocksFor(n), kThreads, 0, st>>>(s.re, s.im, buf, buf + len, ps, 1ull << off, n);
    launchFailed("initProductState");
}

void stateFill(SV s, double vr, double vi) {
    const uint64_t n = 1ull << s.n;
    cudaStream_t st = stream();
    if (vr == 0.0 && vi == 0.0) {
        if (QG_CUDA(cudaMemsetAsync(s.re, 0, n * sizeof(double), st), "initBlankState")) return;
        QG_CUDA(cudaMemsetAsync(s.im, 0, n * sizeof(double), st), "initBlankState");
        return;
    }
    if (n < 2) {
        double v[2] = {vr, vi};
        QG_CUDA(cudaMemcpyAsync(s.re, &v[0], sizeof(double), cudaMemcpyHostToDevice, st), "initPlusState");
        QG_CUDA(cudaMemcpyAsync(s.im, &v[1], sizeof(double), cudaMemcpyHostToDevice, st), "initPlusState");
        QG_CUDA(cudaStreamSynchronize(st), "initPlusState");
        return;
    }
    kFill<<<blocksFor(n / 2), kThreads, 0, st>>>(s.re, s.im, n / 2, vr, vi);
    launchFailed("initPlusState");
}

void stateSetOne(SV s, idx_t index, double vr, double vi) {
    cudaStream_t st = stream();
    // pageable source: the copy stages the values before returning
    double v[2] = {vr, vi};
    if (QG_CUDA(cudaMemcpyAsync(s.re + index, &v[0], sizeof(double), cudaMemcpyHostToDevice, st), "initClassicalState")) return;
    QG_CUDA(cudaMemcpyAsync(s.im + index, &v[1], sizeof(double), cudaMemcpyHostToDevice, st), "initClassicalState");
}

void stateDebug(SV s) {
    const uint64_t n = 1ull << s.n;
    kDebug<<<blocksFor(n), kThreads, 0, stream()>>>(s.re, s.im, n);
    launchFailed("initDebugState");
}

void statePlusDM(SV s, int nRep) { stateFill(s, 1.0 / (double)(1ull << nRep), 0.0); }

void statePureDM(SV rho, const double* pr, const double* pi, int nRep) {
    const uint64_t n = 1ull << rho.n;
    kPureDM<<<blocksFor(n), kThreads, 0, stream()>>>(rho.re, rho.im, pr, pi, nRep, n);
    launchFailed("initPureState");
}

void stateWeighted(SV out, double f1r, double f1i, SV a, double f2r, double f2i, SV b, double for_, double foi) {
    const uint64_t n = 1ull << out.n;
    kWeighted<<<blocksFor(n), kThreads, 0, stream()>>>(out.re, out.im, a.re, a.im, b.re, b.im, f1r, f1i, f2r, f2i, for_, foi, n);
    launchFailed("setWeightedQureg");
}

void stateMixDM(SV a, double p, SV b) {
    const uint64_t n = 1ull << a.n;
    kMixDM<<<blocksFor(n / 2), kThreads, 0, stream()>>>(a.re, a.im, b.re, b.im, p, n / 2);
    launchFailed("mixDensityMatrix");
}

void collapseSV(SV s, int target, int outcome, double renorm) {
    const uint64_t n = 1ull << s.n;
    kCollapseSV<<<blocksFor(n / 2), kThreads, 0, stream()>>>(s.re, s.im, n / 2, 1ull << target, outcome, renorm);
    launchFailed("collapseToOutcome");
}

void collapseDM(SV s, int target, int nRep, int outcome, double renorm) {
    const uint64_t n = 1ull << s.n;
    kCollapseDM<<<blocksFor(n / 2), kThreads, 0, stream()>>>(s.re, s.im, n / 2, 1ull << target, 1ull << (target + nRep),
                                                             outcome, renorm);
    launchFailed("collapseToOutcome");
}

// With capture on, each channel is queued as its superoperator on
// (t, t + N), local index = row bit + 2 column bit (the functors above)
void dmDephase(SV s, int t, int N, double retain) {
    const double S[16] = {1, 0, 0, 0, 0, retain, 0, 0, 0, 0, retain, 0, 0, 0, 0, 1};
    if (s.cap && captureChannel(s, t, N, S)) return;
    launchChannel(s, t, N, Dephase{retain}, "mixDephasing");
}
void dmDepolarise(SV s, int t, int N, double level) {
    const double d = 1 - level / 2, x = level / 2, o = 1 - level;
    const double S[16] = {d, 0, 0, x, 0, o, 0, 0, 0, 0, o, 0, x, 0, 0, d};
    if (s.cap && captureChannel(s, t, N, S)) return;
    launchChannel(s, t, N, Depolarise{level}, "mixDepolarising");
}
void dmPauli(SV s, int t, int N, double pX, double pY, double pZ) {
    const PauliMix op{1 - pX - pY, pX + pY, 1 - pX - pY - 2 * pZ, pX - pY};
    const double S[16] = {op.diagKeep, 0, 0, op.diagSwap, 0, op.offKeep, op.offSwap, 0,
                          0, op.offSwap, op.offKeep, 0, op.diagSwap, 0, 0, op.diagKeep};
    if (s.cap && captureChannel(s, t, N, S)) return;
    launchChannel(s, t, N, op, "mixPauli");
}
void dmTwoQubitDephase(SV s, int q1, int q2, int N, double retain) {
    if (s.cap) {
        double S[256];
        twoQubitSuperop(retain, 1.0, 0.0, S);
        if (captureChannelN(s, (1ull << q1) | (1ull << q2) | (1ull << (q1 + N)) | (1ull << (q2 + N)), S)) return;
    }
    launchTwoQubitChannel<false>(s, q1, q2, N, retain, 1.0, 0.0, "mixTwoQubitDephasing");
}
void dmTwoQubitDepolarise(SV s, int q1, int q2, int N, double level) {
    const double retain = 1 - level, mix = level * 0.25;
    if (s.cap) {
        double S[256];
        twoQubitSuperop(retain, retain, mix, S);
        if (captureChannelN(s, (1ull << q1) | (1ull << q2) | (1ull << (q1 + N)) | (1ull << (q2 + N)), S)) return;
    }
    launchTwoQubitChannel<true>(s, q1, q2, N, retain, retain, mix, "mixTwoQubitDepolarising");
}
void dmDamp(SV s, int t, int N, double p) {
    const double o = sqrt(1 - p);
    const double S[16] = {1, 0, 0, p, 0, o, 0, 0, 0, 0, o, 0, 0, 0, 0, 1 - p};
    if (s.cap && captureChannel(s, t, N, S)) return;
    launchChannel(s, t, N, Damp{p, o}, "mixDamping");
}

}  // namespace qg
