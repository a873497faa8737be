// reduce.cu -- FP64 reductions in one launch each (sm_103a).
//
// The reference (Code/QuEST340/QuEST/src/GPU/QuEST_gpu.cu:1926-2483) reduces
// level by level with a 512-wide shared-memory tree and a
// cudaDeviceSynchronize per level, runs complex inner products twice (real,
// imaginary), and computes calcTotalProb by copying the whole state to the
// host (:1626-1679).  Here every reduction is a single pass: each thread keeps
// FP64 partial sums of two components, warps combine with
// shuffles, blocks through shared memory, and the last block to finish (a
// ticket counter in the register's scratch) adds the per-block partials in a
// fixed order.  The partial layout depends only on the problem size, so
// results are deterministic run to run.  One scalar pair is copied back.
#include "reduce_kernel.cuh"

#include <algorithm>

namespace qg {
namespace {

using namespace red;
constexpr int kThreads = red::kThreads;

// ------------------------------------------------------------------ functors
struct NormSq2 {          // two consecutive amplitudes per item
    const double *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double2 r = ld2(re + 2 * i), m = ld2(im + 2 * i);
        return make_double2(r.x * r.x + m.x * m.x + r.y * r.y + m.y * m.y, 0.0);
    }
};
struct NormSq1 {
    const double *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double r = re[i], m = im[i];
        return make_double2(r * r + m * m, 0.0);
    }
};
struct DiagSum {          // sum of Re rho_rr
    const double* re;
    uint64_t step;        // D + 1
    __device__ __forceinline__ double2 operator()(uint64_t r) const { return make_double2(re[r * step], 0.0); }
};
struct ProbZeroVec {      // target >= 1: amps i with bit t = 0, two per item
    const double *re, *im;
    int t;
    __device__ __forceinline__ double2 operator()(uint64_t k) const {
        const uint64_t i = ins0(2 * k, t);
        const double2 r = ld2(re + i), m = ld2(im + i);
        return make_double2(r.x * r.x + m.x * m.x + r.y * r.y + m.y * m.y, 0.0);
    }
};
struct ProbZeroT0 {       // target 0: even amps
    const double *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t k) const {
        const double2 r = ld2(re + 2 * k), m = ld2(im + 2 * k);
        return make_double2(r.x * r.x + m.x * m.x, 0.0);
    }
};
struct ProbZeroDiag {     // diagonal entries rho_rr with bit t of r = 0
    const double* re;
    uint64_t step;
    int t;
    __device__ __forceinline__ double2 operator()(uint64_t k) const { return make_double2(re[ins0(k, t) * step], 0.0); }
};
struct Inner2 {           // sum conj(bra) ket, two amps per item
    const double *br, *bi, *kr, *ki;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double2 a = ld2(br + 2 * i), b = ld2(bi + 2 * i), c = ld2(kr + 2 * i), d = ld2(ki + 2 * i);
        return make_double2(a.x * c.x + b.x * d.x + a.y * c.y + b.y * d.y, a.x * d.x - b.x * c.x + a.y * d.y - b.y * c.y);
    }
};
struct Inner1 {
    const double *br, *bi, *kr, *ki;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        return make_double2(br[i] * kr[i] + bi[i] * ki[i], br[i] * ki[i] - bi[i] * kr[i]);
    }
};
struct DistSq {
    const double *ar, *ai, *br, *bi;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double dr = ar[i] - br[i], di = ai[i] - bi[i];
        return make_double2(dr * dr + di * di, 0.0);
    }
};
// <psi|rho|psi> = sum_{r,c} Re(conj(psi_r) rho_rc psi_c), one entry per item
struct FidelityDM {
    const double *rr, *ri, *pr, *pi;
    int N;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const uint64_t r = i & ((1ull << N) - 1ull), c = i >> N;
        const double er = rr[i], ei = ri[i];
        const double vr = __ldg(pr + c), vi = __ldg(pi + c);
        const double tr = er * vr - ei * vi, ti = er * vi + ei * vr;     // rho_rc psi_c
        const double ur = __ldg(pr + r), ui = -__ldg(pi + r);            // conj(psi_r)
        return make_double2(tr * ur - ti * ui, 0.0);
    }
};

constexpr int kMaxGroupTerms = 32;
struct PauliGroup {
    uint64_t xmask;
    int low;                     // lowest bit of xmask
    int numTerms;
    uint64_t yz[kMaxGroupTerms];
    int phase[kMaxGroupTerms];   // nY mod 4
    double coeff[kMaxGroupTerms];
};

// Re[(-i)^m w]
__device__ __forceinline__ double rePhase(int m, double wr, double wi) {
    switch (m & 3) {
        case 0: return wr;
        case 1: return wi;
        case 2: return -wr;
        default: return -wi;
    }
}

// SV, xmask != 0: pairs (j, k=j^x); contributes Re(conj(psi_j)(P psi)_j) +
// Re(conj(psi_k)(P psi)_k) for every term of the group
struct ExpecPairs {
    const double *re, *im;
    PauliGroup g;
    __device__ __forceinline__ double2 operator()(uint64_t t) const {
        const uint64_t j = ins0(t, g.low), k = j ^ g.xmask;
        const double jr = re[j], ji = im[j], kr = re[k], ki = im[k];
        const double wr = jr * kr + ji * ki, wi = jr * ki - ji * kr;       // conj(psi_j) psi_k
        double acc = 0.0;
        for (int q = 0; q < g.numTerms; ++q) {
            const double sj = (__popcll(j & g.yz[q]) & 1) ? -1.0 : 1.0;
            const double sk = (__popcll(k & g.yz[q]) & 1) ? -1.0 : 1.0;
            acc += g.coeff[q] * (sj * rePhase(g.phase[q], wr, wi) + sk * rePhase(g.phase[q], wr, -wi));
        }
        return make_double2(acc, 0.0);
    }
};
// SV, diagonal group: |psi_j|^2 sum_t c_t (-1)^popc(j & z_t)
struct ExpecDiag {
    const double *re, *im;
    PauliGroup g;
    __device__ __forceinline__ double2 operator()(uint64_t j) const {
        const double p = re[j] * re[j] + im[j] * im[j];
        double acc = 0.0;
        for (int q = 0; q < g.numTerms; ++q) acc += (__popcll(j & g.yz[q]) & 1) ? -g.coeff[q] : g.coeff[q];
        return make_double2(p * acc, 0.0);
    }
};
// DM: Tr(P rho) = sum_r (-i)^nY (-1)^popc(r & yz) rho[(r^x) + r D]  (real part)
struct ExpecDM {
    const double *re, *im;
    PauliGroup g;
    int N;
    __device__ __forceinline__ double2 operator()(uint64_t r) const {
        const uint64_t idx = (r ^ g.xmask) + (r << N);
        const double er = re[idx], ei = im[idx];
        double acc = 0.0;
        for (int q = 0; q < g.numTerms; ++q) {
            const double s = (__popcll(r & g.yz[q]) & 1) ? -1.0 : 1.0;
            acc += g.coeff[q] * s * rePhase(g.phase[q], er, ei);
        }
        return make_double2(acc, 0.0);
    }
};

// ---- calcProbOfAllOutcomes: shared-memory histogram, FP64 atomics --------
__global__ void kOutcomeHist(const double* __restrict__ re, const double* __restrict__ im, uint64_t nItems,
                             uint64_t step, int nq, const int* __restrict__ qs, double* __restrict__ out, int useShared) {
    extern __shared__ double hist[];
    const int nOut = 1 << nq;
    if (useShared) {
        for (int b = threadIdx.x; b < nOut; b += blockDim.x) hist[b] = 0.0;
        __syncthreads();
    }
    int q[32];
    for (int b = 0; b < nq; ++b) q[b] = qs[b];
    for (uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; it < nItems; it += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = it * step;                 // step = 1 (SV) or D + 1 (DM diagonal)
        const double p = step == 1 ? re[i] * re[i] + im[i] * im[i] : re[i];
        int o = 0;                                    // outcome bits of the amplitude (row) index
        for (int b = 0; b < nq; ++b) o |= (int)((it >> q[b]) & 1ull) << b;
        if (useShared) atomicAdd(hist + o, p);
        else atomicAdd(out + o, p);
    }
    if (useShared) {
        __syncthreads();
        for (int b = threadIdx.x; b < nOut; b += blockDim.x)
            if (hist[b] != 0.0) atomicAdd(out + b, hist[b]);
    }
}

}  // namespace

// ============================================================== public API
double reduceTotalProbSV(SV s, const Scratch& w) {                 // replaces QuEST_gpu.cu:1649-1679
    double v = 0;
    const uint64_t n = 1ull << s.n;
    if (n >= 2) runReduce(NormSq2{s.re, s.im}, n / 2, w, &v, nullptr, "calcTotalProb");
    else runReduce(NormSq1{s.re, s.im}, n, w, &v, nullptr, "calcTotalProb");
    return v;
}

double reduceNormSq(SV s, const Scratch& w) { return reduceTotalProbSV(s, w); }

double reduceTotalProbDM(SV s, int N, const Scratch& w) {          // replaces QuEST_gpu.cu:1626-1647
    double v = 0;
    runReduce(DiagSum{s.re, (1ull << N) + 1}, 1ull << N, w, &v, nullptr, "calcTotalProb");
    return v;
}

double reduceProbZeroSV(SV s, int t, const Scratch& w) {           // QuEST_gpu.cu:1992-2161
    double v = 0;
    const uint64_t half = 1ull << (s.n - 1);
    if (t >= 1 && half >= 2) runReduce(ProbZeroVec{s.re, s.im, t}, half / 2, w, &v, nullptr, "calcProbOfOutcome");
    else if (t == 0 && half >= 1 && s.n >= 1) runReduce(ProbZeroT0{s.re, s.im}, half, w, &v, nullptr, "calcProbOfOutcome");
    else runReduce(ProbZeroDiag{s.re, 1, t}, half, w, &v, nullptr, "calcProbOfOutcome");
    return v;
}

double reduceProbZeroDM(SV s, int t, int N, const Scratch& w) {    // QuEST_gpu.cu:1954-2104
    double v = 0;
    runReduce(ProbZeroDiag{s.re, (1ull << N) + 1, t}, 1ull << (N - 1), w, &v, nullptr, "calcProbOfOutcome");
    return v;
}

void reduceInnerProduct(SV bra, SV ket, const Scratch& w, double* outRe, double* outIm) {   // QuEST_gpu.cu:2368-2483
    const uint64_t n = 1ull << bra.n;
    if (n >= 2) runReduce(Inner2{bra.re, bra.im, ket.re, ket.im}, n / 2, w, outRe, outIm, "calcInnerProduct");
    else runReduce(Inner1{bra.re, bra.im, ket.re, ket.im}, n, w, outRe, outIm, "calcInnerProduct");
}

double reduceDotReal(SV a, SV b, const Scratch& w) {               // QuEST_gpu.cu:2297-2366
    double re = 0;
    reduceInnerProduct(a, b, w, &re, nullptr);
    return re;
}

double reduceDistSq(SV a, SV b, const Scratch& w) {
    double v = 0;
    runReduce(DistSq{a.re, a.im, b.re, b.im}, 1ull << a.n, w, &v, nullptr, "calcHilbertSchmidtDistance");
    return v;
}

double reduceFidelityDM(SV rho, SV psi, int N, const Scratch& w) { // replaces QuEST_gpu.cu:2486-2572
    double v = 0;
    runReduce(FidelityDM{rho.re, rho.im, psi.re, psi.im, N}, 1ull << rho.n, w, &v, nullptr, "calcFidelity");
    return v;
}

double reduceExpecPauliGroup(SV s, int isDM, int N, uint64_t xmask, const PauliTerm* terms, int numTerms, const Scratch& w) {
    double total = 0;
    for (int base = 0; base < numTerms; base += kMaxGroupTerms) {
        PauliGroup g{};
        g.xmask = xmask;
        g.low = xmask ? __builtin_ctzll(xmask) : 0;
        g.numTerms = std::min(kMaxGroupTerms, numTerms - base);
        for (int q = 0; q < g.numTerms; ++q) {
            g.yz[q] = terms[base + q].yz;
            g.phase[q] = terms[base + q].nY & 3;
            g.coeff[q] = terms[base + q].coeff;
        }
        double v = 0;
        if (isDM) runReduce(ExpecDM{s.re, s.im, g, N}, 1ull << N, w, &v, nullptr, "calcExpecPauliSum");
        else if (xmask) runReduce(ExpecPairs{s.re, s.im, g}, 1ull << (s.n - 1), w, &v, nullptr, "calcExpecPauliSum");
        else runReduce(ExpecDiag{s.re, s.im, g}, 1ull << s.n, w, &v, nullptr, "calcExpecPauliSum");
        total += v;
    }
    return total;
}

void reduceProbAllOutcomes(SV s, int isDM, int N, const int* qubits, int nq, double* hostOut, const Scratch& w) {
    (void)w;
    const int nOut = 1 << nq;
    const size_t bytes = (size_t)nOut * sizeof(double) + 32 * sizeof(int);
    static double* dOut = nullptr;
    static size_t cap = 0;
    if (bytes > cap) {
        if (dOut) cudaFree(dOut);
        dOut = nullptr;
        cap = 0;
        if (QG_CUDA(cudaMalloc(&dOut, bytes), "calcProbOfAllOutcomes")) return;
        cap = bytes;
    }
    cudaStream_t st = stream();
    int qs[32];
    for (int b = 0; b < nq; ++b) qs[b] = qubits[b];
    int* dQ = reinterpret_cast<int*>(dOut + nOut);
    if (QG_CUDA(cudaMemsetAsync(dOut, 0, (size_t)nOut * sizeof(double), st), "calcProbOfAllOutcomes")) return;
    if (QG_CUDA(cudaMemcpyAsync(dQ, qs, nq * sizeof(int), cudaMemcpyHostToDevice, st), "calcProbOfAllOutcomes")) return;
    const uint64_t nItems = isDM ? (1ull << N) : (1ull << s.n);
    const uint64_t step = isDM ? (1ull << N) + 1 : 1;
    const int useShared = nq <= 12;
    const size_t smem = useShared ? (size_t)nOut * sizeof(double) : 0;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((nItems + 255) / 256, (uint64_t)numSMs() * 4));
    kOutcomeHist<<<grid, 256, smem, st>>>(s.re, s.im, nItems, step, nq, dQ, dOut, useShared);
    if (launchFailed("calcProbOfAllOutcomes")) return;
    QG_CUDA(cudaMemcpyAsync(hostOut, dOut, (size_t)nOut * sizeof(double), cudaMemcpyDeviceToHost, st), "calcProbOfAllOutcomes");
    QG_CUDA(cudaStreamSynchronize(st), "calcProbOfAllOutcomes");
}

}  // namespace qg
