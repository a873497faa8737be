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

// ---- Pauli-string expectation values -----------------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, and a Pauli sum
// (C4's 80-term Fermi-Hubbard energy) has many terms per X/Y group, so the
// FP64 work per amplitude, not the read of the state, set the time of these
// reductions.  The per-term algebra is therefore done on the host:
//   * pairs (j, k = j ^ x): with w = conj(psi_j) psi_k and s_q(j) =
//     (-1)^popc(j & yz_q), term q adds c_q s_q(j) [Re((-i)^ph w) +
//     tau_q Re((-i)^ph conj w)], tau_q = (-1)^popc(x & yz_q); that is
//     2 c_q s_q(j) (+-Re w or +-Im w) when tau_q fits the phase, else 0.  An
//     item costs wr A(j) + wi B(j) with A, B = sums of +-c over the terms;
//   * DM, Tr(P rho) = sum_r s(r) Re((-i)^ph rho[r ^ x, r]) = er A(r) + ei B(r);
//   * a diagonal group (x = 0, SV): an item is 8 consecutive amplitudes.  A
//     Walsh-Hadamard transform of their |psi|^2 over the 3 low bits gives
//     Q[m] = sum_l p_l (-1)^popc(l & m); each term then adds
//     c (-1)^popc(base & z_high) Q[z & 7].  Terms are bucketed by z & 7 on the
//     host, so an amplitude costs ~6 FP64 operations plus terms / 8.
// Reference semantics: QuEST_common.c:506-533 (calcExpecPauliSum: clone,
// apply the Pauli string, inner product, per term).
constexpr int kMaxGroupTerms = 32;
struct PauliPairGroup {          // SV pairs (xmask != 0) or DM entries (any xmask)
    uint64_t xmask;
    int low;                     // lowest bit of xmask (SV)
    int nA, nB;                  // terms on Re w (er), on Im w (ei)
    uint64_t mA[kMaxGroupTerms], mB[kMaxGroupTerms];
    double cA[kMaxGroupTerms], cB[kMaxGroupTerms];
};
// sum_q c_q (-1)^popc(j & m_q) for n >= 1 terms (n - 1 FP64 additions)
__device__ __forceinline__ double signedSum(uint64_t j, const uint64_t* m, const double* c, int n) {
    double a = (__popcll(j & m[0]) & 1) ? -c[0] : c[0];
    for (int q = 1; q < n; ++q) a += (__popcll(j & m[q]) & 1) ? -c[q] : c[q];
    return a;
}

// x A(j) + y B(j) for a group with at least one term, skipping an empty list
// (the counts are uniform across the launch)
__device__ __forceinline__ double pairValue(uint64_t j, double x, double y, const PauliPairGroup& g) {
    if (g.nB == 0) return x * signedSum(j, g.mA, g.cA, g.nA);
    if (g.nA == 0) return y * signedSum(j, g.mB, g.cB, g.nB);
    return fma(x, signedSum(j, g.mA, g.cA, g.nA), y * signedSum(j, g.mB, g.cB, g.nB));
}
struct ExpecPairs {
    const double *re, *im;
    PauliPairGroup g;
    __device__ __forceinline__ double2 operator()(uint64_t t) const {
        const uint64_t j = ins0(t, g.low), k = j ^ g.xmask;
        const double jr = re[j], ji = im[j], kr = re[k], ki = im[k];
        // conj(psi_j) psi_k, only the parts the group's terms use
        const double wr = g.nA ? fma(jr, kr, ji * ki) : 0.0;
        const double wi = g.nB ? fma(jr, ki, -(ji * kr)) : 0.0;
        return make_double2(pairValue(j, wr, wi, g), 0.0);
    }
};
struct ExpecDM {
    const double *re, *im;
    PauliPairGroup g;
    int N;
    __device__ __forceinline__ double2 operator()(uint64_t r) const {
        const uint64_t idx = (r ^ g.xmask) + (r << N);
        return make_double2(pairValue(r, re[idx], im[idx], g), 0.0);
    }
};
constexpr int kDiagLow = 3;                      // low bits transformed per item
constexpr int kDiagItem = 1 << kDiagLow;
constexpr int kMaxDiagTerms = 64;
struct PauliDiagGroup {
    int off[kDiagItem + 1];                      // terms of bucket m (z & 7 = m): [off[m], off[m + 1])
    uint64_t zh[kMaxDiagTerms];                  // z with the low bits cleared
    double c[kMaxDiagTerms];
};
struct ExpecDiag {                               // SV, x = 0: 8 amplitudes per item (n >= 3)
    const double *re, *im;
    PauliDiagGroup g;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const uint64_t base = i << kDiagLow;
        double p[kDiagItem];
#pragma unroll
        for (int h = 0; h < kDiagItem / 2; ++h) {
            const double2 r = ld2(re + base + 2 * h), m = ld2(im + base + 2 * h);
            p[2 * h] = r.x * r.x + m.x * m.x;
            p[2 * h + 1] = r.y * r.y + m.y * m.y;
        }
#pragma unroll
        for (int sb = 1; sb < kDiagItem; sb <<= 1)
#pragma unroll
            for (int l = 0; l < kDiagItem; ++l)
                if (!(l & sb)) {
                    const double a = p[l], b = p[l | sb];
                    p[l] = a + b;
                    p[l | sb] = a - b;
                }
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m < kDiagItem; ++m) {
            double gm = 0.0;
            for (int t = g.off[m]; t < g.off[m + 1]; ++t) gm += (__popcll(base & g.zh[t]) & 1) ? -g.c[t] : g.c[t];
            acc = fma(gm, p[m], acc);
        }
        return make_double2(acc, 0.0);
    }
};
struct ExpecDiag1 {                              // SV, x = 0, one amplitude per item (n < 3)
    const double *re, *im;
    PauliPairGroup g;
    __device__ __forceinline__ double2 operator()(uint64_t j) const {
        return make_double2(pairValue(j, re[j] * re[j] + im[j] * im[j], 0.0, g), 0.0);
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

void pauliPairTerms(uint64_t x, const std::vector<PauliTerm>& terms, std::vector<std::pair<uint64_t, double>>& A,
                    std::vector<std::pair<uint64_t, double>>& B) {
    for (const PauliTerm& t : terms) {
        const int ph = t.nY & 3;
        const bool tauPlus = (__builtin_popcountll(x & t.yz) & 1) == 0;
        if (ph % 2 == 0 && tauPlus) A.push_back({t.yz, ph == 0 ? 2 * t.coeff : -2 * t.coeff});
        if (ph % 2 == 1 && !tauPlus) B.push_back({t.yz, ph == 1 ? 2 * t.coeff : -2 * t.coeff});
    }
}

double reduceExpecPauliGroups(SV s, int isDM, int N, const std::vector<PauliTermGroup>& groups, const Scratch& w) {
    // Every group (or chunk of a large group) reduces into its own result
    // slot; the slots are read back once per 32 launches, and summed on the
    // host in group order.
    constexpr int kSlots = 32;                   // the scratch holds 64 result doubles
    const char* caller = "calcExpecPauliSum";
    cudaStream_t st = stream();
    double total = 0.0;
    int used = 0;
    auto drain = [&]() -> bool {
        if (!used) return true;
        if (QG_CUDA(cudaMemcpyAsync(w.host, w.result, 2 * used * sizeof(double), cudaMemcpyDeviceToHost, st), caller) ||
            QG_CUDA(cudaStreamSynchronize(st), caller))
            return false;
        for (int k = 0; k < used; ++k) total += w.host[2 * k];
        used = 0;
        return true;
    };
    auto queue = [&](auto f, uint64_t nItems) -> bool {
        if (used == kSlots && !drain()) return false;
        const int grid = reduceGrid(nItems);
        kReduce<<<grid, red::kThreads, 0, st>>>(f, nItems, w.partials, w.counter, w.result + 2 * used);
        if (launchFailed(caller)) return false;
        ++used;
        return true;
    };
    for (const PauliTermGroup& grp : groups) {
        const uint64_t x = grp.xmask;
        const int nt = (int)grp.terms.size();
        if (!isDM && x == 0 && s.n >= kDiagLow) {
            // diagonal group: terms bucketed by their low bits
            for (int b0 = 0; b0 < nt; b0 += kMaxDiagTerms) {
                const int cnt = std::min(kMaxDiagTerms, nt - b0);
                PauliDiagGroup g{};
                int k = 0;
                for (int m = 0; m < kDiagItem; ++m) {
                    g.off[m] = k;
                    for (int t = b0; t < b0 + cnt; ++t)
                        if ((int)(grp.terms[t].yz & (kDiagItem - 1)) == m) {
                            g.zh[k] = grp.terms[t].yz & ~(uint64_t)(kDiagItem - 1);
                            g.c[k++] = grp.terms[t].coeff;    // x = 0: no Y, phase 0
                        }
                }
                g.off[kDiagItem] = k;
                if (!queue(ExpecDiag{s.re, s.im, g}, 1ull << (s.n - kDiagLow))) return total;
            }
            continue;
        }
        // pairs / DM entries: each term goes to the Re (A) or Im (B) list
        std::vector<std::pair<uint64_t, double>> A, B;
        if (isDM) {
            for (const PauliTerm& t : grp.terms) {
                const int ph = t.nY & 3;
                (ph % 2 == 0 ? A : B).push_back({t.yz, ph < 2 ? t.coeff : -t.coeff});
            }
        } else if (x == 0) {                     // n < 3 diagonal group: |psi_j|^2 terms
            for (const PauliTerm& t : grp.terms) A.push_back({t.yz, t.coeff});
        } else {
            pauliPairTerms(x, grp.terms, A, B);
        }
        for (size_t a0 = 0, b0 = 0; a0 < A.size() || b0 < B.size();) {
            PauliPairGroup g{};
            g.xmask = x;
            g.low = x ? __builtin_ctzll(x) : 0;
            for (; a0 < A.size() && g.nA < kMaxGroupTerms; ++a0, ++g.nA) {
                g.mA[g.nA] = A[a0].first;
                g.cA[g.nA] = A[a0].second;
            }
            for (; b0 < B.size() && g.nB < kMaxGroupTerms; ++b0, ++g.nB) {
                g.mB[g.nB] = B[b0].first;
                g.cB[g.nB] = B[b0].second;
            }
            bool ok;
            if (isDM) ok = queue(ExpecDM{s.re, s.im, g, N}, 1ull << N);
            else if (x) ok = queue(ExpecPairs{s.re, s.im, g}, 1ull << (s.n - 1));
            else ok = queue(ExpecDiag1{s.re, s.im, g}, 1ull << s.n);
            if (!ok) return total;
        }
    }
    drain();
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
