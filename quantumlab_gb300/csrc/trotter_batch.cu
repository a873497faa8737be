// trotter_batch.cu -- batched Trotter evolution of many Hamiltonian instances
// (sm_103a).
//
// QuantumLab's Fermi-Hubbard studies run one Trotter circuit per Hamiltonian
// instance (QuEST.c:1079 applyTrotterCircuit -> QuEST_common.c:762-844 per
// instance, then calcExpecPauliSum, QuEST_common.c:506-533).  A batch holds B
// instances as FP32 states and runs them together.  An instance is a Trotter
// circuit or an explicit circuit (the gates of a fusion plan, e.g. one
// circuit shape with other parameters per instance), each with the Pauli sum
// whose expectation the run reports.  Instances that share the
// register size, Pauli strings, order and repetitions form a class: their
// circuits have the same shape with other angles.  Instances of different
// step counts, orders, register sizes or Hamiltonians sit in one batch as
// different classes:
//   * per class, the fusion planner compiles one member's gate stream; every
//     other member takes the same passes with its own FP64 products
//     (compilePlanLike), so the planner runs once per class;
//   * each pass is one launch of the tensor-core applier over all the class's
//     states (the CTAs are shared out among the states, each state's CTAs
//     load that state's operands); passes narrower than 4 qubits are widened
//     with identity factors so that every pass runs on the tensor cores;
//   * the energies <H_b> are reduced from the FP32 states (FP32 products per
//     amplitude pair, FP64 sums), one launch per term group over the class's
//     states, divided by each state's norm, which also removes the norm drift
//     of the FP32 passes to first order;
//   * after the first run the whole sequence (every class's initial states,
//     passes and reductions, and the copy of the results to pinned host
//     memory) is one CUDA graph that later runs replay.
#include "fused_plan.h"
#include "qg_internal.h"
#include "quest_gb300.h"
#include "reduce_kernel.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <tuple>
#include <vector>

namespace qg {

size_t tcImageFloats(int k, int parts);
void tcBuildImage(const FusedPass& pass, float* img, int parts);
int tcImageParts();
bool applyPassTCBatch(float* re, float* im, int n, const FusedPass& pass, const float* images, size_t imageStride,
                      int parts, int batch, int* errFlag, cudaStream_t st);

namespace {

using red::ins0;

constexpr int kMaxTerms = 32;
constexpr int kCoefs = 64;           // coefficients per instance per reduction
// The reductions of a batch share their Pauli masks; only the coefficients
// differ per instance (coef[b * kCoefs ...], in device memory).
struct PairShape {                   // X/Y mask x != 0: pairs (j, j ^ x)
    uint64_t xmask;
    int low, nA, nB;
    uint64_t mA[kMaxTerms], mB[kMaxTerms];
};
__device__ __forceinline__ float signedSumF(uint64_t j, const uint64_t* m, const float* c, int n) {
    float a = 0.f;
    for (int q = 0; q < n; ++q) a += (__popcll(j & m[q]) & 1) ? -c[q] : c[q];
    return a;
}
// Re(conj(psi_j) psi_k) A(j) + Im(conj(psi_j) psi_k) B(j), in FP32, for
// instance b (A's coefficients at coef[b * kCoefs], B's kMaxTerms later)
struct PairsF32 {
    const float *re, *im;
    uint64_t dim;
    PairShape g;
    const float* coef;
    __device__ __forceinline__ double operator()(int b, uint64_t t) const {
        const float* r = re + (uint64_t)b * dim;
        const float* m = im + (uint64_t)b * dim;
        const float* cA = coef + b * kCoefs;
        const uint64_t j = ins0(t, g.low), k = j ^ g.xmask;
        const float jr = r[j], ji = m[j], kr = r[k], ki = m[k];
        const float wr = fmaf(jr, kr, ji * ki), wi = fmaf(jr, ki, -(ji * kr));
        return (double)(wr * signedSumF(j, g.mA, cA, g.nA) + wi * signedSumF(j, g.mB, cA + kMaxTerms, g.nB));
    }
};
// The same for four consecutive pairs per item (x has no bit below 2, so the
// four j and the four k are contiguous): four 16-byte loads per item instead
// of sixteen 4-byte ones, one FP64 addition per four pairs.  The scalar form
// was bound by load latency and FP64 work (one conversion and addition per
// pair, GB300's FP64 pipe 55 % busy).
struct PairsF32x4 {
    const float *re, *im;
    uint64_t dim;
    PairShape g;
    const float* coef;
    __device__ __forceinline__ double operator()(int b, uint64_t i) const {
        const float* r = re + (uint64_t)b * dim;
        const float* m = im + (uint64_t)b * dim;
        const float* cA = coef + b * kCoefs;
        const uint64_t j = ins0(4 * i, g.low), k = j ^ g.xmask;
        const float4 jr = *reinterpret_cast<const float4*>(r + j), ji = *reinterpret_cast<const float4*>(m + j);
        const float4 kr = *reinterpret_cast<const float4*>(r + k), ki = *reinterpret_cast<const float4*>(m + k);
        const float ar[4] = {jr.x, jr.y, jr.z, jr.w}, ai[4] = {ji.x, ji.y, ji.z, ji.w};
        const float br[4] = {kr.x, kr.y, kr.z, kr.w}, bi[4] = {ki.x, ki.y, ki.z, ki.w};
        float acc = 0.f;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float wr = fmaf(ar[e], br[e], ai[e] * bi[e]), wi = fmaf(ar[e], bi[e], -(ai[e] * br[e]));
            acc += wr * signedSumF(j + e, g.mA, cA, g.nA) + wi * signedSumF(j + e, g.mB, cA + kMaxTerms, g.nB);
        }
        return (double)acc;
    }
};
constexpr int kDiagItem = 16;
struct DiagShape {                   // x = 0: terms bucketed by their 4 low mask bits
    int off[kDiagItem + 1];
    uint64_t zh[kCoefs];
};
// sum over 16 amplitudes of |psi|^2 sum_t c_t (-1)^popc(j & z_t), through the
// Walsh-Hadamard transform of the 16 probabilities (as in reduce.cu, which
// takes 8), in FP32: a term then costs one signed addition per 16 amplitudes
struct DiagF32 {
    const float *re, *im;
    uint64_t dim;
    DiagShape g;
    const float* coef;
    __device__ __forceinline__ double operator()(int b, uint64_t i) const {
        const uint64_t base = i * kDiagItem;
        const float* r = re + (uint64_t)b * dim + base;
        const float* m = im + (uint64_t)b * dim + base;
        const float* c = coef + b * kCoefs;
        float p[kDiagItem];
#pragma unroll
        for (int h = 0; h < kDiagItem / 4; ++h) {
            const float4 a = *reinterpret_cast<const float4*>(r + 4 * h), q = *reinterpret_cast<const float4*>(m + 4 * h);
            p[4 * h] = fmaf(a.x, a.x, q.x * q.x);
            p[4 * h + 1] = fmaf(a.y, a.y, q.y * q.y);
            p[4 * h + 2] = fmaf(a.z, a.z, q.z * q.z);
            p[4 * h + 3] = fmaf(a.w, a.w, q.w * q.w);
        }
#pragma unroll
        for (int sb = 1; sb < kDiagItem; sb <<= 1)
#pragma unroll
            for (int l = 0; l < kDiagItem; ++l)
                if (!(l & sb)) {
                    const float a = p[l], bb = p[l | sb];
                    p[l] = a + bb;
                    p[l | sb] = a - bb;
                }
        float acc = 0.f;
#pragma unroll
        for (int mm = 0; mm < kDiagItem; ++mm) {
            float gm = 0.f;
            for (int t = g.off[mm]; t < g.off[mm + 1]; ++t) gm += (__popcll(base & g.zh[t]) & 1) ? -c[t] : c[t];
            acc = fmaf(gm, p[mm], acc);
        }
        return (double)acc;
    }
};
struct NormF32b {                    // 8 amplitudes per item
    const float *re, *im;
    uint64_t dim;
    __device__ __forceinline__ double operator()(int b, uint64_t i) const {
        const float4* r4 = reinterpret_cast<const float4*>(re + (uint64_t)b * dim + 8 * i);
        const float4* m4 = reinterpret_cast<const float4*>(im + (uint64_t)b * dim + 8 * i);
        const float4 a = r4[0], bb = r4[1], c = m4[0], d = m4[1];
        float s = a.x * a.x;
        s = fmaf(a.y, a.y, s); s = fmaf(a.z, a.z, s); s = fmaf(a.w, a.w, s);
        s = fmaf(bb.x, bb.x, s); s = fmaf(bb.y, bb.y, s); s = fmaf(bb.z, bb.z, s); s = fmaf(bb.w, bb.w, s);
        s = fmaf(c.x, c.x, s); s = fmaf(c.y, c.y, s); s = fmaf(c.z, c.z, s); s = fmaf(c.w, c.w, s);
        s = fmaf(d.x, d.x, s); s = fmaf(d.y, d.y, s); s = fmaf(d.z, d.z, s); s = fmaf(d.w, d.w, s);
        return (double)s;
    }
};

// One reduction for every instance of the batch: block (x, b) sums items of
// instance b; the last block of instance b (its ticket in counters[b]) adds
// the instance's block partials in a fixed order into results[2 b].
constexpr int kMaxBlocksPerInst = 2048;
template <class F>
__global__ void __launch_bounds__(red::kThreads) kReduceBatch(F f, uint64_t nItems, double* __restrict__ partials,
                                                              unsigned int* __restrict__ counters,
                                                              double* __restrict__ results) {
    __shared__ double sx[red::kWarps];
    __shared__ bool amLast;
    const int b = blockIdx.y;
    const uint64_t stride = (uint64_t)gridDim.x * red::kThreads;
    uint64_t i = (uint64_t)blockIdx.x * red::kThreads + threadIdx.x;
    double a0 = 0.0, a1 = 0.0;
    for (; i + stride < nItems; i += 2 * stride) {
        a0 += f(b, i);
        a1 += f(b, i + stride);
    }
    for (; i < nItems; i += stride) a0 += f(b, i);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double x = red::warpSum(a0 + a1);
    if (lane == 0) sx[w] = x;
    __syncthreads();
    double* part = partials + (size_t)b * kMaxBlocksPerInst;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < red::kWarps; ++k) t += sx[k];
        part[blockIdx.x] = t;
        __threadfence();
        amLast = atomicAdd(counters + b, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    double v = 0.0;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += red::kThreads) v += __ldcg(part + k);
    v = red::warpSum(v);
    if (lane == 0) sx[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < red::kWarps; ++k) t += sx[k];
        results[2 * b] = t;
        results[2 * b + 1] = 0.0;
        counters[b] = 0u;
    }
}

__global__ void kBatchClassical(float* re, uint64_t stride, const long long* idx, int B) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B) re[(uint64_t)b * stride + (uint64_t)idx[b]] = 1.f;
}
__global__ void kBatchToF64(const float* __restrict__ sr, const float* __restrict__ si, double* __restrict__ dr,
                            double* __restrict__ di, uint64_t n, double scale) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        dr[i] = (double)sr[i] * scale;
        di[i] = (double)si[i] * scale;
    }
}

struct Instance {
    bool circuit = false;            // an explicit gate list instead of a Trotter circuit
    std::vector<FusedGate> gates;    // (circuit) its gates, in order
    int n = 0;                       // qubits
    std::vector<int> codes;          // numTerms x n, QuEST pauliOpType values
    std::vector<double> coeffs;
    double time = 0.0;
    int order = 1, reps = 1;
    long long init = 0;
    bool set = false;
};

// The gates QuEST's applyTrotterCircuit applies (QuEST_common.c:762-844):
// per repetition the symmetrised product of order `order`, each term as
// exp(-i fac c P) = multiRotatePauli(angle 2 fac c); identity terms apply
// nothing.
void trotterTerms(const Instance& in, int n, double time, int order, std::vector<FusedGate>& out) {
    if (order == 1 || order == 2) {
        const int T = (int)in.coeffs.size();
        const double fac = order == 1 ? time : time / 2;
        for (int pass = 0; pass < order; ++pass)
            for (int i = 0; i < T; ++i) {
                const int t = pass == 0 ? i : T - 1 - i;
                uint64_t x = 0, y = 0, z = 0;
                for (int q = 0; q < n; ++q) {
                    const int c = in.codes[(size_t)t * n + q];
                    if (c == PAULI_X) x |= 1ull << q;
                    if (c == PAULI_Y) { x |= 1ull << q; y |= 1ull << q; }
                    if (c == PAULI_Z) z |= 1ull << q;
                }
                if ((x | z) == 0) continue;
                out.push_back(pauliRotationGate(x, y, z, 2 * fac * in.coeffs[t]));
            }
        return;
    }
    const double p = 1. / (4 - std::pow(4, 1. / (order - 1)));
    const int lo = order - 2;
    trotterTerms(in, n, p * time, lo, out);
    trotterTerms(in, n, p * time, lo, out);
    trotterTerms(in, n, (1 - 4 * p) * time, lo, out);
    trotterTerms(in, n, p * time, lo, out);
    trotterTerms(in, n, p * time, lo, out);
}

// Widen a pass of k < 4 qubits with identity factors on the lowest other
// qubits (the tensor-core applier takes 4..6): to 6 qubits where the
// register allows (n >= 13), whose pipelined kernel runs a batch pass faster
// than the 4-qubit one (measured on configuration 4: 0.41 against 0.50 ms
// per launch over a class), else to 4.
FusedPass widenNarrow(const FusedPass& p, int n) {
    const int k = (int)p.targets.size();
    if (k >= 4) return p;
    const int kw = n >= 13 ? 6 : 4;
    std::vector<int> t = p.targets;
    for (int q = 0; q < n && (int)t.size() < kw; ++q)
        if (std::find(t.begin(), t.end(), q) == t.end()) t.push_back(q);
    std::sort(t.begin(), t.end());
    std::vector<int> pos(k);                       // new matrix bit of old bit b
    for (int b = 0; b < k; ++b) pos[b] = (int)(std::find(t.begin(), t.end(), p.targets[b]) - t.begin());
    const int D = 1 << k, W = 1 << kw;
    FusedPass w;
    w.targets = t;
    w.numGates = p.numGates;
    w.unitary = p.unitary;
    w.m.assign((size_t)W * W, cplx(0, 0));
    uint64_t oldMask = 0;
    for (int b = 0; b < k; ++b) oldMask |= 1ull << pos[b];
    auto gather = [&](int i) {                     // old index of the new index's target bits
        int r = 0;
        for (int b = 0; b < k; ++b)
            if (i >> pos[b] & 1) r |= 1 << b;
        return r;
    };
    for (int r = 0; r < W; ++r)
        for (int c = 0; c < W; ++c)
            if ((r & ~oldMask) == (c & ~oldMask)) w.m[(size_t)r * W + c] = p.m[(size_t)gather(r) * D + gather(c)];
    return w;
}

// The energy reductions of one class: one launch each over the class's
// instances (blockIdx.y = instance).
struct Red {
    int kind;                                      // 0 pairs, 3 pairs by four, 1 diagonal, 2 norm
    PairShape ps;
    DiagShape ds;
};

// Instances that share register size, Pauli strings, order and repetitions:
// one fusion plan, one launch per pass over all of them.
struct TrotterClass {
    int n = 0;
    std::vector<int> members;                      // instance indices, in batch order
    size_t stateOffset = 0;                        // floats into re / im of member 0's planes
    int posBase = 0;                               // first row of partials / counters / dInit
    int slotBase = 0;                              // first result slot
    size_t coefOffset = 0;                         // floats into dCoef
    std::vector<FusedPass> shape;                  // per pass: the targets (member 0's pass)
    std::vector<size_t> imgOffset, imgStride;      // per pass, in floats into images
    std::vector<Red> reds;
    // energy of member m = sum of its group slots / its norm slot + identity
    std::vector<std::vector<int>> groupSlots;
    std::vector<int> normSlot;
    std::vector<double> identity;
};

}  // namespace

struct TrotterBatch {
    int maxQubits = 0, B = 0;
    std::vector<Instance> inst;
    bool compiled = false;
    int parts = 0;                                 // operand image parts built (tcImageParts)
    std::vector<TrotterClass> classes;
    std::vector<int> classOf, posOf;               // per instance: its class, its place in it
    float *re = nullptr, *im = nullptr;            // every class's states, class after class
    float* images = nullptr;
    long long* dInit = nullptr;
    int* errFlag = nullptr;
    double* partials = nullptr;                    // per instance kMaxBlocksPerInst block partials
    unsigned int* counters = nullptr;              // per instance last-block tickets
    double* dResults = nullptr;                    // per class: slot slotBase + l * size + m
    double* hResults = nullptr;                    // pinned
    float* dCoef = nullptr;                        // per class, reduction l, member m: kCoefs floats
    int numSlots = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long runs = 0;
};

namespace {

void freeDevice(TrotterBatch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    for (void* p : {(void*)b->re, (void*)b->im, (void*)b->images, (void*)b->dInit, (void*)b->dCoef, (void*)b->dResults})
        if (p) cudaFree(p);
    if (b->hResults) cudaFreeHost(b->hResults);
    b->re = b->im = nullptr;
    b->images = nullptr;
    b->dInit = nullptr;
    b->dCoef = nullptr;
    b->dResults = nullptr;
    b->hResults = nullptr;
    b->classes.clear();
    b->compiled = false;
    b->runs = 0;
}

const char* kFn = "quest_gb300_trotterBatchRun";

// The energy reductions of class c (Pauli strings grouped by X/Y mask, one
// read of a state per group, plus the norm), with the coefficients of every
// member appended to coef ([reduction][member][kCoefs]).
void buildReductions(const TrotterBatch* b, TrotterClass& c, std::vector<float>& coef) {
    const int n = c.n, M = (int)c.members.size();
    const Instance& i0 = b->inst[c.members[0]];
    std::map<uint64_t, std::vector<int>> groups;   // x -> term indices
    std::vector<uint64_t> yzOf(i0.coeffs.size());
    std::vector<int> nYOf(i0.coeffs.size());
    std::vector<int> identityTerms;
    for (size_t t = 0; t < i0.coeffs.size(); ++t) {
        uint64_t x = 0, y = 0, z = 0;
        for (int q = 0; q < n; ++q) {
            const int cd = i0.codes[t * n + q];
            if (cd == PAULI_X) x |= 1ull << q;
            if (cd == PAULI_Y) { x |= 1ull << q; y |= 1ull << q; }
            if (cd == PAULI_Z) z |= 1ull << q;
        }
        yzOf[t] = y | z;
        nYOf[t] = __builtin_popcountll(y);
        if ((x | z) == 0) identityTerms.push_back((int)t);
        else groups[x].push_back((int)t);
    }
    c.reds.clear();
    c.identity.assign(M, 0.0);
    for (int m = 0; m < M; ++m)
        for (int t : identityTerms) c.identity[m] += b->inst[c.members[m]].coeffs[t];
    auto addRed = [&](const Red& r, const std::vector<std::vector<float>>& perMember) {
        c.reds.push_back(r);
        for (int m = 0; m < M; ++m) {
            std::vector<float> v(kCoefs, 0.f);
            if (!perMember.empty()) std::copy(perMember[m].begin(), perMember[m].end(), v.begin());
            coef.insert(coef.end(), v.begin(), v.end());
        }
    };
    for (auto& g : groups) {
        const uint64_t x = g.first;
        if (x == 0) {
            // diagonal terms, bucketed by their low mask bits
            for (size_t c0 = 0; c0 < g.second.size(); c0 += kCoefs) {
                Red r{};
                r.kind = 1;
                std::vector<int> order;
                const size_t c1 = std::min(g.second.size(), c0 + kCoefs);
                for (int bk = 0; bk < kDiagItem; ++bk) {
                    r.ds.off[bk] = (int)order.size();
                    for (size_t u = c0; u < c1; ++u) {
                        const int t = g.second[u];
                        if ((int)(yzOf[t] & (kDiagItem - 1)) == bk) {
                            r.ds.zh[order.size()] = yzOf[t] & ~(uint64_t)(kDiagItem - 1);
                            order.push_back(t);
                        }
                    }
                }
                r.ds.off[kDiagItem] = (int)order.size();
                std::vector<std::vector<float>> per(M);
                for (int m = 0; m < M; ++m)
                    for (int t : order) per[m].push_back((float)b->inst[c.members[m]].coeffs[t]);
                addRed(r, per);
            }
            continue;
        }
        // the A / B lists depend on the masks only, so they line up across
        // the members
        std::vector<std::vector<std::pair<uint64_t, double>>> A(M), Bl(M);
        for (int m = 0; m < M; ++m) {
            std::vector<PauliTerm> terms;
            for (int t : g.second) terms.push_back(PauliTerm{yzOf[t], nYOf[t], b->inst[c.members[m]].coeffs[t]});
            pauliPairTerms(x, terms, A[m], Bl[m]);
        }
        for (size_t a0 = 0, b0 = 0; a0 < A[0].size() || b0 < Bl[0].size();) {
            Red r{};
            r.kind = (x & 3) ? 0 : 3;                  // 3: four contiguous pairs per item
            r.ps.xmask = x;
            r.ps.low = __builtin_ctzll(x);
            const size_t a1 = std::min(A[0].size(), a0 + kMaxTerms), b1 = std::min(Bl[0].size(), b0 + kMaxTerms);
            r.ps.nA = (int)(a1 - a0);
            r.ps.nB = (int)(b1 - b0);
            for (size_t u = a0; u < a1; ++u) r.ps.mA[u - a0] = A[0][u].first;
            for (size_t u = b0; u < b1; ++u) r.ps.mB[u - b0] = Bl[0][u].first;
            std::vector<std::vector<float>> per(M, std::vector<float>(kCoefs, 0.f));
            for (int m = 0; m < M; ++m) {
                for (size_t u = a0; u < a1; ++u) per[m][u - a0] = (float)A[m][u].second;
                for (size_t u = b0; u < b1; ++u) per[m][kMaxTerms + u - b0] = (float)Bl[m][u].second;
            }
            addRed(r, per);
            a0 = a1;
            b0 = b1;
        }
    }
    const int groupReds = (int)c.reds.size();
    Red norm{};
    norm.kind = 2;
    addRed(norm, {});
    c.groupSlots.assign(M, {});
    c.normSlot.assign(M, 0);
    for (int m = 0; m < M; ++m) {
        for (int l = 0; l < groupReds; ++l) c.groupSlots[m].push_back(c.slotBase + l * M + m);
        c.normSlot[m] = c.slotBase + groupReds * M + m;
    }
}

// Run fn(j) for j in [0, jobs) on up to `threads` host threads.
template <class F>
void parallelFor(size_t jobs, unsigned threads, F fn) {
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t j; (j = next.fetch_add(1)) < jobs;) fn(j);
    };
    const unsigned nt = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, jobs));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) {
        try {
            pool.emplace_back(work);
        } catch (...) {                     // fewer threads: the work items are shared
            break;
        }
    }
    work();
    for (auto& t : pool) t.join();
}

bool compileBatch(TrotterBatch* b) {
    const int B = b->B;
    for (int k = 0; k < B; ++k)
        if (!b->inst[k].set) {
            invalidQuESTInputError("Every instance of the Trotter batch must be set before it runs.", kFn);
            return false;
        }
    // classes: instances of one register size, measured Pauli strings and
    // circuit shape (Trotter order and repetitions, or the qubits of every
    // gate of an explicit circuit), in order of first appearance
    auto sameShape = [](const Instance& r, const Instance& in) {
        if (r.n != in.n || r.circuit != in.circuit || r.codes != in.codes) return false;
        if (!in.circuit) return r.order == in.order && r.reps == in.reps;
        if (r.gates.size() != in.gates.size()) return false;
        for (size_t g = 0; g < r.gates.size(); ++g)
            if (r.gates[g].qubits != in.gates[g].qubits) return false;
        return true;
    };
    b->classes.clear();
    std::vector<int> leaderOf(B, -1);
    for (int k = 0; k < B; ++k) {
        const Instance& in = b->inst[k];
        int c = 0;
        for (; c < (int)b->classes.size(); ++c)
            if (sameShape(b->inst[b->classes[c].members[0]], in)) break;
        if (c == (int)b->classes.size()) {
            b->classes.emplace_back();
            b->classes.back().n = in.n;
        }
        b->classes[c].members.push_back(k);
        leaderOf[k] = b->classes[c].members[0];
    }
    // gate streams; every class's first member is searched (classes in
    // parallel), the others reuse its passes with their own FP64 products.
    // Passes are at most min(6, n - 7) qubits wide, the tensor-core limit.
    std::vector<FusedPlan> plan(B);
    for (int k = 0; k < B; ++k) {
        const Instance& in = b->inst[k];
        FusedPlan& p = plan[k];
        p.numQubits = in.n;
        p.maxFused = std::min(widestPass(in.n), in.n - 7);
        if (in.circuit) p.gates = in.gates;
        else
            for (int r = 0; r < in.reps; ++r) trotterTerms(in, in.n, in.time / in.reps, in.order, p.gates);
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    std::vector<int> leaders, others;
    for (const TrotterClass& cl : b->classes) {
        leaders.push_back(cl.members[0]);
        for (size_t m = 1; m < cl.members.size(); ++m) others.push_back(cl.members[m]);
    }
    parallelFor(leaders.size(), std::min(hw, 8u), [&](size_t i) { compilePlan(plan[leaders[i]]); });
    for (int l : leaders)
        if (!plan[l].compiled) {
            invalidQuESTInputError("A circuit of the batch could not be fused.", kFn);
            return false;
        }
    std::vector<char> like(B, 1);
    parallelFor(others.size(), std::min(hw, 8u),
                [&](size_t i) { like[others[i]] = compilePlanLike(plan[others[i]], plan[leaderOf[others[i]]]) ? 1 : 0; });
    // a member whose gates cannot take its class's passes (an explicit
    // circuit with a gate less diagonal than the leader's) gets a class and a
    // search of its own
    std::vector<int> alone;
    for (int o : others)
        if (!like[o]) alone.push_back(o);
    parallelFor(alone.size(), std::min(hw, 8u), [&](size_t i) { compilePlan(plan[alone[i]]); });
    for (int o : alone)
        if (!plan[o].compiled) {
            invalidQuESTInputError("A circuit of the batch could not be fused.", kFn);
            return false;
        }
    if (!alone.empty()) {
        for (TrotterClass& cl : b->classes) {
            std::vector<int> keep;
            for (int k : cl.members)
                if (like[k]) keep.push_back(k);
            cl.members.swap(keep);
        }
        for (int o : alone) {
            b->classes.emplace_back();
            b->classes.back().n = b->inst[o].n;
            b->classes.back().members.push_back(o);
        }
    }
    b->classOf.assign(B, -1);
    b->posOf.assign(B, -1);
    for (int c = 0; c < (int)b->classes.size(); ++c)
        for (size_t m = 0; m < b->classes[c].members.size(); ++m) {
            b->classOf[b->classes[c].members[m]] = c;
            b->posOf[b->classes[c].members[m]] = (int)m;
        }
    const int C = (int)b->classes.size();
    auto planOf = [&](int c, size_t m) -> FusedPlan& { return plan[b->classes[c].members[m]]; };
    // layout: states, image offsets, result slots and rows, class after class
    size_t stateFloats = 0, imgTotal = 0;
    // the operand image parts the current precision and kernel choice read
    b->parts = tcImageParts();
    int pos = 0, slots = 0;
    std::vector<float> coef;                       // [class][reduction][member][kCoefs]
    for (int c = 0; c < C; ++c) {
        TrotterClass& cl = b->classes[c];
        const size_t M = cl.members.size();
        cl.stateOffset = stateFloats;
        stateFloats += ((size_t)1 << cl.n) * M;
        cl.posBase = pos;
        pos += (int)M;
        const size_t np = planOf(c, 0).passes.size();
        cl.shape.clear();
        cl.imgOffset.assign(np, 0);
        cl.imgStride.assign(np, 0);
        for (size_t p = 0; p < np; ++p) {
            cl.shape.push_back(widenNarrow(planOf(c, 0).passes[p], cl.n));
            cl.imgStride[p] = tcImageFloats((int)cl.shape[p].targets.size(), b->parts);
            cl.imgOffset[p] = imgTotal;
            imgTotal += cl.imgStride[p] * M;
        }
        cl.slotBase = slots;
        cl.coefOffset = coef.size();
        buildReductions(b, cl, coef);
        slots += (int)(cl.reds.size() * M);
    }
    b->numSlots = slots;
    // operand images of every (class, pass, member), on host threads
    std::vector<float> host(std::max<size_t>(imgTotal, 4));
    std::vector<std::tuple<int, int, int>> imgJobs;            // class, pass, member
    for (int c = 0; c < C; ++c)
        for (size_t p = 0; p < b->classes[c].shape.size(); ++p)
            for (size_t m = 0; m < b->classes[c].members.size(); ++m) imgJobs.emplace_back(c, (int)p, (int)m);
    parallelFor(imgJobs.size(), std::min(hw, 16u), [&](size_t j) {
        const int c = std::get<0>(imgJobs[j]), p = std::get<1>(imgJobs[j]), m = std::get<2>(imgJobs[j]);
        const TrotterClass& cl = b->classes[c];
        tcBuildImage(widenNarrow(planOf(c, m).passes[p], cl.n), host.data() + cl.imgOffset[p] + m * cl.imgStride[p],
                     b->parts);
    });
    // device side
    cudaStream_t st = stream();
    std::vector<long long> init(B);
    for (int k = 0; k < B; ++k) init[b->classes[b->classOf[k]].posBase + b->posOf[k]] = b->inst[k].init;
    if (QG_CUDA(cudaMalloc(&b->re, stateFloats * sizeof(float)), kFn) ||
        QG_CUDA(cudaMalloc(&b->im, stateFloats * sizeof(float)), kFn) ||
        QG_CUDA(cudaMalloc(&b->images, host.size() * sizeof(float)), kFn) ||
        QG_CUDA(cudaMalloc(&b->dInit, B * sizeof(long long)), kFn) ||
        QG_CUDA(cudaMalloc(&b->dCoef, std::max<size_t>(1, coef.size()) * sizeof(float)), kFn) ||
        QG_CUDA(cudaMalloc(&b->dResults, 2 * (size_t)b->numSlots * sizeof(double)), kFn) ||
        QG_CUDA(cudaMallocHost(&b->hResults, 2 * (size_t)b->numSlots * sizeof(double)), kFn))
        return false;
    if (QG_CUDA(cudaMemcpyAsync(b->images, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice, st), kFn) ||
        QG_CUDA(cudaMemcpyAsync(b->dInit, init.data(), B * sizeof(long long), cudaMemcpyHostToDevice, st), kFn) ||
        QG_CUDA(cudaMemcpyAsync(b->dCoef, coef.data(), coef.size() * sizeof(float), cudaMemcpyHostToDevice, st), kFn) ||
        QG_CUDA(cudaStreamSynchronize(st), kFn))
        return false;
    b->compiled = true;
    return true;
}

// the run's work, queued on `st` (the library stream, or a capture stream):
// class after class, its states' initialisation, its passes (one launch each
// over the class's states) and its reductions (one launch each over the
// class's states), then one copy of every result to pinned host memory
bool queueRun(TrotterBatch* b, cudaStream_t st) {
    if (QG_CUDA(cudaMemsetAsync(b->errFlag, 0, sizeof(int), st), kFn)) return false;
    for (const TrotterClass& cl : b->classes) {
        const int M = (int)cl.members.size();
        const uint64_t dim = 1ull << cl.n, all = dim * (uint64_t)M;
        float* re = b->re + cl.stateOffset;
        float* im = b->im + cl.stateOffset;
        if (QG_CUDA(cudaMemsetAsync(re, 0, all * sizeof(float), st), kFn) ||
            QG_CUDA(cudaMemsetAsync(im, 0, all * sizeof(float), st), kFn))
            return false;
        kBatchClassical<<<(M + 127) / 128, 128, 0, st>>>(re, dim, b->dInit + cl.posBase, M);
        if (launchFailed(kFn)) return false;
        for (size_t p = 0; p < cl.shape.size(); ++p)
            if (!applyPassTCBatch(re, im, cl.n, cl.shape[p], b->images + cl.imgOffset[p], cl.imgStride[p], b->parts, M,
                                  b->errFlag, st)) {
                invalidQuESTInputError("A pass of the Trotter batch could not be launched on the tensor cores.", kFn);
                return false;
            }
        double* partials = b->partials + (size_t)cl.posBase * kMaxBlocksPerInst;
        unsigned int* counters = b->counters + cl.posBase;
        for (size_t l = 0; l < cl.reds.size(); ++l) {
            const Red& r = cl.reds[l];
            const float* coef = b->dCoef + cl.coefOffset + l * (size_t)M * kCoefs;
            double* out = b->dResults + 2 * ((size_t)cl.slotBase + l * (size_t)M);
            // items: a pair (kind 0), four pairs or 8 amplitudes (kinds 3, 2), kDiagItem amplitudes (kind 1)
            const uint64_t items = r.kind == 0 ? dim / 2 : r.kind == 1 ? dim / kDiagItem : dim / 8;
            const unsigned bx = (unsigned)std::max<uint64_t>(
                1, std::min<uint64_t>({(uint64_t)kMaxBlocksPerInst, (items + red::kThreads - 1) / red::kThreads,
                                       std::max<uint64_t>(1, 8ull * (uint64_t)numSMs() / (uint64_t)M)}));
            const dim3 grid(bx, (unsigned)M);
            if (r.kind == 0)
                kReduceBatch<<<grid, red::kThreads, 0, st>>>(PairsF32{re, im, dim, r.ps, coef}, items, partials,
                                                             counters, out);
            else if (r.kind == 3)
                kReduceBatch<<<grid, red::kThreads, 0, st>>>(PairsF32x4{re, im, dim, r.ps, coef}, items, partials,
                                                             counters, out);
            else if (r.kind == 1)
                kReduceBatch<<<grid, red::kThreads, 0, st>>>(DiagF32{re, im, dim, r.ds, coef}, items, partials,
                                                             counters, out);
            else
                kReduceBatch<<<grid, red::kThreads, 0, st>>>(NormF32b{re, im, dim}, items, partials, counters, out);
            if (launchFailed(kFn)) return false;
        }
    }
    return !QG_CUDA(cudaMemcpyAsync(b->hResults, b->dResults, 2 * (size_t)b->numSlots * sizeof(double),
                                    cudaMemcpyDeviceToHost, st), kFn);
}

}  // namespace
}  // namespace qg

// ============================================================ C ABI
using qg::TrotterBatch;

extern "C" {

void* quest_gb300_trotterBatchCreate(int numQubits, int numInstances) {
    const char* fn = "quest_gb300_trotterBatchCreate";
    if (numQubits < 11 || numQubits > 34 || numInstances < 1 || numInstances > 4096) {
        invalidQuESTInputError("A Trotter batch takes 11 to 34 qubits and 1 to 4096 instances.", fn);
        return nullptr;
    }
    TrotterBatch* b = new TrotterBatch();
    b->maxQubits = numQubits;
    b->B = numInstances;
    b->inst.resize(numInstances);
    if (QG_CUDA(cudaMalloc(&b->errFlag, sizeof(int)), fn) ||
        QG_CUDA(cudaMalloc(&b->partials, (size_t)numInstances * (qg::kMaxBlocksPerInst + 1) * sizeof(double)), fn)) {
        if (b->errFlag) cudaFree(b->errFlag);
        if (b->partials) cudaFree(b->partials);
        delete b;
        return nullptr;
    }
    b->counters = reinterpret_cast<unsigned int*>(b->partials + (size_t)numInstances * qg::kMaxBlocksPerInst);
    cudaMemsetAsync(b->counters, 0, numInstances * sizeof(unsigned int), qg::stream());
    return b;
}

int quest_gb300_trotterBatchSetInstance(void* batch, int instance, PauliHamil hamil, double time, int order, int reps,
                                        long long initClassicalState) {
    const char* fn = "quest_gb300_trotterBatchSetInstance";
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    if (!b || instance < 0 || instance >= b->B) {
        invalidQuESTInputError("Invalid Trotter batch or instance index.", fn);
        return -1;
    }
    if (hamil.numQubits < 11 || hamil.numQubits > b->maxQubits || hamil.numSumTerms < 1 || !hamil.pauliCodes ||
        !hamil.termCoeffs || !(order == 1 || (order >= 2 && order % 2 == 0)) || reps < 1 || initClassicalState < 0 ||
        initClassicalState >= (1ll << hamil.numQubits)) {
        invalidQuESTInputError("Invalid Hamiltonian, order, repetitions or initial state for the Trotter batch.", fn);
        return -1;
    }
    qg::Instance& in = b->inst[instance];
    in.codes.resize((size_t)hamil.numSumTerms * hamil.numQubits);
    for (size_t i = 0; i < in.codes.size(); ++i) {
        const int c = (int)hamil.pauliCodes[i];
        if (c < 0 || c > 3) {
            invalidQuESTInputError("Invalid Pauli code in the Trotter batch's Hamiltonian.", fn);
            return -1;
        }
        in.codes[i] = c;
    }
    in.circuit = false;
    in.gates.clear();
    in.n = hamil.numQubits;
    in.coeffs.assign(hamil.termCoeffs, hamil.termCoeffs + hamil.numSumTerms);
    in.time = time;
    in.order = order;
    in.reps = reps;
    in.init = initClassicalState;
    in.set = true;
    cudaStreamSynchronize(qg::stream());
    qg::freeDevice(b);                               // recompiled at the next run
    return 0;
}

int quest_gb300_trotterBatchSetCircuit(void* batch, int instance, void* plan, PauliHamil hamil,
                                       long long initClassicalState) {
    const char* fn = "quest_gb300_trotterBatchSetCircuit";
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    const qg::FusedPlan* p = reinterpret_cast<const qg::FusedPlan*>(plan);
    if (!b || instance < 0 || instance >= b->B || !p) {
        invalidQuESTInputError("Invalid batch, instance index or plan.", fn);
        return -1;
    }
    const int n = p->numQubits;
    if (n < 11 || n > b->maxQubits || initClassicalState < 0 || initClassicalState >= (1ll << n)) {
        invalidQuESTInputError("Invalid register size or initial state for the batch.", fn);
        return -1;
    }
    if (hamil.numSumTerms > 0 && (hamil.numQubits != n || !hamil.pauliCodes || !hamil.termCoeffs)) {
        invalidQuESTInputError("The measured Hamiltonian must act on the circuit's qubits.", fn);
        return -1;
    }
    qg::Instance& in = b->inst[instance];
    in.codes.clear();
    in.coeffs.clear();
    if (hamil.numSumTerms > 0) {
        in.codes.resize((size_t)hamil.numSumTerms * n);
        for (size_t i = 0; i < in.codes.size(); ++i) {
            const int c = (int)hamil.pauliCodes[i];
            if (c < 0 || c > 3) {
                invalidQuESTInputError("Invalid Pauli code in the measured Hamiltonian.", fn);
                return -1;
            }
            in.codes[i] = c;
        }
        in.coeffs.assign(hamil.termCoeffs, hamil.termCoeffs + hamil.numSumTerms);
    }
    in.circuit = true;
    in.gates = p->gates;
    in.n = n;
    in.time = 0.0;
    in.order = 1;
    in.reps = 1;
    in.init = initClassicalState;
    in.set = true;
    cudaStreamSynchronize(qg::stream());
    qg::freeDevice(b);                               // recompiled at the next run
    return 0;
}

int quest_gb300_trotterBatchRun(void* batch, double* energies) {
    const char* fn = "quest_gb300_trotterBatchRun";
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    if (!b) return -1;
    // images built for another precision or kernel choice are rebuilt
    if (b->compiled && (qg::tcImageParts() & ~b->parts) != 0) {
        cudaStreamSynchronize(qg::stream());
        qg::freeDevice(b);
    }
    if (!b->compiled && !qg::compileBatch(b)) {
        qg::freeDevice(b);
        return -1;
    }
    cudaStream_t st = qg::stream();
    if (b->exec) {
        if (QG_CUDA(cudaGraphLaunch(b->exec, st), fn)) return -1;
        qg::g_launches.fetch_add(1);
    } else {
        if (!qg::queueRun(b, st)) return -1;
    }
    if (QG_CUDA(cudaStreamSynchronize(st), fn)) return -1;
    int err = 0;
    if (QG_CUDA(cudaMemcpy(&err, b->errFlag, sizeof(int), cudaMemcpyDeviceToHost), fn)) return -1;
    if (err) {
        invalidQuESTInputError(err == 6 ? "A split-FP16 tensor-core pass of the Trotter batch gave a non-finite output."
                                        : "A tensor-core pass of the Trotter batch timed out waiting on its pipeline.",
                               fn);
        return -1;
    }
    if (energies)
        for (int k = 0; k < b->B; ++k) {
            const qg::TrotterClass& cl = b->classes[b->classOf[k]];
            const int m = b->posOf[k];
            double e = 0.0;
            for (int s : cl.groupSlots[m]) e += b->hResults[2 * s];
            const double norm = b->hResults[2 * cl.normSlot[m]];
            energies[k] = (norm > 0 ? e / norm : 0.0) + cl.identity[m];
        }
    if (!b->exec) {
        // later runs replay the same work as one graph
        cudaStream_t cap = nullptr;
        if (!QG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), fn)) {
            bool ok = !QG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), fn);
            if (ok) {
                const bool queued = qg::queueRun(b, cap);
                ok = !QG_CUDA(cudaStreamEndCapture(cap, &b->graph), fn) && queued;
            }
            if (ok) ok = !QG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), fn);
            if (!ok) {
                if (b->graph) cudaGraphDestroy(b->graph);
                b->graph = nullptr;
                b->exec = nullptr;
            }
            cudaStreamDestroy(cap);
        }
    }
    ++b->runs;
    return 0;
}

int quest_gb300_trotterBatchCopyState(void* batch, int instance, Qureg dst) {
    const char* fn = "quest_gb300_trotterBatchCopyState";
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    if (!b || instance < 0 || instance >= b->B || dst.isDensityMatrix || !dst.deviceStateVec.real) {
        invalidQuESTInputError("Invalid Trotter batch instance or destination register.", fn);
        return -1;
    }
    if (b->runs == 0 || !b->compiled) {
        invalidQuESTInputError("The Trotter batch has no state to copy: run it first.", fn);
        return -1;
    }
    const qg::TrotterClass& cl = b->classes[b->classOf[instance]];
    const int m = b->posOf[instance];
    if (dst.numQubitsRepresented != cl.n) {
        invalidQuESTInputError("The destination register's size differs from the instance's.", fn);
        return -1;
    }
    qg::captureDiscard(dst.deviceStateVec.real);
    const uint64_t dim = 1ull << cl.n;
    cudaStream_t st = qg::stream();
    // the FP32 passes drift the norm by ~1e-7 each (no correction inside a
    // batch): the copy restores the start state's norm, 1, from the norm the
    // last run measured
    double scale = 1.0;
    const double norm = b->hResults[2 * cl.normSlot[m]];
    if (norm > 0) scale = 1.0 / std::sqrt(norm);
    const size_t off = cl.stateOffset + (size_t)m * dim;
    qg::kBatchToF64<<<4 * qg::numSMs(), 256, 0, st>>>(b->re + off, b->im + off, dst.deviceStateVec.real,
                                                      dst.deviceStateVec.imag, dim, scale);
    if (qg::launchFailed(fn)) return -1;
    return QG_CUDA(cudaStreamSynchronize(st), fn) ? -1 : 0;
}

int quest_gb300_trotterBatchNumPasses(void* batch) {
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    if (!b || !b->compiled) return -1;
    size_t passes = 0;
    for (const qg::TrotterClass& cl : b->classes) passes += cl.shape.size();
    return (int)passes;
}

int quest_gb300_trotterBatchNumClasses(void* batch) {
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    return b && b->compiled ? (int)b->classes.size() : -1;
}

void quest_gb300_trotterBatchDestroy(void* batch) {
    TrotterBatch* b = reinterpret_cast<TrotterBatch*>(batch);
    if (!b) return;
    cudaStreamSynchronize(qg::stream());
    qg::freeDevice(b);
    if (b->errFlag) cudaFree(b->errFlag);
    if (b->partials) cudaFree(b->partials);
    delete b;
}

}  // extern "C"
