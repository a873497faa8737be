// batch_swap.cu -- batched swap tests (QKMeans distances) in one persistent
// kernel, replayed through a CUDA graph.  No counterpart in the reference:
// QuantumLab runs one (2d+1)-qubit circuit at a time through the QuEST API
// (Code/QuantumLab/Circuit/Subroutine/QKMeans.cu:1158-1290,
// Code/QuantumLab/Circuit/Gates/SwapTest.cpp:15-68), each gate a launch.
//
// Circuit of one test (u, v of length 2^d, qubits: u = 0..d-1, v = d..2d-1,
// ancilla = 2d):   |0>|v>|u>  ->  H(anc)  ->  prod_i CSWAP(anc; u_i, v_i)
//                  ->  H(anc)  ->  P(anc = 0).
// The engine simulates it on an explicit FP32 state vector of 2^(2d+1)
// amplitudes, with two fused passes:
//   pass A = state preparation + H(anc): phi(x, a, b) = u_a v_b / sqrt2 for
//            both ancilla values (a = u-register index, b = v-register index);
//   pass B = the d controlled swaps (they share the control and commute, so
//            together they exchange the u and v registers on the anc = 1
//            half: chi(1, a, b) = phi(1, b, a)) + H(anc) + the probability
//            P0 = sum_{a,b} |(chi(0,a,b) + chi(1,a,b)) / sqrt2|^2.
// Small states (2^(2d+1) <= kSmemAmps) live in shared memory; larger ones in
// a per-CTA slice of a global arena, where pass B reads the swapped half
// through a shared-memory tile transpose so both reads stay coalesced.
// Amplitudes are FP32; each thread sums its |omega|^2 terms with FP32 Kahan
// compensation and the thread / block totals are combined in FP64.
//
// Scheduling: tests are sorted by size (largest first) and CTAs take the
// next one from a global ticket (atomicAdd), so uneven sizes balance.
#include "qg_internal.h"
#include "quest_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

namespace qg {
namespace {

constexpr int kSwapThreads = 256;
constexpr int kSmemAmps = 8192;          // pass A/B in shared memory up to 2^13 amplitudes (d <= 6)
constexpr int kMaxD = 10;
constexpr double kInvSqrt2 = 0.70710678118654752440;

struct SwapJob {
    long long offA, offB;    // offsets of u and v in the vector pool
    int d;
    int out;                 // index into the result array
};

__device__ __forceinline__ void kahanAdd(float& s, float& c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ double blockSum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kSwapThreads) kSwapTests(const float* __restrict__ pool, const SwapJob* __restrict__ jobs,
                                                           int numJobs, unsigned int* __restrict__ ticket,
                                                           float* __restrict__ arena, size_t arenaPerCta,
                                                           double* __restrict__ out) {
    __shared__ float su[1 << kMaxD], sv[1 << kMaxD];
    __shared__ float sstate[kSmemAmps];
    __shared__ float tile[32][33];
    __shared__ double red[kSwapThreads / 32];
    __shared__ int sJob;
    float* myArena = arena + (size_t)blockIdx.x * arenaPerCta;
    for (;;) {
        if (threadIdx.x == 0) sJob = (int)atomicAdd(ticket, 1u);
        __syncthreads();
        const int j = sJob;
        __syncthreads();
        if (j >= numJobs) break;
        const SwapJob job = jobs[j];
        const int d = job.d;
        const int D = 1 << d;
        const uint64_t half = 1ull << (2 * d);          // amplitudes per ancilla value
        for (int i = threadIdx.x; i < D; i += kSwapThreads) {
            su[i] = pool[job.offA + i];
            sv[i] = pool[job.offB + i];
        }
        __syncthreads();
        const bool inSmem = 2 * half <= (uint64_t)kSmemAmps;
        float* phi = inSmem ? sstate : myArena;
        // ---- pass A: |0>|v>|u> then H(anc): both halves = u_a v_b / sqrt2
        for (uint64_t idx = threadIdx.x; idx < half; idx += kSwapThreads) {
            const int a = (int)(idx & (D - 1)), b = (int)(idx >> d);
            const float val = su[a] * sv[b] * (float)kInvSqrt2;
            phi[idx] = val;
            phi[half + idx] = val;
        }
        __syncthreads();
        // ---- pass B: CSWAPs (anc=1 half: u <-> v), H(anc), P(anc = 0)
        float s = 0.f, c = 0.f;
        if (inSmem || D < 32) {
            for (uint64_t idx = threadIdx.x; idx < half; idx += kSwapThreads) {
                const int a = (int)(idx & (D - 1)), b = (int)(idx >> d);
                const float w = (phi[idx] + phi[half + (uint64_t)b + ((uint64_t)a << d)]) * (float)kInvSqrt2;
                kahanAdd(s, c, w * w);
            }
        } else {
            // 32 x 32 tiles of (a, b); the swapped half is read transposed via smem
            const int tiles = D / 32;
            const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;     // 8 rows of 32
            for (int t = 0; t < tiles * tiles; ++t) {
                const int a0 = (t % tiles) * 32, b0 = (t / tiles) * 32;
                // load anc=1 half at (row a0+r, col b0+tx): element phi(1, b, a) for a = a0+r, b = b0+tx
                for (int r = ty; r < 32; r += kSwapThreads / 32)
                    tile[r][tx] = phi[half + (uint64_t)(b0 + tx) + ((uint64_t)(a0 + r) << d)];
                __syncthreads();
                for (int r = ty; r < 32; r += kSwapThreads / 32) {
                    const int a = a0 + tx, b = b0 + r;
                    const float w = (phi[(uint64_t)a + ((uint64_t)b << d)] + tile[tx][r]) * (float)kInvSqrt2;
                    kahanAdd(s, c, w * w);
                }
                __syncthreads();
            }
        }
        const double p0 = blockSum((double)s - (double)c, red);
        if (threadIdx.x == 0) out[job.out] = p0;
        __syncthreads();
    }
}

struct SwapBatch {
    int numTests = 0;
    float* pool = nullptr;
    SwapJob* jobs = nullptr;
    unsigned int* ticket = nullptr;
    float* arena = nullptr;
    size_t arenaPerCta = 0;
    double* out = nullptr;
    int grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double* hostOut = nullptr;        // pinned
};

void freeBatch(SwapBatch* b) {
    if (!b) return;
    cudaStreamSynchronize(stream());
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->pool);
    cudaFree(b->jobs);
    cudaFree(b->ticket);
    cudaFree(b->arena);
    cudaFree(b->out);
    cudaFreeHost(b->hostOut);
    delete b;
}

}  // namespace
}  // namespace qg

using qg::SwapBatch;
using qg::SwapJob;

extern "C" {

void* quest_gb300_swapTestBatchCreate(const double* vectors, const long long* offsets, const int* dimLog2,
                                      int numVectors, const int* idxA, const int* idxB, int numTests) {
    const char* fn = "quest_gb300_swapTestBatchCreate";
    if (!vectors || !offsets || !dimLog2 || !idxA || !idxB || numVectors < 1 || numTests < 1) {
        invalidQuESTInputError("Invalid swap-test batch arguments.", fn);
        return nullptr;
    }
    long long poolLen = 0;
    for (int i = 0; i < numVectors; ++i) {
        if (dimLog2[i] < 1 || dimLog2[i] > qg::kMaxD || offsets[i] < 0) {
            invalidQuESTInputError("Swap-test vectors must have length 2^d with 1 <= d <= 10.", fn);
            return nullptr;
        }
        poolLen = std::max(poolLen, offsets[i] + (1ll << dimLog2[i]));
    }
    std::vector<SwapJob> jobs(numTests);
    int maxD = 1;
    for (int t = 0; t < numTests; ++t) {
        const int a = idxA[t], b = idxB[t];
        if (a < 0 || a >= numVectors || b < 0 || b >= numVectors || dimLog2[a] != dimLog2[b]) {
            invalidQuESTInputError("Swap-test pair indices out of range or of unequal dimension.", fn);
            return nullptr;
        }
        jobs[t] = SwapJob{offsets[a], offsets[b], dimLog2[a], t};
        maxD = std::max(maxD, dimLog2[a]);
    }
    // largest circuits first: dynamic scheduling then balances the tail
    std::stable_sort(jobs.begin(), jobs.end(), [](const SwapJob& x, const SwapJob& y) { return x.d > y.d; });
    SwapBatch* b = new SwapBatch();
    b->numTests = numTests;
    b->grid = qg::numSMs() * 2;
    const size_t arenaNeed = (2ull << (2 * maxD)) > (size_t)qg::kSmemAmps ? (2ull << (2 * maxD)) : 0;
    b->arenaPerCta = arenaNeed;
    std::vector<float> pool32(poolLen);
    for (long long i = 0; i < poolLen; ++i) pool32[i] = (float)vectors[i];
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaMalloc(&b->pool, poolLen * sizeof(float)), fn) ||
        QG_CUDA(cudaMalloc(&b->jobs, numTests * sizeof(SwapJob)), fn) ||
        QG_CUDA(cudaMalloc(&b->ticket, sizeof(unsigned int)), fn) ||
        QG_CUDA(cudaMalloc(&b->out, numTests * sizeof(double)), fn) ||
        QG_CUDA(cudaMallocHost(&b->hostOut, numTests * sizeof(double)), fn) ||
        (arenaNeed && QG_CUDA(cudaMalloc(&b->arena, arenaNeed * b->grid * sizeof(float)), fn))) {
        qg::freeBatch(b);
        return nullptr;
    }
    QG_CUDA(cudaMemcpyAsync(b->pool, pool32.data(), poolLen * sizeof(float), cudaMemcpyHostToDevice, st), fn);
    QG_CUDA(cudaMemcpyAsync(b->jobs, jobs.data(), numTests * sizeof(SwapJob), cudaMemcpyHostToDevice, st), fn);
    QG_CUDA(cudaStreamSynchronize(st), fn);
    // capture: reset ticket, the persistent kernel, results to pinned host
    cudaStream_t cap = nullptr;
    if (QG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), fn)) {
        qg::freeBatch(b);
        return nullptr;
    }
    bool ok = !QG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), fn);
    if (ok) {
        cudaMemsetAsync(b->ticket, 0, sizeof(unsigned int), cap);
        qg::kSwapTests<<<b->grid, qg::kSwapThreads, 0, cap>>>(b->pool, b->jobs, numTests, b->ticket, b->arena,
                                                               b->arenaPerCta, b->out);
        cudaMemcpyAsync(b->hostOut, b->out, numTests * sizeof(double), cudaMemcpyDeviceToHost, cap);
        ok = !QG_CUDA(cudaStreamEndCapture(cap, &b->graph), fn);
    }
    if (ok) ok = !QG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), fn);
    cudaStreamDestroy(cap);
    if (!ok) {
        qg::freeBatch(b);
        return nullptr;
    }
    return b;
}

// Replay the batch's graph on the library stream and write P(anc = 0) of
// every test (in the caller's order) to p0Out (host memory).
int quest_gb300_swapTestBatchRun(void* batch, double* p0Out) {
    SwapBatch* b = reinterpret_cast<SwapBatch*>(batch);
    const char* fn = "quest_gb300_swapTestBatchRun";
    if (!b) return -1;
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaGraphLaunch(b->exec, st), fn)) return -1;
    qg::g_launches.fetch_add(1);
    if (QG_CUDA(cudaStreamSynchronize(st), fn)) return -1;
    if (p0Out) std::memcpy(p0Out, b->hostOut, b->numTests * sizeof(double));
    return 0;
}

void quest_gb300_swapTestBatchDestroy(void* batch) { qg::freeBatch(reinterpret_cast<SwapBatch*>(batch)); }

}  // extern "C"
