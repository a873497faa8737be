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
// a per-CTA slice of a global arena: pass A writes it with 16-byte stores,
// and in pass B each warp takes 32 x 32 (a, b) tiles, reading the swapped
// half row by row (coalesced) and transposing it through its own
// shared-memory tile, so no block-wide barrier is needed inside the pass.
// Amplitudes are FP32; |omega|^2 terms are summed in FP32 within a thread's
// share of a tile (at most 32 terms) and in FP64 above that.
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
constexpr int kSwapCtasPerSM = 4;        // the most CTAs per SM (launch bounds); the default
constexpr int kAreaFloats = (kSwapThreads / 32) * 32 * 33;   // 8 transpose tiles (33.8 KB)
constexpr int kSmemAmps = 8192;          // default: pass A/B in shared memory up to 2^13 amplitudes (d <= 6)
static_assert(kSmemAmps <= kAreaFloats, "a small state must fit the tile area");
constexpr int kMaxD = 10;
constexpr double kInvSqrt2 = 0.70710678118654752440;

struct SwapJob {
    long long offA, offB;    // offsets of u and v in the vector pool
    int d;
    int out;                 // index into the result array
};

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

__global__ void __launch_bounds__(kSwapThreads, kSwapCtasPerSM) kSwapTests(const float* __restrict__ pool,
                                                                           const SwapJob* __restrict__ jobs, int numJobs,
                                                                           unsigned int* __restrict__ ticket,
                                                                           float* __restrict__ arena, size_t arenaPerCta,
                                                                           double* __restrict__ out, int smemAmps) {
    __shared__ __align__(16) float su[1 << kMaxD];
    __shared__ float sv[1 << kMaxD];
    // the whole state of a small test, or the warps' 32 x 33 transpose tiles
    __shared__ __align__(16) float area[kAreaFloats];
    __shared__ double red[kSwapThreads / 32];
    __shared__ int sJob;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
        double total = 0.0;
        if (2 * half <= (uint64_t)smemAmps) {
            // ---- small state, in shared memory
            float* phi = area;
            for (uint32_t idx = threadIdx.x; idx < half; idx += kSwapThreads) {
                const float val = su[idx & (D - 1)] * sv[idx >> d] * (float)kInvSqrt2;
                phi[idx] = val;
                phi[half + idx] = val;
            }
            __syncthreads();
            float s = 0.f;
            for (uint32_t idx = threadIdx.x; idx < half; idx += kSwapThreads) {
                const uint32_t a = idx & (D - 1), b = idx >> d;
                const float w = (phi[idx] + phi[half + b + (a << d)]) * (float)kInvSqrt2;
                s = fmaf(w, w, s);
            }
            total = (double)s;
        } else {
            // ---- pass A: |0>|v>|u> then H(anc): both halves = u_a v_b / sqrt2,
            // written as 16-byte vectors (4 consecutive a, one b)
            float4* phi4 = reinterpret_cast<float4*>(myArena);
            const uint32_t half4 = (uint32_t)(half >> 2);
            for (uint32_t i4 = threadIdx.x; i4 < half4; i4 += kSwapThreads) {
                const uint32_t idx = i4 << 2;
                const float vb = sv[idx >> d] * (float)kInvSqrt2;
                const float4 u4 = *reinterpret_cast<const float4*>(su + (idx & (D - 1)));
                const float4 val = make_float4(u4.x * vb, u4.y * vb, u4.z * vb, u4.w * vb);
                __stcg(phi4 + i4, val);
                __stcg(phi4 + half4 + i4, val);
            }
            __syncthreads();
            // ---- pass B: CSWAPs (anc=1 half: u <-> v), H(anc), P(anc = 0),
            // over 32 x 32 (a, b) tiles, one warp per tile: the swapped half
            // is read row by row (coalesced) and transposed through the
            // warp's own shared-memory tile
            const float* phi = myArena;
            float(*tile)[33] = reinterpret_cast<float(*)[33]>(area + warp * 32 * 33);
            const int T = D / 32;
            for (int t = warp; t < T * T; t += kSwapThreads / 32) {
                const int a0 = (t % T) * 32, b0 = (t / T) * 32;
                const float* row1 = phi + half + (uint64_t)(b0 + lane) + ((uint64_t)a0 << d);
#pragma unroll 8
                for (int r = 0; r < 32; ++r) tile[r][lane] = __ldcg(row1 + ((uint64_t)r << d));   // phi(1, b0+lane, a0+r)
                __syncwarp();
                const float* col0 = phi + (uint64_t)(a0 + lane) + ((uint64_t)b0 << d);
                float s = 0.f;
#pragma unroll 8
                for (int r = 0; r < 32; ++r) {
                    const float w = (__ldcg(col0 + ((uint64_t)r << d)) + tile[lane][r]) * (float)kInvSqrt2;
                    s = fmaf(w, w, s);
                }
                __syncwarp();
                total += (double)s;                      // FP32 within a tile (32 terms), FP64 across tiles
            }
        }
        const double p0 = blockSum(total, red);
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
    size_t arenaPerCta = 0;           // floats per CTA of the arena (for up to kSwapCtasPerSM CTAs per SM)
    double* out = nullptr;
    int maxD = 1;
    int ctasPerSM = kSwapCtasPerSM;   // tunable: 1 .. kSwapCtasPerSM
    int smemAmps = kSmemAmps;         // tunable: states of at most this many amplitudes stay in shared memory
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double* hostOut = nullptr;        // pinned
};

void dropGraph(SwapBatch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// the run's work on `st`: reset the ticket, the persistent kernel, results to
// pinned host memory
void queueSwaps(SwapBatch* b, cudaStream_t st) {
    cudaMemsetAsync(b->ticket, 0, sizeof(unsigned int), st);
    kSwapTests<<<numSMs() * b->ctasPerSM, kSwapThreads, 0, st>>>(b->pool, b->jobs, b->numTests, b->ticket, b->arena,
                                                                  b->arenaPerCta, b->out, b->smemAmps);
    cudaMemcpyAsync(b->hostOut, b->out, b->numTests * sizeof(double), cudaMemcpyDeviceToHost, st);
}

// (re)capture the graph for the current parameters
bool captureSwaps(SwapBatch* b, const char* fn) {
    dropGraph(b);
    cudaStream_t cap = nullptr;
    if (QG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), fn)) return false;
    bool ok = !QG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), fn);
    if (ok) {
        queueSwaps(b, cap);
        ok = !QG_CUDA(cudaStreamEndCapture(cap, &b->graph), fn);
    }
    if (ok) ok = !QG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), fn);
    cudaStreamDestroy(cap);
    if (!ok) dropGraph(b);
    return ok;
}

void freeBatch(SwapBatch* b) {
    if (!b) return;
    cudaStreamSynchronize(stream());
    dropGraph(b);
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
    b->maxD = maxD;
    // an arena slice per CTA for every state that may leave shared memory
    // (any state above the smallest tunable threshold)
    const size_t arenaNeed = (2ull << (2 * maxD)) > 512 ? (2ull << (2 * maxD)) : 0;
    b->arenaPerCta = arenaNeed;
    const size_t maxGrid = (size_t)qg::numSMs() * qg::kSwapCtasPerSM;
    std::vector<float> pool32(poolLen);
    for (long long i = 0; i < poolLen; ++i) pool32[i] = (float)vectors[i];
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaMalloc(&b->pool, poolLen * sizeof(float)), fn) ||
        QG_CUDA(cudaMalloc(&b->jobs, numTests * sizeof(SwapJob)), fn) ||
        QG_CUDA(cudaMalloc(&b->ticket, sizeof(unsigned int)), fn) ||
        QG_CUDA(cudaMalloc(&b->out, numTests * sizeof(double)), fn) ||
        QG_CUDA(cudaMallocHost(&b->hostOut, numTests * sizeof(double)), fn) ||
        (arenaNeed && QG_CUDA(cudaMalloc(&b->arena, arenaNeed * maxGrid * sizeof(float)), fn))) {
        qg::freeBatch(b);
        return nullptr;
    }
    QG_CUDA(cudaMemcpyAsync(b->pool, pool32.data(), poolLen * sizeof(float), cudaMemcpyHostToDevice, st), fn);
    QG_CUDA(cudaMemcpyAsync(b->jobs, jobs.data(), numTests * sizeof(SwapJob), cudaMemcpyHostToDevice, st), fn);
    QG_CUDA(cudaStreamSynchronize(st), fn);
    if (!qg::captureSwaps(b, fn)) {
        qg::freeBatch(b);
        return nullptr;
    }
    return b;
}

// Time the batch with every pairing of CTAs per SM (2, 3, 4) and
// shared-memory threshold (states of up to 2^9, 2^11 or 2^13 amplitudes stay
// in shared memory: d <= 4, 5 or 6), two runs each, keep the fastest and
// capture the graph again with it.  Writes the choice, its time and the time
// of the default (4 CTAs per SM, 2^13) in ms; returns 0 or -1.
int quest_gb300_swapTestBatchTune(void* batch, int* ctasPerSM, int* smemAmps, double* msBest, double* msDefault) {
    SwapBatch* b = reinterpret_cast<SwapBatch*>(batch);
    const char* fn = "quest_gb300_swapTestBatchTune";
    if (!b) return -1;
    cudaStream_t st = qg::stream();
    cudaEvent_t e0, e1;
    if (QG_CUDA(cudaEventCreate(&e0), fn) || QG_CUDA(cudaEventCreate(&e1), fn)) return -1;
    double best = -1, dflt = -1;
    int bestC = qg::kSwapCtasPerSM, bestS = qg::kSmemAmps;
    for (int c = 2; c <= qg::kSwapCtasPerSM; ++c)
        for (int sm : {512, 2048, 8192}) {
            b->ctasPerSM = c;
            b->smemAmps = sm;
            qg::queueSwaps(b, st);                    // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < 2; ++r) qg::queueSwaps(b, st);
            cudaEventRecord(e1, st);
            if (QG_CUDA(cudaEventSynchronize(e1), fn)) return -1;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            const double per = ms / 2.0;
            if (c == qg::kSwapCtasPerSM && sm == qg::kSmemAmps) dflt = per;
            if (best < 0 || per < best) {
                best = per;
                bestC = c;
                bestS = sm;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->ctasPerSM = bestC;
    b->smemAmps = bestS;
    if (!qg::captureSwaps(b, fn)) return -1;
    if (ctasPerSM) *ctasPerSM = bestC;
    if (smemAmps) *smemAmps = bestS;
    if (msBest) *msBest = best;
    if (msDefault) *msDefault = dflt;
    return 0;
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
