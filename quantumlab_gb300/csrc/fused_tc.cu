// fused_tc.cu -- tensor-core applier of the FP32 fused engine (sm_103a,
// tcgen05 + TMEM, 3-term split-TF32).  No counterpart in the reference.
//
// A pass multiplies the FP32 state by a dense 2^k x 2^k complex matrix G on
// qubits T (k = 4..6).  With D = 2^k, a tile of 128 consecutive "groups"
// (the non-target bits, inserted around T) is the GEMM
//
//     Out[c][r] = sum_j X[c][j] * Gr[r][j]          c < 128, r, j < 2D
//
// where X[c] = (re of the group's D amplitudes, then im) and Gr is the real
// form [[Re G, -Im G], [Im G, Re G]].  On tcgen05: A = X (M = 128, K = 2D,
// kept in TMEM), B = Gr (N = 2D, K-major in shared memory), D = Out in TMEM.
// Split-TF32: X = Xh + Xl and Gr = Gh + Gl with Xh, Gh exact TF32 values and
// the MMA truncating Xl, Gl to TF32; Out = Xh.Gh + Xl.Gh + Xh.Gl accumulated
// in FP32 (relative error ~2^-21 per product instead of 2^-11).
//
// Data path (per CTA, persistent over tiles):
//   * Gh/Gl: prepared on the host in the canonical no-swizzle K-major UMMA
//     layout and staged once per CTA by a TMA bulk copy (cp.async.bulk) into
//     shared memory;
//   * X: each thread owns one tile column (TMEM lane) and loads its 2D values
//     straight from global memory -- the 32 lanes of a warp read 32
//     consecutive amplitudes, so every load is a coalesced 128-byte line --
//     splits them in registers and writes Xh, Xl to TMEM with tcgen05.st.
//     Staging X through shared memory would add two shared-memory passes over
//     the data for no gain: the split needs it in registers anyway;
//   * one thread issues the 3 x (2D/8) MMAs (K = 8 each) and commits them to
//     an mbarrier; all threads wait on it (bounded spin), read Out with
//     tcgen05.ld and store it with coalesced 128-byte warp stores.
// Several CTAs share an SM where TMEM allows, so one CTA's loads overlap
// another's MMAs and stores.
//
// Every wait is bounded: on timeout the CTA records an error code in a
// device flag, skips the rest of its tiles, frees its TMEM and returns; the
// host reads the flag after the pass.
#include "fused_plan.h"
#include "qg_internal.h"

#include <cstdint>
#include <algorithm>
#include <cstring>
#include <vector>

namespace qg {

struct QuregF32;   // fused_f32.cu
float* f32re(QuregF32& q);
float* f32im(QuregF32& q);
int f32n(const QuregF32& q);

namespace {

constexpr int kTile = 128;              // groups per tile = MMA M = TMEM lanes
constexpr int kThreadsTC = 128;         // 4 warps: one TMEM lane quarter each
constexpr long long kSpinLimit = 1ll << 26;

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count));
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
}
// bounded wait for the phase with the given parity to complete; false on timeout
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smemAddr(bar);
    for (long long i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulkG2S(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(dst)),
                 "l"(src), "r"(bytes), "r"(smemAddr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmemAlloc(uint32_t* dstSmem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dstSmem)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmemSt16(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
__device__ __forceinline__ void tmemWaitSt() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmemLd16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmemWaitLd() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// D[tmem] (+)= A[tmem] * B[smem desc]
__device__ __forceinline__ void mmaTF32(uint32_t dT, uint32_t aT, uint64_t bDesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}" ::"r"(dT),
        "r"(aT), "l"(bDesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mmaCommit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
                 : "memory");
}

// shared-memory matrix descriptor: no swizzle, K-major
//   bits 0-13 start>>4, 16-29 LBO>>4, 32-45 SBO>>4, 46-47 version 1, 61-63 layout 0
__device__ __forceinline__ uint64_t smemDesc(uint32_t start, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((start >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major
__host__ __device__ constexpr uint32_t idescTF32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t tf32Hi(float x) { return __float_as_uint(x) & 0xFFFFE000u; }

// ------------------------------------------------------------ the kernel
// TMEM columns: [0, K) Xh, [K, 2K) Xl, [2K, 2K+N) Out, with K = N = 2D.
template <int KQ>
struct TCParams {
    uint64_t off[1 << KQ];      // amplitude offset of matrix index j
    int ins[KQ];                // ascending target positions
};

template <int KQ>
__global__ void __launch_bounds__(kThreadsTC) kApplyTC(float* __restrict__ re, float* __restrict__ im,
                                                       const float* __restrict__ gImage, uint64_t numTiles,
                                                       int* __restrict__ errFlag,
                                                       const __grid_constant__ TCParams<KQ> p) {
    constexpr int D = 1 << KQ;
    constexpr int K = 2 * D;                    // GEMM K = N
    constexpr int N = 2 * D;
    constexpr uint32_t kGBytes = (uint32_t)N * K * 4;   // one of Gh / Gl
    constexpr uint32_t kCols = (2 * K + N) <= 64 ? 64 : ((2 * K + N) <= 128 ? 128 : ((2 * K + N) <= 256 ? 256 : 512));
    constexpr uint32_t kLBO = 128;               // K-adjacent core matrices
    constexpr uint32_t kSBO = (K / 4) * 128;     // 8-row groups
    constexpr uint32_t idesc = idescTF32(kTile, N);

    extern __shared__ __align__(1024) uint8_t smem[];
    float* gh = reinterpret_cast<float*>(smem);
    float* gl = reinterpret_cast<float*>(smem + kGBytes);
    __shared__ __align__(8) uint64_t barG, barMma;
    __shared__ uint32_t tmemBase;
    __shared__ int abortFlag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        abortFlag = 0;
        mbarInit(&barG, 1);
        mbarInit(&barMma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0) tmemAlloc(&tmemBase, kCols);
    if (threadIdx.x == 0) {
        mbarExpectTx(&barG, 2 * kGBytes);
        bulkG2S(gh, gImage, kGBytes, &barG);
        bulkG2S(gl, gImage + (size_t)N * K, kGBytes, &barG);
    }
    fenceBefore();
    __syncthreads();
    fenceAfter();
    const uint32_t tbase = tmemBase;
    const uint32_t laneBase = (uint32_t)(warp * 32) << 16;
    const uint32_t tXh = tbase, tXl = tbase + K, tOut = tbase + 2 * K;

    if (threadIdx.x == 0 && !mbarWait(&barG, 0)) {
        atomicExch(errFlag, 1);
        abortFlag = 1;
        mbarWait(&barG, 0);            // bounded second wait for the copies in flight
    }
    __syncthreads();
    uint32_t mmaPhase = 0;
    const uint32_t ghAddr = smemAddr(gh), glAddr = smemAddr(gl);

    const bool aborted = abortFlag != 0;                   // read after the barrier above: uniform
    for (uint64_t tile = blockIdx.x; tile < numTiles && !aborted; tile += gridDim.x) {
        // ---- load this lane's group, split, write Xh / Xl rows to TMEM
        uint64_t base = tile * kTile + (uint64_t)threadIdx.x;
#pragma unroll
        for (int b = 0; b < KQ; ++b) {
            const int s = p.ins[b];
            base = ((base >> s) << (s + 1)) | (base & ((1ull << s) - 1ull));
        }
        // K index: re rows (j < D), then im rows.  Loads go in chunks of at
        // most 64 values so all of a chunk's loads are in flight together.
        constexpr int CH = K < 64 ? K : 64;
#pragma unroll
        for (int h = 0; h < K; h += CH) {
            float x[CH];
#pragma unroll
            for (int e = 0; e < CH; ++e) {
                const int j = h + e;
                x[e] = (j < D) ? re[base + p.off[j]] : im[base + p.off[j - D]];
            }
#pragma unroll
            for (int c0 = 0; c0 < CH; c0 += 16) {
                uint32_t hi[16], lo[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    hi[e] = tf32Hi(x[c0 + e]);
                    lo[e] = __float_as_uint(x[c0 + e] - __uint_as_float(hi[e]));
                }
                tmemSt16(tXh + laneBase + h + c0, hi);
                tmemSt16(tXl + laneBase + h + c0, lo);
            }
        }
        tmemWaitSt();
        fenceBefore();
        __syncthreads();
        // ---- MMAs (one thread): Out = Xh.Gh + Xl.Gh + Xh.Gl
        if (threadIdx.x == 0) {
            fenceAfter();
#pragma unroll
            for (int s = 0; s < K / 8; ++s) {
                const uint64_t dh = smemDesc(ghAddr + 256u * s, kLBO, kSBO);
                mmaTF32(tOut, tXh + 8 * s, dh, idesc, s > 0);
            }
#pragma unroll
            for (int s = 0; s < K / 8; ++s) {
                const uint64_t dh = smemDesc(ghAddr + 256u * s, kLBO, kSBO);
                mmaTF32(tOut, tXl + 8 * s, dh, idesc, 1);
            }
#pragma unroll
            for (int s = 0; s < K / 8; ++s) {
                const uint64_t dl = smemDesc(glAddr + 256u * s, kLBO, kSBO);
                mmaTF32(tOut, tXh + 8 * s, dl, idesc, 1);
            }
            mmaCommit(&barMma);
        }
        // ---- wait for the MMAs, then store Out[c][r] (r < D: re, else im)
        const bool ok = mbarWait(&barMma, mmaPhase);
        mmaPhase ^= 1u;
        if (__syncthreads_or(!ok)) {                        // uniform decision
            if (threadIdx.x == 0) {
                atomicExch(errFlag, 2);
                mbarWait(&barMma, mmaPhase ^ 1u);           // bounded second wait for the MMAs in flight
            }
            break;
        }
        fenceAfter();
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            tmemLd16(tOut + laneBase + c0, v);
            tmemWaitLd();
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int r = c0 + e;
                if (r < D) re[base + p.off[r]] = __uint_as_float(v[e]);
                else im[base + p.off[r - D]] = __uint_as_float(v[e]);
            }
        }
        fenceBefore();
        __syncthreads();
        fenceAfter();
    }
    __syncthreads();
    if (warp == 0) tmemDealloc(tbase, kCols);
}

// ------------------------------------------------------------ host side
struct DevicePlan {
    std::vector<float*> images;      // per pass: Gh image then Gl image (or nullptr)
    int* errFlag = nullptr;
};

// Canonical no-swizzle K-major image of an N x K operand (rows r, K index j):
// byte (r/8)*SBO + (j/4)*128 + (r%8)*16 + (j%4)*4 with SBO = (K/4)*128.
void packKMajor(const std::vector<float>& rowMajor, int N, int K, float* out) {
    for (int r = 0; r < N; ++r)
        for (int j = 0; j < K; ++j) {
            const size_t byteOff = (size_t)(r / 8) * (K / 4) * 128 + (size_t)(j / 4) * 128 + (r % 8) * 16 + (j % 4) * 4;
            out[byteOff / 4] = rowMajor[(size_t)r * K + j];
        }
}

float hostTf32Hi(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u &= 0xFFFFE000u;
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}

template <int KQ>
bool launchTC(float* re, float* im, int n, const FusedPass& pass, const float* img, int* errFlag, cudaStream_t st) {
    constexpr int D = 1 << KQ;
    constexpr int K = 2 * D;
    const size_t smem = 2 * (size_t)K * K * 4;
    TCParams<KQ> p;
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
        for (int b = 0; b < KQ; ++b)
            if (j >> b & 1) o |= 1ull << pass.targets[b];
        p.off[j] = o;
    }
    for (int b = 0; b < KQ; ++b) p.ins[b] = pass.targets[b];
    const uint64_t numTiles = (1ull << (n - KQ)) / kTile;
    // TMEM columns per CTA (power of two); at most 512 / cols CTAs can hold
    // TMEM on one SM at a time.  Request enough shared memory that the block
    // scheduler never places more CTAs than that on an SM.
    constexpr int cols = (3 * K) <= 64 ? 64 : ((3 * K) <= 128 ? 128 : ((3 * K) <= 256 ? 256 : 512));
    constexpr int perSM = 512 / cols;
    const size_t smemReq = std::max(smem + 1024, (size_t)(220 * 1024 / perSM));
    static bool configured[8] = {};
    if (!configured[KQ]) {
        if (QG_CUDA(cudaFuncSetAttribute(kApplyTC<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemReq),
                    "applyPlanF32"))
            return false;
        configured[KQ] = true;
    }
    const uint64_t grid = std::min<uint64_t>(numTiles, (uint64_t)perSM * numSMs());
    kApplyTC<KQ><<<(unsigned)grid, kThreadsTC, smemReq, st>>>(re, im, img, numTiles, errFlag, p);
    return !launchFailed("applyPlanF32");
}

bool g_tcEnabled = true;
bool g_tcChecked = false;

}  // namespace

void* uploadPlanTC(const FusedPlan& plan) {
    DevicePlan* dp = new DevicePlan();
    if (cudaMalloc(&dp->errFlag, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        delete dp;
        return nullptr;
    }
    cudaMemsetAsync(dp->errFlag, 0, sizeof(int), stream());
    for (const FusedPass& pass : plan.passes) {
        const int k = (int)pass.targets.size();
        if (k < 4 || k > 6 || plan.numQubits < k + 7) {
            dp->images.push_back(nullptr);
            continue;
        }
        const int D = 1 << k, K = 2 * D, N = 2 * D;
        // real form [[Re, -Im], [Im, Re]] as B = Gr (rows r = output index, K index j)
        std::vector<float> hi((size_t)N * K), lo((size_t)N * K);
        for (int r = 0; r < N; ++r)
            for (int j = 0; j < K; ++j) {
                const cplx g = pass.m[(size_t)(r % D) * D + (j % D)];
                double v;
                if (r < D) v = (j < D) ? g.real() : -g.imag();
                else v = (j < D) ? g.imag() : g.real();
                const float h = hostTf32Hi((float)v);
                hi[(size_t)r * K + j] = h;
                lo[(size_t)r * K + j] = (float)(v - (double)h);
            }
        std::vector<float> img(2 * (size_t)N * K);
        packKMajor(hi, N, K, img.data());
        packKMajor(lo, N, K, img.data() + (size_t)N * K);
        float* d = nullptr;
        if (cudaMalloc(&d, img.size() * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            dp->images.push_back(nullptr);
            continue;
        }
        cudaMemcpy(d, img.data(), img.size() * sizeof(float), cudaMemcpyHostToDevice);
        dp->images.push_back(d);
    }
    return dp;
}

void freePlanTC(void* h) {
    DevicePlan* dp = reinterpret_cast<DevicePlan*>(h);
    if (!dp) return;
    cudaStreamSynchronize(stream());
    for (float* f : dp->images)
        if (f) cudaFree(f);
    if (dp->errFlag) cudaFree(dp->errFlag);
    delete dp;
}

// explicit entry used by the FP32 engine with the pass index
bool applyPassTCIndexed(QuregF32& q, const FusedPass& pass, const void* devPlan, size_t index, cudaStream_t st) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    if (!dp || !g_tcEnabled || index >= dp->images.size() || !dp->images[index]) return false;
    const int k = (int)pass.targets.size();
    float* re = f32re(q);
    float* im = f32im(q);
    const int n = f32n(q);
    switch (k) {
        case 4: return launchTC<4>(re, im, n, pass, dp->images[index], dp->errFlag, st);
        case 5: return launchTC<5>(re, im, n, pass, dp->images[index], dp->errFlag, st);
        case 6: return launchTC<6>(re, im, n, pass, dp->images[index], dp->errFlag, st);
        default: return false;
    }
}

int tcErrorFlag(const void* devPlan) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    if (!dp || !dp->errFlag) return 0;
    int v = 0;
    cudaMemcpyAsync(&v, dp->errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    return v;
}

void setTensorCoresEnabled(bool on) { g_tcEnabled = on; }
bool tensorCoresEnabled() { return g_tcEnabled; }

}  // namespace qg
