// fused_tc.cu -- tensor-core appliers of the FP32 fused engine (sm_103a,
// tcgen05 + TMEM).  No counterpart in the reference.
//
// A pass multiplies the FP32 state by a dense 2^k x 2^k complex matrix G on
// qubits T (k = 4..6).  With D = 2^k, a tile of 128 "groups" (the non-target
// bits, inserted around T) is the GEMM
//
//     Out[c][r] = sum_j X[c][j] * Gr[r][j]          c < 128, r, j < 2D
//
// where X[c] = (re of the group's D amplitudes, then im) and Gr is the real
// form [[Re G, -Im G], [Im G, Re G]].  On tcgen05: A = X (M = 128, K = 2D,
// kept in TMEM), B = Gr (N = 2D, K-major in shared memory), D = Out in TMEM.
//
// Two kernels:
//   * kApplyTC2 (the default; "pipelined kernel" below): warp-specialised and
//     persistent, with one of three operand forms (setTensorCorePrecision):
//       - 3-term split-TF32, the default: X = Xh + Xl and Gr = Gh + Gl in
//         TF32 parts, Out = Xh.Gh + Xl.Gh + Xh.Gl accumulated in FP32 by
//         kind::tf32 MMAs;
//       - 4-term split-BF16: X = Xh + Xl (two BF16 parts, ~2^-17) and
//         Gr = Gh + Gl + Gll (three BF16 parts, ~2^-24), Out = Xh.Gh + Xl.Gh
//         + Xh.Gl + Xh.Gll accumulated in FP32 by kind::f16 MMAs, which run
//         at twice the TF32 rate;
//       - 3-term split-FP16: the split-TF32 scheme with FP16 parts (the same
//         11-bit significands, so the same ~2^-22 precision) on kind::f16
//         MMAs at twice the TF32 rate.  FP16's exponent range is met by
//         power-of-two scales: X is multiplied by 2^e before the split, with
//         e from the input's norm where a previous pass of the chain or the
//         caller (a capture flush's conversion) measured it, else 14
//         (amplitudes of modulus below ~3.99 fit), and each
//         matrix block by the 2^s its operand image records (|G| * 2^s <=
//         2^14); the epilogue multiplies by 2^-(e + s), all exact.  A
//         non-finite output (an amplitude out of range) sets error code 6;
//   * kApplyTC (setTensorCoreKernel(1)): the direct-load kernel, split-TF32.
//     Each thread owns one tile column and loads its 2D values straight from
//     global memory (the 32 lanes of a warp read 32 consecutive amplitudes),
//     X = Xh + Xl and Gr = Gh + Gl in TF32 parts, Out = Xh.Gh + Xl.Gh + Xh.Gl.
//
// Every wait is bounded: on timeout the CTA records an error code in a
// device flag, skips the rest of its tiles, frees its TMEM and returns; the
// host reads the flag after the pass.
#include "fused_plan.h"
#include "qg_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

namespace qg {

struct QuregF32;   // fused_f32.cu
float* f32re(QuregF32& q);
float* f32im(QuregF32& q);
int f32n(const QuregF32& q);

namespace {

constexpr int kTile = 128;              // groups per tile = MMA M = TMEM lanes
constexpr int kThreadsTC = 128;         // 4 warps: one TMEM lane quarter each
// every wait gives up after this much wall-clock time (read from %globaltimer)
constexpr unsigned long long kWaitLimitNs = 1000000000ull;   // 1 s

// Operand precision of kApplyTC2: 3-term split-TF32, 4-term split-BF16 or
// 3-term split-FP16.  Split-FP16 scales X by 2^kF16XExp before its split
// unless the input's norm is known (f16XExp).
constexpr int kPrecTF32 = 0, kPrecBF16 = 1, kPrecF16 = 2;
constexpr int kF16XExp = 14;
constexpr int kF16GMaxExp = 14;        // the largest |G| entry * 2^s stays <= 2^14

__device__ __forceinline__ unsigned long long globalTimerNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

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
    const unsigned long long t0 = globalTimerNs();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (globalTimerNs() - t0 > kWaitLimitNs) return false;
    }
}
__device__ __forceinline__ void bulkG2S(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(dst)),
                 "l"(src), "r"(bytes), "r"(smemAddr(bar))
                 : "memory");
}

// order this thread's generic-proxy accesses of shared memory before later
// async-proxy (bulk copy) accesses
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// one test of a phase (acquire); true when the phase with the parity completed
__device__ __forceinline__ bool mbarTest(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// 16-byte asynchronous copy global -> shared (no register staging, L1
// bypassed); completion is tracked per thread by commit groups
__device__ __forceinline__ void cpAsync16(float* dst, const float* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smemAddr(dst)), "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
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
__device__ __forceinline__ void tmemSt8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
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
// D[tmem] (+)= A[tmem] * B[smem desc], kind::f16: A and B both bf16 or both
// f16, as the instruction descriptor says (two per 32-bit TMEM column, the
// lower K index in the low half), D f32
__device__ __forceinline__ void mma16(uint32_t dT, uint32_t aT, uint64_t bDesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}" ::"r"(dT),
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

// instruction descriptor, kind::f16: D f32, A/B bf16, both K-major
__host__ __device__ constexpr uint32_t idescBF16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// instruction descriptor, kind::f16: D f32, A/B f16, both K-major
__host__ __device__ constexpr uint32_t idescF16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Split-FP16 of two consecutive K elements (already scaled into FP16's
// range): hi = both rounded to the nearest FP16 (packed, the first in the low
// half), lo = the exact remainders rounded to the nearest FP16.  x = hi + lo
// to ~2^-22 relative, unbiased, while lo is a normal FP16 number (|x| >= 2^-3);
// below that the measured precision is hi's alone, as if the MMA read
// subnormal parts as zero (f16XExp keeps the amplitudes above it).
__device__ __forceinline__ void splitF16x2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(x0, x1);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Split-BF16 of two consecutive K elements: hi = both rounded to the nearest
// bf16 (packed, the first in the low half), lo = the exact remainders rounded
// to the nearest bf16.  x = hi + lo to ~2^-17 relative, unbiased.
__device__ __forceinline__ void splitBF16x2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - __uint_as_float(hi << 16), x1 - __uint_as_float(hi & 0xFFFF0000u));
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// nearest TF32 value of a finite x (ties away from zero), as cvt.rna.tf32.f32,
// in two integer operations
__device__ __forceinline__ uint32_t tf32Bits(float x) { return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u; }

// Round to the nearest TF32 value (ties away from zero).  Both split parts are
// rounded to nearest: the MMA reads operands by dropping their low 13 bits,
// and a truncated split (hi = x with the low bits cleared) leaves lo with the
// sign of x, so the dropped bits of lo would bias every product toward zero
// (a norm loss of ~1e-6 per pass); with hi rounded to nearest lo takes both
// signs and is itself rounded to nearest, so the residual error is unbiased.
__device__ __forceinline__ uint32_t tf32RN(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void splitTF32(float x, uint32_t& hi, uint32_t& lo) {
    hi = tf32RN(x);
    lo = tf32RN(x - __uint_as_float(hi));
}


// Norm bookkeeping of one tensor-core pass (FP64 sums, accumulated with atomics):
//   out      sum |y|^2 of this pass's output;
//   in       sum |x|^2 of its input, or null when the host takes it from the
//            previous pass's output (nothing changed the state in between);
//   scaleSq  where this pass writes the square of the scale it applied;
//   corrIn, corrOut, corrScaleSq  the same three numbers of the previous
//            unitary tensor-core pass, or null.  Its norm factor
//            f = out / (in * scale^2) predicts this pass's own (the drift of
//            the tensor cores' accumulation is systematic);
//   corrTarget  when this pass continues a chain of unitary passes, the input
//            norm T of the chain's first pass, else null;
//   boundSq  sum |x|^2 of this pass's input when a previous tensor-core pass
//            of the chain measured it (its output) or the caller did (the
//            first pass), else null: it bounds every |x|, and split-FP16
//            takes the scale of X from it.
// The scale makes this pass's output norm T (chained: its input norm is the
// previous output, so scale^2 = T / (out * f)) or, unchained, its own input
// norm (scale^2 = 1 / f).  With a constant drift every output after the first
// is on target, instead of one drift factor behind.
struct NormLinks {
    double* out;
    double* in;
    double* scaleSq;
    const double* corrIn;
    const double* corrOut;
    const double* corrScaleSq;
    const double* corrTarget;
    const double* boundSq;
};
// the scale minus one (kept exact to FP32 relative precision)
__device__ __forceinline__ float driftCorrection(const NormLinks& nl) {
    if (!nl.corrIn || !nl.corrOut || !nl.corrScaleSq || !(*nl.corrOut > 0.0)) return 0.f;
    const double invF = *nl.corrIn * *nl.corrScaleSq / *nl.corrOut;
    const double s2 = nl.corrTarget ? *nl.corrTarget * invF / *nl.corrOut : invF;
    return (s2 > 0.0) ? (float)(sqrt(s2) - 1.0) : 0.f;
}
// written once per launch, by the calling thread when `writer`
__device__ __forceinline__ void recordScale(const NormLinks& nl, float sm1, bool writer) {
    if (nl.scaleSq && writer) *nl.scaleSq = (1.0 + (double)sm1) * (1.0 + (double)sm1);
}
// Split-FP16: the exponent e of X's scale 2^e.  With a bound B on every |x|,
// the largest e with B * 2^e <= 2^15, which keeps the lo parts of small
// amplitudes normal FP16 numbers (splitF16x2), else kF16XExp (|x| below
// ~3.99).
__device__ __forceinline__ int f16XExp(const NormLinks& nl) {
    if (!nl.boundSq) return kF16XExp;
    const double b = *nl.boundSq;
    if (!(b > 0.0) || !(b < 1.0e300)) return kF16XExp;
    int e = 0;
    frexp(sqrt(b), &e);                                  // sqrt(b) < 2^e
    return min(40, max(-40, 15 - e));
}

__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------ the kernel
// TMEM columns: [0, K) Xh, [K, 2K) Xl, [2K, 2K+N) Out, with K = N = 2D.
template <int KQ>
struct TCParams {
    uint64_t off[1 << KQ];      // amplitude offset of matrix index j
    int ins[KQ];                // ascending target positions
};

template <int KQ>
__global__ void __launch_bounds__(kThreadsTC, (KQ == 4 ? 4 : 1)) kApplyTC(float* __restrict__ re, float* __restrict__ im,
                                                       const float* __restrict__ gImage, uint64_t numTiles,
                                                       int* __restrict__ errFlag, const NormLinks nl,
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
    const float sm1 = driftCorrection(nl);               // input scaled by 1 + sm1
    recordScale(nl, sm1, blockIdx.x == 0 && threadIdx.x == 0);
    double normIn = 0.0, normOut = 0.0;
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
            float nrm = 0.f;
#pragma unroll
            for (int e = 0; e < CH; ++e) {
                nrm = fmaf(x[e], x[e], nrm);
                x[e] = fmaf(x[e], sm1, x[e]);
            }
            normIn += (double)nrm;
#pragma unroll
            for (int c0 = 0; c0 < CH; c0 += 16) {
                uint32_t hi[16], lo[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) splitTF32(x[c0 + e], hi[e], lo[e]);
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
        float nrmOut = 0.f;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            tmemLd16(tOut + laneBase + c0, v);
            tmemWaitLd();
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int r = c0 + e;
                const float y = __uint_as_float(v[e]);
                nrmOut = fmaf(y, y, nrmOut);
                if (r < D) re[base + p.off[r]] = y;
                else im[base + p.off[r - D]] = y;
            }
        }
        normOut += (double)nrmOut;
        fenceBefore();
        __syncthreads();
        fenceAfter();
    }
    normIn = warpSumD(normIn);
    normOut = warpSumD(normOut);
    if (lane == 0) {
        if (nl.in) atomicAdd(nl.in, normIn);
        if (nl.out) atomicAdd(nl.out, normOut);
    }
    __syncthreads();
    if (warp == 0) tmemDealloc(tbase, kCols);
}

// ------------------------------------------------------------ pipelined kernel
// Warp-specialised kernel used for every tensor-core pass by default (one
// persistent CTA per SM):
//   LG loader groups of 4 warps: 16-byte cp.async copies of their part of a
//              chunk into one of XST shared-memory row stages (up to three
//              chunks in flight per warp, no register staging); then each
//              thread reads its tile column back, splits it into BF16 parts
//              (two K entries per 32-bit word) and writes Xh/Xl to the TMEM
//              operand stage of the chunk with tcgen05.st;
//   EG epilogue groups of 4 warps: tcgen05.ld of a finished accumulator, the
//              drift-correction scale in FP32, column-order stores to shared
//              memory, 16-byte row-order reads, coalesced 16-byte stores;
//   1 warp:    TMEM allocation, the one-time TMA bulk copy of the three G
//              parts, and the MMA issue loop (one thread).
// TMEM holds four operand stages (64 columns each at k = 6) and two
// accumulators, so the loaders can run three chunks ahead of the MMAs while
// the epilogue drains the previous tile.  A tile is 128 groups (TMEM lanes)
// over the qubit set I = targets + the 7 lowest other qubits; I always
// contains qubits [0, r) with r >= 7, so the tile is made of contiguous runs
// of >= 128 amplitudes and every global access is coalesced whatever the
// targets are.  For k = 6 a tile's K = 128 is split into two chunks (real
// parts, imaginary parts of X).
//
// Warp-local staging.  Warp w of a role owns TMEM lanes (groups) 32w..32w+31,
// whose tile positions have the 6th and 7th column bits equal to w.  Each
// warp stages, and reads back, only those positions, in its own buffers, so
// the row <-> column transposition needs __syncwarp and no barrier across
// warps.  A warp's positions are split into two parts of at most 1024
// (k <= 5: the two planes; k = 6: the two halves by the top target bit, which
// the region index puts in its top bit).  Inside a part, index q lives at
// pad(q) = q + 4 (q >> 5) + 4 (q >> 8): every row of 32 positions starts on
// a 16-byte boundary, and pad is additive over disjoint bit sets, so
//   * a row access (4 positions q = 4 lane + 128 m) is the 16-byte word at
//     pad(4 lane) + pad(128 m): a per-thread base plus an immediate offset;
//   * a column access (group bits of the lane | bits of matrix index j) is
//     pad(lane bits) + pad(j bits): one add of a per-pass constant.
// When qubits 0 and 1 are both targets, the lanes' group bits all sit above
// bit 1 of the in-part index, and a scalar column access would be a 4-way bank
// conflict; the CV = 4 variant reads and writes entries j .. j + 3 of a column
// as one 16-byte word instead.
// The column accesses average 1.65 shared-memory wavefronts over the 6-qubit
// passes of a 30-qubit random circuit (1.71 with one float of padding per
// row, which breaks the 16-byte alignment).
constexpr int kTileBitsC = 7;

__host__ __device__ constexpr uint32_t padIdx(uint32_t q) { return q + 4 * (q >> 5) + 4 * (q >> 8); }

template <int KQ>
struct TC2Params {
    uint64_t scatterHigh[1 << KQ];        // address bits of the tile-position bits above the low run
    uint64_t warpOff[4][1 << (KQ - 2)];   // amplitude offset of region index 128 m of warp w
    uint64_t laneOff[32];                 // amplitude offset of region index 4 lane
    uint32_t colLane[32];                 // pad(in-part index of the group bits of lane l)
    uint32_t colJ[1 << KQ];               // pad(in-part index of the position bits of matrix index j)
    int insI[KQ + kTileBitsC + 3];        // ascending qubits of I and of the controls (zero in a tile base)
    int numIns;                           // entries of insI
    int runBits;                          // I contains qubits [0, runBits)
    uint64_t outMask;                     // the qubits outside I (where tile index bits go)
    uint64_t gridStep;                    // the tile base offset of ctasPerInst tiles
    // Batches of states (one launch for the same pass on several registers):
    // CTA b runs tiles b % ctasPerInst, + ctasPerInst, ... of state
    // b / ctasPerInst, which starts instStride floats after the previous one
    // and has its own operand image, imageStride floats after the previous
    // one.  A single register: ctasPerInst = gridDim.x, the strides 0.
    uint32_t ctasPerInst;
    uint64_t instStride;
    uint64_t imageStride;
    // Controlled passes: 2^ctrlBits matrices, one per value c of the control
    // qubits (outside I and outside the tile bases).  The CTAs of a register
    // come in 2^ctrlBits groups of ctasPerInst; group c runs the amplitudes
    // whose control bits are c, ctrlOff[c] amplitudes into the register (c
    // deposited into the control qubits), with operand image block c,
    // ctrlImageStride floats after block c - 1.
    uint32_t ctrlBits;
    uint64_t ctrlOff[8];
    uint64_t ctrlImageStride;
};

// Layout of kApplyTC2<KQ, LG, EG, LS, PR>, used by the kernel and its
// launcher.  Shared memory: the parts of G (split-TF32: Gh, Gl in FP32 words,
// G to ~2^-22; split-BF16: Gh, Gl, Gll in BF16, G to ~2^-24; split-FP16: Gh,
// Gl in FP16, G to ~2^-22), the loader row
// stages and the epilogue buffers.  At k = 6, G is the compact real form
// [-Im G; Re G; Im G] (192 rows x 64 K).  The B operand of the K-chunk of the
// real parts of X is rows 64..191 ([Re; Im]).  That of the imaginary parts is
// rows 0..127 ([-Im; Re]).  Loader row buffers: XST stages per loader warp
// (three at k = 4, two at k >= 5).  TMEM: NST operand stages (Xh then Xl; one
// TF32 or two 16-bit values per column), then two accumulators of N columns.
template <int KQ, int LG, int EG, int LS, int PR>
struct TC2Shape {
    static constexpr int D = 1 << KQ, K = 2 * D, N = 2 * D;
    static constexpr int TILE = 1 << (KQ + kTileBitsC);       // amplitudes per plane per tile
    static constexpr int ESZ = (PR != kPrecTF32) ? 2 : 4;     // bytes per operand entry
    // K chunks per tile: chunks of <= 64 (BF16, FP16) or <= 32 (TF32) K entries,
    // so that four operand stages fit beside the two accumulators
    static constexpr int NCH = (PR != kPrecTF32) ? ((KQ == 6) ? 2 : 1) : ((KQ == 6) ? 4 : (KQ == 5) ? 2 : 1);
    static constexpr int KC = K / NCH;                        // K entries per chunk
    // Parts: the positions a warp stages at once (<= 1024).  k <= 5: the two
    // planes; k = 6: the halves of a plane by the top target bit.  A chunk is
    // one part (a plane at k = 5 in TF32; a plane half at k = 6 in TF32) or
    // two (both planes at k <= 5; both halves of a plane at k = 6 in BF16 or FP16).
    static constexpr int PART = (KQ == 6) ? TILE / 8 : TILE / 4;   // positions per warp per part (<= 1024)
    static constexpr int PPC = ((KQ == 6) ? (NCH == 2) : (NCH == 1)) ? 2 : 1;   // parts per chunk
    static constexpr int JPP = KC / PPC;                      // K entries (matrix indices) per part
    // SPLIT: the loader groups split every chunk, group g taking part g;
    // otherwise each group takes whole chunks, the groups alternating
    static constexpr bool SPLIT = (LS == 2 && PPC == 2);
    static constexpr int PPG = SPLIT ? 1 : PPC;               // parts per loader group per chunk
    static constexpr int R = (int)((padIdx(PART - 1) + 1 + 3) & ~3u);   // floats per part buffer
    static constexpr int NST = 4;                             // TMEM operand stages
    static constexpr uint32_t STAGE_COLS = (uint32_t)(2 * KC * ESZ / 4);   // Xh then Xl
    static constexpr int NGP = (PR == kPrecBF16) ? 3 : 2;     // parts of G
    static constexpr uint32_t GE = (KQ == 6) ? 3u * D * D : (uint32_t)(N * K);   // entries of each G part
    static constexpr uint32_t GW = GE * ESZ / 4;              // ... in 32-bit words
    static constexpr uint32_t GSBO = (uint32_t)(((KQ == 6) ? D : K) * ESZ / 16) * 128u;    // B descriptor stride
    static constexpr size_t fixedFloats = (size_t)NGP * GW + (size_t)EG * 4 * R;
    static constexpr size_t stageFloats = (size_t)LG * 4 * PPG * R;
    static constexpr bool fits(int st) { return (fixedFloats + (size_t)st * stageFloats) * 4 + 2048 <= 227 * 1024; }
    // loader row stages: three where they fit at k = 4, two at k >= 5.  Measured
    // on the 30-qubit circuit: at k = 6 (split-BF16) three stages took 282 ms
    // against 267 with two; at k = 5, 360 / 364 ms against 358 / 364; at
    // k = 4 two stages took 578 / 514 ms against 509 / 500 with three; one
    // stage is 15-20 % slower everywhere.
    static constexpr int XST = (KQ <= 4 && fits(3)) ? 3 : (fits(2) ? 2 : 1);
    static constexpr size_t smemBytes = (fixedFloats + (size_t)XST * stageFloats) * 4;
    static_assert(NST * STAGE_COLS + 2 * N <= 512, "TMEM");
    // plane, plane half (k = 6) and first matrix index of part pt of chunk ch
    __host__ __device__ static constexpr int plane(int ch, int pt) {
        return (KQ == 6) ? ((NCH == 2) ? ch : ch >> 1) : ((NCH == 1) ? pt : ch);
    }
    __host__ __device__ static constexpr int half(int ch, int pt) { return (NCH == 4) ? (ch & 1) : pt; }
};

__device__ __forceinline__ void mbarArrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}
// bounded wait that also gives up when another role has aborted
__device__ __forceinline__ bool mbarWaitOrAbort(uint64_t* bar, uint32_t parity, volatile int* abortF) {
    const uint32_t a = smemAddr(bar);
    const unsigned long long t0 = globalTimerNs();
    for (unsigned i = 1;; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 15) == 0 && (*abortF || globalTimerNs() - t0 > kWaitLimitNs)) return false;
    }
}
// the same wait for a whole warp: lane 0 polls, the result goes to every lane
__device__ __forceinline__ bool warpWaitOrAbort(uint64_t* bar, uint32_t parity, volatile int* abortF, int lane) {
    int ok = 1;
    if (lane == 0) ok = mbarWaitOrAbort(bar, parity, abortF) ? 1 : 0;
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// amplitude offset of the first amplitude of a tile: the tile index bits go,
// in order, to the qubits outside I and outside the control qubits (host and
// device: the host check of the addressing walks tiles with it)
template <int KQ>
__host__ __device__ __forceinline__ uint64_t tileBase(const TC2Params<KQ>& p, uint64_t tile) {
    uint64_t tb = tile << p.runBits;
#ifdef __CUDA_ARCH__
#pragma unroll 1
#endif
    for (int b = p.runBits; b < p.numIns; ++b) {
        const int s = p.insI[b];
        tb = ((tb >> s) << (s + 1)) | (tb & ((1ull << s) - 1ull));
    }
    return tb;
}
// Tile bases of one role's increasing tile sequence (tiles differ by
// multiples of ctasPerInst).  The base is the tile index deposited into
// outMask, and deposits add by masked addition:
// base(t + ctasPerInst) = ((base(t) | ~outMask) + gridStep) & outMask.
template <int KQ>
struct TileWalker {
    uint64_t tile = ~0ull, base = 0;
    __host__ __device__ __forceinline__ uint64_t at(const TC2Params<KQ>& p, uint64_t t) {
        if (tile == ~0ull || t < tile) {
            base = tileBase(p, t);
            tile = t;
        }
        while (tile < t) {
            base = ((base | ~p.outMask) + p.gridStep) & p.outMask;
            tile += p.ctasPerInst;
        }
        return base;
    }
};

// CV = 4: the targets include qubits 0 and 1, and columns are read and
// written as 16-byte words (see colWords4).
// ST: how the loaders stage a chunk.  0: 16-byte cp.async per lane (commit
// groups); 1: TMA bulk copies, one 128-byte row (32 positions, contiguous in
// global memory and in the padded shared layout) per lane and part,
// completing on one mbarrier per warp and row stage.
template <int KQ, int LG, int EG, int LS, int PR, int CV, int ST>
__global__ void __launch_bounds__((4 * (LG + EG) + 1) * 32, 1) kApplyTC2(float* __restrict__ re, float* __restrict__ im,
                                                                  const float* __restrict__ gImage, uint64_t numTiles,
                                                                  int* __restrict__ errFlag, const NormLinks nl,
                                                                  const __grid_constant__ TC2Params<KQ> p) {
    using S = TC2Shape<KQ, LG, EG, LS, PR>;
    constexpr bool BF = (PR == kPrecBF16), F16 = (PR == kPrecF16), H16 = BF || F16;
    // split-FP16: X's scale 2^xe before the split (the epilogue undoes it)
    const int xe = F16 ? f16XExp(nl) : 0;
    const float kXs = __int_as_float((127 + xe) << 23);
    // this CTA's register of a batch and control value, and its place among
    // the CTAs of that pair
    const uint32_t cta = blockIdx.x % p.ctasPerInst, ncta = p.ctasPerInst;
    {
        const uint64_t u = blockIdx.x / p.ctasPerInst;
        const uint64_t inst = u >> p.ctrlBits, cv = u & ((1u << p.ctrlBits) - 1u);
        re += inst * p.instStride + p.ctrlOff[cv];
        im += inst * p.instStride + p.ctrlOff[cv];
        gImage += inst * p.imageStride + cv * p.ctrlImageStride;
    }
    constexpr int D = S::D, N = S::N;
    constexpr int NCH = S::NCH, KC = S::KC, PART = S::PART, R = S::R, PPG = S::PPG, XST = S::XST, NST = S::NST;
    constexpr uint32_t kGW = S::GW;
    constexpr int V4P = PART / 128;                      // 128-position blocks per part
    constexpr int JP = S::JPP;                           // matrix indices per part
    constexpr int EPARTS = (KQ == 6) ? 4 : 2;            // epilogue parts per tile (plane x half)
    constexpr uint32_t kStageCols = S::STAGE_COLS;       // Xh, then Xl at + kStageCols / 2
    constexpr uint32_t kDCol0 = NST * kStageCols;
    constexpr uint32_t kUsed = kDCol0 + 2 * N;
    constexpr uint32_t kCols = kUsed <= 64 ? 64 : (kUsed <= 128 ? 128 : (kUsed <= 256 ? 256 : 512));
    static_assert(kUsed <= 512, "TMEM");
    constexpr uint32_t kLBO = 128;
    constexpr uint32_t idesc = BF ? idescBF16(kTile, N) : F16 ? idescF16(kTile, N) : idescTF32(kTile, N);
    constexpr int kEpiWarp0 = 4 * LG, kMmaWarp = 4 * (LG + EG);
    // loader groups split every chunk (S::SPLIT) or take alternate chunks
    static_assert(LS == 1 || LG == 2, "part-split loading needs two loader groups");

    extern __shared__ __align__(1024) uint8_t smem[];
    uint32_t* gh = reinterpret_cast<uint32_t*>(smem);
    uint32_t* gl = gh + kGW;
    uint32_t* gll = gl + kGW;                            // (split-BF16 only)
    float* xs = reinterpret_cast<float*>(gh + S::NGP * kGW);   // [loader group][warp][stage][part][R]
    float* es = xs + (size_t)XST * LG * 4 * PPG * R;     // [epilogue group][warp][R]
    __shared__ __align__(8) uint64_t barG, fullB[NST], emptyB[NST], dFullB[2], dEmptyB[2];
    constexpr int kStageBars = ST == 1 ? 4 * LG * XST : 1;
    __shared__ __align__(8) uint64_t stageB[kStageBars];   // bulk staging: [loader warp][row stage]
    __shared__ uint32_t tmemBase;
    __shared__ volatile int abortF;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == kMmaWarp) {
        if (lane == 0) {
            abortF = 0;
            mbarInit(&barG, 1);
            for (int b = 0; b < NST; ++b) {
                mbarInit(&fullB[b], 128 * (S::SPLIT ? LG : 1));
                mbarInit(&emptyB[b], 1);
            }
            for (int b = 0; b < 2; ++b) {
                mbarInit(&dFullB[b], 1);
                mbarInit(&dEmptyB[b], 128);
            }
            if (ST == 1)
                for (int b = 0; b < kStageBars; ++b) mbarInit(&stageB[b], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        tmemAlloc(&tmemBase, kCols);
    }
    fenceBefore();
    __syncthreads();
    fenceAfter();
    const uint32_t tmem = tmemBase;
    const int rw = warp & 3;                             // warp within its role = TMEM lane quarter
    const uint32_t laneSel = (uint32_t)(32 * rw) << 16;
    const uint32_t rowBase = padIdx(4u * lane);

    if (warp < kEpiWarp0) {
        // ------------------------------------------------ loaders
        const int g = warp >> 2;
        const uint64_t laneA = p.laneOff[lane];
        const uint32_t colBase = p.colLane[lane];
        // this CTA's chunks, in order: chunk s = (tile cta + (s / NCH) * ncta, K chunk s % NCH);
        // split: every s, part g; otherwise group g takes s = g, g + LG, ...
        const int p0 = S::SPLIT ? g : 0;
        const uint32_t s0 = S::SPLIT ? 0u : (uint32_t)g, sStep = S::SPLIT ? 1u : (uint32_t)LG;
        const uint32_t nMy = cta < numTiles ? (uint32_t)((numTiles - 1 - cta) / ncta + 1) * NCH : 0u;
        const uint32_t nMine = nMy > s0 ? (nMy - s0 + sStep - 1) / sStep : 0u;     // chunks of this group
        double normIn = 0.0;
        const bool measure = nl.in != nullptr;             // input norm wanted (uniform)
        float* const wbuf = xs + (size_t)(g * 4 + rw) * XST * PPG * R;             // this warp's stages
        // Copy this group's parts of chunk sc into a stage (a k = 6 part is a
        // plane half: region indices < 1024 or >= 1024).  Region index bits
        // 0, 1 are qubits 0, 1, so positions q = 4 lane + 128 m .. + 3 are four
        // consecutive amplitudes: one 16-byte copy to pad(q); a warp's copy
        // reads four 128-byte lines.
        TileWalker<KQ> walk;
        // bulk staging: lane l < ROWS copies row l of each part, region
        // indices 32 l .. 32 l + 31 (qubits 0..4 are region bits 0..4, so a
        // row is 128 contiguous bytes in global memory; in the padded layout
        // it starts at pad(32 l), a 16-byte boundary)
        constexpr int ROWS = PART / 32;
        static_assert(ROWS <= 32 && ROWS / 4 <= V4P, "one row per lane");
        const uint64_t rowA = p.laneOff[8 * (lane & 3)];
        uint64_t* const wbar = stageB + (ST == 1 ? (g * 4 + rw) * XST : 0);
        auto issue = [&](uint32_t sc, float* buf, int stage) {
            const uint64_t tile = cta + (uint64_t)(sc / NCH) * ncta;
            const int ch = sc % NCH;
            if constexpr (ST == 1) {
                const uint64_t tb = walk.at(p, tile) + rowA;
                if (lane == 0) mbarExpectTx(&wbar[stage], (uint32_t)(PPG * ROWS * 128));
                if (lane < ROWS) {
#pragma unroll
                    for (int pp = 0; pp < PPG; ++pp) {
                        const int pt = p0 + pp;
                        const int m = ((KQ == 6) ? V4P * S::half(ch, pt) : 0) + (lane >> 2);
                        const float* const src = (S::plane(ch, pt) == 0 ? re : im) + tb + p.warpOff[rw][m];
                        bulkG2S(buf + pp * R + padIdx(32u * lane), src, 128u, &wbar[stage]);
                    }
                }
            } else {
                const uint64_t tb = walk.at(p, tile) + laneA;
#pragma unroll
                for (int pp = 0; pp < PPG; ++pp) {
                    const int pt = p0 + pp;
                    const float* const src = (S::plane(ch, pt) == 0 ? re : im) + tb;
                    float* const dst = buf + pp * R + rowBase;
#pragma unroll
                    for (int mm = 0; mm < V4P; ++mm) {
                        const int m = ((KQ == 6) ? V4P * S::half(ch, pt) : 0) + mm;
                        cpAsync16(dst + padIdx(128u * mm), src + p.warpOff[rw][m]);
                    }
                }
            }
        };
        // XST chunks in flight ahead of the split (cp.async: one commit group each)
        for (int st = 0; st < XST; ++st) {
            if ((uint32_t)st < nMine) issue(s0 + st * sStep, wbuf + (size_t)st * PPG * R, st);
            if (ST == 0) cpAsyncCommit();
        }
        bool ok = true;
        uint32_t stopAt = nMine;                             // bulk staging: first chunk not waited for
        for (uint32_t idx = 0; idx < nMine; ++idx) {
            const uint32_t sq = s0 + idx * sStep;
            // TMEM stage b of chunk sq; its previous use was chunk sq - NST
            const int b = (int)(sq % NST);
            const uint32_t u = sq / NST;
            float* const xr = wbuf + (size_t)(idx % XST) * PPG * R;
            if (u > 0 && !warpWaitOrAbort(&emptyB[b], (u - 1) & 1, &abortF, lane)) {
                ok = false;
                stopAt = idx;
                break;
            }
            if constexpr (ST == 1) {
                const uint32_t par = (idx / XST) & 1u;
                if (!warpWaitOrAbort(&wbar[idx % XST], par, &abortF, lane)) {
                    ok = false;
                    stopAt = idx;
                    break;
                }
                mbarTest(&wbar[idx % XST], par);                 // every lane acquires the landed rows
            } else {
                cpAsyncWait<XST - 1>();                          // this lane's copies of the chunk landed
                __syncwarp();                                    // ... and every lane's
            }
            // this group's K entries of the stage: [p0 JP, (p0 + PPG) JP); EPW per column
            constexpr int EPW = H16 ? 2 : 1;
            const uint32_t aH = tmem + laneSel + b * kStageCols + p0 * JP / EPW;
            const int chq = (int)(sq % NCH);
            const float* const cb = xr + colBase;
            // split the chunk into TMEM; the sum of squares of what the warp
            // reads (the pass's input norm) only when this pass measures it
            auto splitChunk = [&](auto withNorm) -> float {
                constexpr bool WN = decltype(withNorm)::value;
                float nrm = 0.f;
#pragma unroll
                for (int c0 = 0; c0 < PPG * JP; c0 += 8 * EPW) {
                    uint32_t hi[8], lo[8];
                    if constexpr (CV == 4) {
                        // targets on qubits 0, 1: a column's entries j .. j + 3 are one
                        // 16-byte word (scalar reads would be a 4-way bank conflict);
                        // four consecutive local entries stay in one part
                        float xv[8 * EPW];
#pragma unroll
                        for (int v = 0; v < 2 * EPW; ++v) {
                            const int cl = c0 + 4 * v;
                            const int pl = cl / JP;
                            const int j = (KQ == 6) ? 32 * S::half(chq, p0 + pl) + cl % JP : cl % JP;
                            const float4 f = *reinterpret_cast<const float4*>(cb + pl * R + p.colJ[j]);
                            xv[4 * v] = f.x;
                            xv[4 * v + 1] = f.y;
                            xv[4 * v + 2] = f.z;
                            xv[4 * v + 3] = f.w;
                        }
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
#pragma unroll
                            for (int h = 0; h < EPW; ++h)
                                if constexpr (WN) nrm = fmaf(xv[EPW * e + h], xv[EPW * e + h], nrm);
                            if constexpr (BF) {
                                splitBF16x2(xv[2 * e], xv[2 * e + 1], hi[e], lo[e]);
                            } else if constexpr (F16) {
                                splitF16x2(xv[2 * e] * kXs, xv[2 * e + 1] * kXs, hi[e], lo[e]);
                            } else {
                                hi[e] = tf32Bits(xv[e]);
                                lo[e] = __float_as_uint(xv[e] - __uint_as_float(hi[e]));
                            }
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            float x[EPW];
#pragma unroll
                            for (int h = 0; h < EPW; ++h) {
                                const int cl = c0 + EPW * e + h;     // local entry: buffer part cl / JP
                                const int pl = cl / JP;
                                const int j = (KQ == 6) ? 32 * S::half(chq, p0 + pl) + cl % JP : cl % JP;
                                x[h] = (cb + pl * R)[p.colJ[j]];
                                if constexpr (WN) nrm = fmaf(x[h], x[h], nrm);   // the warp reads every element once
                            }
                            if constexpr (BF) {
                                splitBF16x2(x[0], x[EPW - 1], hi[e], lo[e]);
                            } else if constexpr (F16) {
                                splitF16x2(x[0] * kXs, x[EPW - 1] * kXs, hi[e], lo[e]);
                            } else {
                                // hi = x rounded to TF32; lo = x - hi (exact), which the MMA
                                // reads as its leading TF32 bits; lo takes both signs, so
                                // that truncation is unbiased
                                hi[e] = tf32Bits(x[0]);
                                lo[e] = __float_as_uint(x[0] - __uint_as_float(hi[e]));
                            }
                        }
                    }
                    tmemSt8(aH + c0 / EPW, hi);
                    tmemSt8(aH + kStageCols / 2 + c0 / EPW, lo);
                }
                return nrm;
            };
            const float nrm = measure ? splitChunk(std::true_type{}) : splitChunk(std::false_type{});
            if (measure) normIn += (double)nrm;
            tmemWaitSt();
            fenceBefore();
            mbarArrive(&fullB[b]);
            if (ST == 1) fenceProxyAsync();                  // column reads before the bulk refill
            __syncwarp();                                    // column reads done before the stage is refilled
            if (idx + XST < nMine) issue(sq + XST * sStep, xr, (int)(idx % XST));
            if (ST == 0) cpAsyncCommit();
        }
        if constexpr (ST == 1) {
            // no copy in flight when the warp leaves: chunks stopAt .. were issued
            // and not waited for (bounded waits)
            const uint32_t end = nMine < stopAt + XST ? nMine : stopAt + XST;
            for (uint32_t c = stopAt; c < end; ++c)
                if (lane == 0) mbarWait(&wbar[c % XST], (c / XST) & 1u);
            __syncwarp();
        } else {
            cpAsyncWait<0>();                                // no copy in flight when the warp leaves
        }
        if (!ok) {
            if (lane == 0) atomicExch(errFlag, 3);
            abortF = 1;
        }
        normIn = warpSumD(normIn);
        if (lane == 0 && measure) atomicAdd(nl.in, normIn);
    } else if (warp < kMmaWarp) {
        // ------------------------------------------------ epilogue
        // epilogue group eg drains accumulator eg, i.e. tiles tl with tl % EG == eg
        const int et = threadIdx.x - 32 * kEpiWarp0;
        const int eg = et >> 7;
        const uint64_t laneA = p.laneOff[lane];
        const uint32_t colBase = p.colLane[lane];
        float* const er = es + (size_t)(eg * 4 + rw) * R;
        // the drift correction: every output is scaled by 1 + sm1 in FP32
        // (split-BF16 parts of a rescaled G would carry the scale only to their
        // ~2^-17 precision, far coarser than the drift)
        bool ok = true;
        const float sm1 = driftCorrection(nl);
        recordScale(nl, sm1, blockIdx.x == 0 && et == 0);
        // split-FP16: 2^-(xe + s), s the scale of this CTA's matrix block (its
        // image records 2^-(14 + s) after the two parts)
        const float unscale = F16 ? __ldg(gImage + 2 * kGW) * __int_as_float((127 + kF16XExp - xe) << 23) : 1.f;
        uint32_t tl = eg;
        double normOut = 0.0;
        TileWalker<KQ> walk;
        for (uint64_t tile = cta + (uint64_t)eg * ncta; tile < numTiles && ok;
             tile += (uint64_t)EG * ncta, tl += EG) {
            const uint64_t tb = walk.at(p, tile) + laneA;
            const int bd = tl & 1;
            if (!warpWaitOrAbort(&dFullB[bd], (tl >> 1) & 1, &abortF, lane)) {
                ok = false;
                break;
            }
            fenceAfter();
            const uint32_t dA = tmem + laneSel + kDCol0 + bd * N;
            float nrmTile = 0.f;
            float* const cb = er + colBase;
            const float* const rb = er + rowBase;
            // (rolled at k = 6, whose four unrolled parts would not fit the registers)
#pragma unroll(KQ == 6 ? 1 : EPARTS)
            for (int ep = 0; ep < EPARTS; ++ep) {
                // part ep: plane pl (output rows r = pl * D + j), matrix indices j = h * 32 + jj
                const int pl = (KQ == 6) ? ep >> 1 : ep;
                const int h = (KQ == 6) ? ep & 1 : 0;
                const int c0 = pl * D + h * 32;
                uint32_t va[16], vb[16];
                tmemLd16(dA + c0, va);
                if (JP == 32) tmemLd16(dA + c0 + 16, vb);
                tmemWaitLd();
                if (ep == EPARTS - 1) {                              // accumulator drained
                    fenceBefore();
                    mbarArrive(&dEmptyB[bd]);
                }
                if constexpr (CV == 4) {
                    // targets on qubits 0, 1: 16-byte column words
#pragma unroll
                    for (int e = 0; e < JP; ++e) {
                        uint32_t& w = e < 16 ? va[e] : vb[e - 16];
                        const float y0 = F16 ? __uint_as_float(w) * unscale : __uint_as_float(w);
                        const float y = fmaf(y0, sm1, y0);
                        nrmTile = fmaf(y, y, nrmTile);
                        w = __float_as_uint(y);
                    }
                    auto yAt = [&](int e) { return __uint_as_float(e < 16 ? va[e] : vb[e - 16]); };
#pragma unroll
                    for (int e = 0; e < JP; e += 4)
                        *reinterpret_cast<float4*>(cb + p.colJ[h * 32 + e]) = make_float4(yAt(e), yAt(e + 1), yAt(e + 2), yAt(e + 3));
                } else {
#pragma unroll
                    for (int e = 0; e < JP; ++e) {
                        const float y0 = F16 ? __uint_as_float(e < 16 ? va[e] : vb[e - 16]) * unscale
                                             : __uint_as_float(e < 16 ? va[e] : vb[e - 16]);
                        const float y = fmaf(y0, sm1, y0);
                        nrmTile = fmaf(y, y, nrmTile);
                        cb[p.colJ[h * 32 + e]] = y;
                    }
                }
                __syncwarp();
                float* const dstPlane = (pl == 0 ? re : im) + tb;
#pragma unroll
                for (int mm = 0; mm < V4P; ++mm) {
                    const int m = (KQ == 6) ? V4P * h + mm : mm;
                    const float4 w = *reinterpret_cast<const float4*>(rb + padIdx(128u * mm));
                    __stcs(reinterpret_cast<float4*>(dstPlane + p.warpOff[rw][m]), w);
                }
                __syncwarp();
            }
            normOut += (double)nrmTile;
        }
        if (!ok) {
            if (lane == 0) atomicExch(errFlag, 4);
            abortF = 1;
        }
        // split-FP16: an input beyond FP16's range after scaling gave a
        // non-finite output
        if (F16 && !(normOut <= 1.0e300)) atomicExch(errFlag, 6);
        normOut = warpSumD(normOut);
        if (lane == 0 && nl.out) atomicAdd(nl.out, normOut);
    } else if (lane == 0) {
        // ------------------------------------------------ TMA of G, then MMAs
        mbarExpectTx(&barG, S::NGP * kGW * 4);
        bulkG2S(gh, gImage, kGW * 4, &barG);
        bulkG2S(gl, gImage + kGW, kGW * 4, &barG);
        if (BF) bulkG2S(gll, gImage + 2 * kGW, kGW * 4, &barG);
        bool ok = mbarWaitOrAbort(&barG, 0, &abortF);
        if (!ok) mbarWaitOrAbort(&barG, 0, &abortF);                // once more for the copies in flight
        const uint32_t ghA = smemAddr(gh), glA = smemAddr(gl), gllA = smemAddr(gll);
        uint32_t sq = 0, tl = 0;
        for (uint64_t tile = cta; tile < numTiles && ok; tile += ncta, ++tl) {
            const int bd = tl & 1;
            if (tl >= 2 && !mbarWaitOrAbort(&dEmptyB[bd], ((tl >> 1) - 1) & 1, &abortF)) {
                ok = false;
                break;
            }
            fenceAfter();
            const uint32_t dT = tmem + kDCol0 + bd * N;
            for (int ch = 0; ch < NCH; ++ch, ++sq) {
                const int b = (int)(sq % NST);
                if (!mbarWaitOrAbort(&fullB[b], (sq / NST) & 1, &abortF)) {
                    ok = false;
                    break;
                }
                fenceAfter();
                const uint32_t aH = tmem + b * kStageCols, aL = aH + kStageCols / 2;
                // chunk ch's B: k <= 5 the rows of G's real form and K entries
                // [ch KC, (ch + 1) KC); k = 6 rows 64..191 of the compact form for
                // the real parts of X, rows 0..127 for the imaginary parts, and
                // the chunk's plane half of the 64 K entries.  Each K step (8 TF32
                // or 16 BF16 entries) reads the next 8 TMEM columns of A and the
                // next 256 bytes of B: the descriptor's start field (address >> 4)
                // advances by 16 per step
                const uint32_t kEnt = (KQ == 6) ? 32u * (uint32_t)S::half(ch, 0) * (NCH == 4) : (uint32_t)(ch * KC);
                const uint32_t gOff = ((KQ == 6 && S::plane(ch, 0) == 0) ? 8u * S::GSBO : 0u) + kEnt * S::ESZ / 16u * 128u;
                const uint64_t dH = smemDesc(ghA + gOff, kLBO, S::GSBO);
                const uint64_t dL = smemDesc(glA + gOff, kLBO, S::GSBO);
                const uint64_t dLL = smemDesc(gllA + gOff, kLBO, S::GSBO);
                if constexpr (BF) {
                    // Xh.Gh + Xl.Gh + Xh.Gl + Xh.Gll: G to ~2^-24 (a ~2^-17 G
                    // would change the norm by up to ~1e-6 per pass, depending
                    // on the state); the dropped Xl.Gl is unbiased
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks)
                        mma16(dT, aH + 8 * ks, dH + 16u * ks, idesc, (ch | ks) != 0);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) mma16(dT, aL + 8 * ks, dH + 16u * ks, idesc, 1);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) mma16(dT, aH + 8 * ks, dL + 16u * ks, idesc, 1);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) mma16(dT, aH + 8 * ks, dLL + 16u * ks, idesc, 1);
                } else if constexpr (F16) {
                    // Xh.Gh + Xl.Gh + Xh.Gl (K = 16 per MMA), as split-TF32
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks)
                        mma16(dT, aH + 8 * ks, dH + 16u * ks, idesc, (ch | ks) != 0);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) mma16(dT, aL + 8 * ks, dH + 16u * ks, idesc, 1);
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) mma16(dT, aH + 8 * ks, dL + 16u * ks, idesc, 1);
                } else {
                    // Xh.Gh + Xl.Gh + Xh.Gl (K = 8 per MMA)
#pragma unroll
                    for (int ks = 0; ks < KC / 8; ++ks)
                        mmaTF32(dT, aH + 8 * ks, dH + 16u * ks, idesc, (ch | ks) != 0);
#pragma unroll
                    for (int ks = 0; ks < KC / 8; ++ks) mmaTF32(dT, aL + 8 * ks, dH + 16u * ks, idesc, 1);
#pragma unroll
                    for (int ks = 0; ks < KC / 8; ++ks) mmaTF32(dT, aH + 8 * ks, dL + 16u * ks, idesc, 1);
                }
                mmaCommit(&emptyB[b]);
            }
            if (!ok) break;
            mmaCommit(&dFullB[bd]);
        }
        if (!ok) {
            atomicExch(errFlag, 5);
            abortF = 1;
        }
        // drain: wait (bounded) for the last accumulator to finish before TMEM is freed
        if (tl > 0) mbarWaitOrAbort(&dFullB[(tl - 1) & 1], ((tl - 1) >> 1) & 1, &abortF);
    }
    fenceBefore();
    __syncthreads();
    fenceAfter();
    if (warp == kMmaWarp) tmemDealloc(tmem, kCols);
}

// ------------------------------------------------------------ host side
struct DevicePlan {
    std::vector<float*> images;      // per pass: its operand images (or nullptr), inside imageBuf
    float* imageBuf = nullptr;
    int* errFlag = nullptr;
    // per pass: (sum |x|^2 of its input, sum |y|^2 of its output, square of
    // the scale it applied) in FP64, written by the tensor-core kernels.  The
    // next tensor-core pass scales by sqrt(in * scale^2 / out) of the previous
    // one, which removes the norm drift of the tensor cores' FP32 accumulation.
    double* norms = nullptr;
    // per pass: where its input norm lives (its own slot, or the output slot
    // of the previous tensor-core pass when nothing changed the state between)
    std::vector<const double*> inNorm;
    // per pass: the input norm of the first pass of its chain of unitary passes
    std::vector<const double*> target;
    int lastTC = -1;        // last tensor-core pass applied (its drift is corrected next)
    bool chain = false;     // the state is still lastTC's output up to unitary SIMT passes
    // sum |x|^2 of the state this range started from, when the caller measured
    // it (device; until a non-unitary SIMT pass): the bound of the first
    // tensor-core pass's split-FP16 scale
    const double* entryBound = nullptr;
    // per pass: 1 if its matrix is unitary to 1e-10.  Only the drift of a
    // unitary pass is corrected; a non-unitary pass changes the norm on purpose.
    std::vector<char> unitary;
    int parts = 0;          // the image parts built (kPart*)
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

// nearest TF32 value of x (ties away from zero), as cvt.rna.tf32.f32
float hostTf32RN(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;   // finite values
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}

// nearest bf16 (ties to even) of a finite x, and the value of a bf16
uint16_t hostBF16RN(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
float bf16Value(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}

// Nearest IEEE binary16 value (ties to even) of a double, rounded once:
// below 2^-14 on the subnormal grid of 2^-24, else to 11 significant bits;
// beyond the largest finite value (65504) ties and above give infinity.
uint16_t hostF16RN(double v) {
    const uint16_t sign = std::signbit(v) ? 0x8000u : 0u;
    const double a = std::fabs(v);
    if (std::isnan(v)) return 0x7E00u;
    if (a >= 65520.0) return sign | 0x7C00u;
    int e = 0;
    std::frexp(a, &e);                                   // a in [2^(e-1), 2^e)
    const int qe = std::max(e - 11, -24);                // exponent of the quantum
    const double m = std::nearbyint(std::ldexp(a, -qe));   // a / quantum, exact, then rounded (ties even)
    const double r = std::ldexp(m, qe);
    if (r == 0.0) return sign;
    if (r < 0x1p-14) return sign | (uint16_t)m;          // subnormal: the count of 2^-24
    int re = 0;
    std::frexp(r, &re);                                  // r in [2^(re-1), 2^re)
    const int E = re - 1;                                // r = 2^E (1 + f / 1024)
    const uint32_t f = (uint32_t)(std::ldexp(r, 10 - E) - 1024.0);
    return sign | (uint16_t)(((E + 15) << 10) | f);
}
double f16Value(uint16_t h) {
    const int ex = (h >> 10) & 31, man = h & 1023;
    const double s = (h & 0x8000u) ? -1.0 : 1.0;
    if (ex == 31) return man ? std::nan("") : s * INFINITY;
    return s * (ex == 0 ? std::ldexp((double)man, -24) : std::ldexp((double)(1024 + man), ex - 25));
}

template <int KQ>
bool launchTC(float* re, float* im, int n, const FusedPass& pass, const float* img, int* errFlag, const NormLinks& nl,
              cudaStream_t st) {
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
    kApplyTC<KQ><<<(unsigned)grid, kThreadsTC, smemReq, st>>>(re, im, img, numTiles, errFlag, nl, p);
    return !launchFailed("applyPlanF32");
}


// Whether a column's entries j .. j + 3 (j % 4 = 0) are one 16-byte word
// for every lane: true when targets[0..1] are qubits 0, 1, which are bits 0, 1
// of every in-part index, while the lanes' group bits sit above them.
template <int KQ>
bool colWords4(const TC2Params<KQ>& p) {
    for (int l = 0; l < 32; ++l)
        if (p.colLane[l] % 4) return false;
    for (int j = 0; j < (1 << KQ); j += 4)
        for (uint32_t c = 0; c < 4; ++c)
            if (p.colJ[j] % 4 || p.colJ[j + c] != p.colJ[j] + c) return false;
    return true;
}

// Parts of an image: what the split-TF32 pipelined kernels read (the full
// real form at k <= 5, the compact form at k = 6), what the split-BF16 ones
// read, the full TF32 form at every k for the direct-load kernel, and what the
// split-FP16 ones read.
constexpr int kPartTF32 = 1, kPartBF16 = 2, kPartDirect = 4, kPartF16 = 8;
constexpr size_t kNoPart = ~(size_t)0;

// Layout of the operand image of one matrix block of a k-qubit pass holding
// `parts`: float offsets of the full TF32 real form (hi, lo), of the three
// BF16 parts, of the compact TF32 form (hi, lo) and of the two FP16 parts
// with their scale, kNoPart where absent, and the block's size; every part
// starts on a 16-byte boundary (the kernels copy them with cp.async.bulk).
// The part contents are described at buildImageBlock.
struct ImageLayout {
    size_t full = kNoPart, bf16 = kNoPart, compact = kNoPart, f16 = kNoPart, stride = 0;
};
static ImageLayout imageLayout(int k, int parts) {
    ImageLayout L;
    if (k < 4 || k > 6) return L;
    const size_t D = (size_t)1 << k, fullN = 4 * D * D;
    const size_t bEntries = (k == 6) ? 3 * D * D : fullN;
    size_t at = 0;
    if ((parts & kPartDirect) || ((parts & kPartTF32) && k <= 5)) {
        L.full = at;
        at += 2 * fullN;
    }
    if (parts & kPartBF16) {
        L.bf16 = at;
        at += ((3 * bEntries + 1) / 2 + 3) & ~(size_t)3;
    }
    if ((parts & kPartTF32) && k == 6) {
        L.compact = at;
        at += 2 * 3 * D * D;
    }
    if (parts & kPartF16) {
        L.f16 = at;
        at += bEntries + 4;                              // two FP16 parts, then 16 bytes: the unscale factor
    }
    L.stride = (at + 3) & ~(size_t)3;
    return L;
}

// Launch parameters of kApplyTC2 for a pass of KQ qubits on `batch`
// registers of n qubits (instStride floats apart, each with its own image,
// imageStride floats apart): the tile layout tables, the tiles per register
// and control value, and the grid.  False when the pass does not fit.
template <int KQ>
bool tc2Params(int n, const FusedPass& pass, int batch, uint64_t instStride, uint64_t imageStride, TC2Params<KQ>& p,
               uint64_t& numTiles, uint64_t& grid) {
    constexpr int D = 1 << KQ;
    constexpr int TILE = 1 << (KQ + kTileBitsC);
    constexpr int PART = (KQ == 6) ? TILE / 8 : TILE / 4;     // as TC2Shape
    constexpr int V4 = TILE / 512;
    p = TC2Params<KQ>{};
    // I = targets + the 7 lowest other qubits (ascending); tile position b <-> qubit I[b]
    uint64_t tmask = 0;
    for (int b = 0; b < KQ; ++b) tmask |= 1ull << pass.targets[b];
    uint64_t imask = tmask;
    for (int q = 0, added = 0; q < n && added < kTileBitsC; ++q)
        if (!(tmask >> q & 1ull)) {
            imask |= 1ull << q;
            ++added;
        }
    int I[64], ni = 0;
    for (int q = 0; q < n; ++q)
        if (imask >> q & 1ull) I[ni++] = q;
    if (ni != KQ + kTileBitsC) return false;
    // control qubits: outside I (so constant over every tile), at most three
    uint64_t cmask = 0;
    for (int c : pass.controls) cmask |= 1ull << c;
    const int nctl = (int)pass.controls.size();
    if (nctl > 3 || (cmask & imask) || (nctl && (cmask >> n) != 0)) return false;
    int run = 0;
    while (run < ni && I[run] == run) ++run;
    p.runBits = run;
    p.numIns = 0;
    for (int q = 0; q < n; ++q)
        if ((imask | cmask) >> q & 1ull) p.insI[p.numIns++] = q;
    for (uint32_t h = 0; h < (1u << (ni - run)); ++h) {
        uint64_t a = 0;
        for (int i = 0; i < ni - run; ++i)
            if (h >> i & 1u) a |= 1ull << I[run + i];
        p.scatterHigh[h] = a;
    }
    // amplitude offset of a tile position
    auto addrOf = [&](uint32_t pos) -> uint64_t {
        return (uint64_t)(pos & ((1u << run) - 1u)) | p.scatterHigh[pos >> run];
    };
    int posOf[64];
    for (int b = 0; b < ni; ++b) posOf[I[b]] = b;
    int pcPos[kTileBitsC];
    for (int b = 0, m = 0; b < ni; ++b)
        if (!(tmask >> I[b] & 1ull)) pcPos[m++] = b;
    // warp regions: the positions whose bits pcPos[5], pcPos[6] equal the warp
    // index.  Region index = the position with those two bits removed, the
    // others in ascending order, except at k = 6 the top target bit, which goes
    // to the top (it selects the part)
    const int P5 = pcPos[5], P6 = pcPos[6];
    const int J5 = (KQ == 6) ? posOf[pass.targets[5]] : -1;
    int order[24], no = 0;
    for (int b = 0; b < ni; ++b)
        if (b != P5 && b != P6 && b != J5) order[no++] = b;
    if (KQ == 6) order[no++] = J5;
    auto compress = [&](uint32_t pos) -> uint32_t {
        uint32_t q = 0;
        for (int o = 0; o < no; ++o)
            if (pos >> order[o] & 1u) q |= 1u << o;
        return q;
    };
    auto deposit = [&](uint32_t q) -> uint32_t {
        uint32_t pos = 0;
        for (int o = 0; o < no; ++o)
            if (q >> o & 1u) pos |= 1u << order[o];
        return pos;
    };
    for (int w = 0; w < 4; ++w)
        for (int m = 0; m < V4; ++m)
            p.warpOff[w][m] = addrOf(deposit(128u * m) | ((uint32_t)(w & 1) << P5) | ((uint32_t)(w >> 1) << P6));
    for (int l = 0; l < 32; ++l) {
        p.laneOff[l] = addrOf(deposit(4u * l));
        uint32_t pc = 0;
        for (int b = 0; b < 5; ++b)
            if (l >> b & 1) pc |= 1u << pcPos[b];
        p.colLane[l] = padIdx(compress(pc) % PART);
    }
    for (int j = 0; j < D; ++j) {
        uint32_t v = 0;
        for (int b = 0; b < KQ; ++b)
            if (j >> b & 1) v |= 1u << posOf[pass.targets[b]];
        p.colJ[j] = padIdx(compress(v) % PART);
    }
    // tiles per register and control value
    numTiles = 1ull << (n - KQ - kTileBitsC - nctl);
    // one CTA per SM: a batch and the control values share the SMs
    const uint64_t groups = (uint64_t)std::max(1, batch) << nctl;
    const uint64_t ctas = std::min<uint64_t>(numTiles, std::max<uint64_t>(1, (uint64_t)numSMs() / groups));
    grid = ctas * groups;
    p.outMask = ~imask & ~cmask;
    p.ctasPerInst = (uint32_t)ctas;
    p.instStride = instStride;
    p.imageStride = imageStride;
    p.ctrlBits = (uint32_t)nctl;
    for (uint32_t c = 0; c < (1u << nctl); ++c) {
        uint64_t off = 0;
        for (int j = 0; j < nctl; ++j)
            if (c >> j & 1u) off |= 1ull << pass.controls[j];
        p.ctrlOff[c] = off;
    }
    {
        // gridStep = ctas deposited into the qubits outside I
        uint64_t dep = 0, src = ctas;
        for (int q = 0; q < 64 && src; ++q)
            if (p.outMask >> q & 1ull) {
                if (src & 1ull) dep |= 1ull << q;
                src >>= 1;
            }
        p.gridStep = dep;
    }
    return true;
}

// batch > 1: the same pass on `batch` registers of n qubits, instStride floats
// apart, each with its own image, imageStride floats apart
// `img` is the first image block of the pass, `blockStride` floats per block
// (control value); the kernel reads its operand part at partOff.
template <int KQ, int LG, int EG, int LS, int PR, int CV = 1, int ST = 0>
bool launchTC2(float* re, float* im, int n, const FusedPass& pass, const float* img, size_t partOff, size_t blockStride,
               int* errFlag, const NormLinks& nl, cudaStream_t st, int batch = 1, uint64_t instStride = 0,
               uint64_t imageStride = 0) {
    using S = TC2Shape<KQ, LG, EG, LS, PR>;
    static_assert(S::PART == ((KQ == 6) ? S::TILE / 8 : S::TILE / 4), "part layout of tc2Params");
    const size_t smem = S::smemBytes;
    TC2Params<KQ> p;
    uint64_t numTiles = 0, grid = 0;
    if (!tc2Params<KQ>(n, pass, batch, instStride, imageStride, p, numTiles, grid)) return false;
    if constexpr (CV == 4) {
        if (!colWords4(p))
            return launchTC2<KQ, LG, EG, LS, PR, 1, ST>(re, im, n, pass, img, partOff, blockStride, errFlag, nl, st, batch,
                                                        instStride, imageStride);
    }
    img += partOff;
    p.ctrlImageStride = blockStride;
    static bool configured = false;
    if (!configured) {
        if (QG_CUDA(cudaFuncSetAttribute(kApplyTC2<KQ, LG, EG, LS, PR, CV, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "applyPlanF32"))
            return false;
        configured = true;
    }
    kApplyTC2<KQ, LG, EG, LS, PR, CV, ST><<<(unsigned)grid, (4 * (LG + EG) + 1) * 32, smem, st>>>(re, im, img, numTiles, errFlag, nl, p);
    return !launchFailed("applyPlanF32");
}

bool g_tcEnabled = true;
int g_tcPrecision = kPrecTF32;   // operands of the pipelined kernel
int g_tcVersion = 0;      // 0: per pass by target layout; 1, 2, 3: force one kernel
int g_tcTrial = 0;        // autotuner: the pipelined variant being timed (0: none)
bool g_tcTuning = true;   // use the tuned variant of a pass class when there is one
int g_tcStaging = 0;      // loader staging of the pipelined kernels: 0 cp.async, 1 TMA bulk rows
// tuned pipelined variant (2..5, 0 = none) by register size, precision,
// width k and target layout (tuneLayout)
constexpr int kTuneMaxN = 40;
int g_tcTuned[kTuneMaxN + 1][3][7][3] = {};

}  // namespace

// The image of one matrix block of a pass (block c: control value c), with
// the parts of `parts` at the offsets of imageLayout: the full real form
// [[Re, -Im], [Im, Re]] as TF32 hi, lo (canonical K-major, N = K = 2^(k+1));
// its three BF16 parts (at k = 6 the compact form [-Im G; Re G; Im G], 3D
// rows and D K columns, in 8 x 8 core blocks); the compact form as TF32 hi,
// lo (K-major); the two FP16 parts of 2^s times the BF16 parts' form, with
// 2^s the largest power of two for which every |entry| * 2^s <= 2^14, and
// after them the float 2^-(14 + s) the split-FP16 epilogue multiplies by.
static void buildImageBlock(const FusedPass& pass, int block, float* img, int parts) {
    const int k = (int)pass.targets.size();
    const int D = 1 << k, K = 2 * D, N = 2 * D;
    const cplx* const M = pass.m.data() + (size_t)block * D * D;
    const ImageLayout lay = imageLayout(k, parts);
    const bool full = lay.full != kNoPart;
    const bool compact = lay.compact != kNoPart;
    // real form [[Re, -Im], [Im, Re]] as B = Gr (rows r = output index, K index j)
    std::vector<float> hi, lo;
    if (full || compact) {
        hi.resize((size_t)N * K);
        lo.resize((size_t)N * K);
    }
    for (int r = 0; r < N && (full || compact); ++r)
        for (int j = 0; j < K; ++j) {
            const cplx g = M[(size_t)(r % D) * D + (j % D)];
            double v;
            if (r < D) v = (j < D) ? g.real() : -g.imag();
            else v = (j < D) ? g.imag() : g.real();
            const float h = hostTf32RN((float)v);
            hi[(size_t)r * K + j] = h;
            lo[(size_t)r * K + j] = hostTf32RN((float)(v - (double)h));
        }
    // then the three BF16 parts of the pipelined kernel: the real form, or
    // at k = 6 the compact form [-Im G; Re G; Im G] (3D rows, D K columns)
    const size_t fullN = (size_t)N * K;
    const int bRows = (k == 6) ? 3 * D : N, bK = (k == 6) ? D : K;
    const size_t bEntries = (size_t)bRows * bK;
    if (full) {
        packKMajor(hi, N, K, img + lay.full);
        packKMajor(lo, N, K, img + lay.full + fullN);
    }
    uint16_t* bh = reinterpret_cast<uint16_t*>(img + (lay.bf16 != kNoPart ? lay.bf16 : 0));
    uint16_t* bl = bh + bEntries;
    uint16_t* bll = bl + bEntries;
    for (int r = 0; r < bRows && lay.bf16 != kNoPart; ++r)
        for (int j = 0; j < bK; ++j) {
            // k = 6: rows 0..D-1 take the (r, D + j) entries of the real form
            // (-Im), rows D..3D-1 the (r - D, j) entries (Re, then Im)
            const int rr = (k == 6 && r >= D) ? r - D : r, jj = (k == 6 && r < D) ? D + j : j;
            const cplx g = M[(size_t)(rr % D) * D + (jj % D)];
            const double v = (rr < D) ? ((jj < D) ? g.real() : -g.imag()) : ((jj < D) ? g.imag() : g.real());
            const uint16_t h = hostBF16RN((float)v);
            const double r1 = v - (double)bf16Value(h);
            const uint16_t l = hostBF16RN((float)r1);
            const size_t at = (size_t)(r / 8) * (bK / 8) * 64 + (size_t)(j / 8) * 64 + (r % 8) * 8 + (j % 8);
            bh[at] = h;
            bl[at] = l;
            bll[at] = hostBF16RN((float)(r1 - (double)bf16Value(l)));
        }
    if (lay.f16 != kNoPart) {
        double mx = 0.0;
        for (size_t e = 0; e < (size_t)D * D; ++e) mx = std::max(mx, std::max(std::fabs(M[e].real()), std::fabs(M[e].imag())));
        int sc = 24;                                     // all-zero block: any scale
        if (mx > 0.0) {
            int e2 = 0;
            std::frexp(mx, &e2);                         // mx in [2^(e2-1), 2^e2)
            sc = std::min(24, std::max(-24, kF16GMaxExp - e2));
        }
        uint16_t* fh = reinterpret_cast<uint16_t*>(img + lay.f16);
        uint16_t* fl = fh + bEntries;
        for (int r = 0; r < bRows; ++r)
            for (int j = 0; j < bK; ++j) {
                const int rr = (k == 6 && r >= D) ? r - D : r, jj = (k == 6 && r < D) ? D + j : j;
                const cplx g = M[(size_t)(rr % D) * D + (jj % D)];
                const double v = (rr < D) ? ((jj < D) ? g.real() : -g.imag()) : ((jj < D) ? g.imag() : g.real());
                const double vs = std::ldexp(v, sc);             // exact
                const uint16_t h = hostF16RN(vs);
                const size_t at = (size_t)(r / 8) * (bK / 8) * 64 + (size_t)(j / 8) * 64 + (r % 8) * 8 + (j % 8);
                fh[at] = h;
                fl[at] = hostF16RN(vs - f16Value(h));
            }
        float* const tail = img + lay.f16 + bEntries;
        tail[0] = std::ldexp(1.0f, -(kF16XExp + sc));
        tail[1] = tail[2] = tail[3] = 0.f;
    }
    if (compact) {
        // the compact TF32 form for the split-TF32 pipelined kernel
        std::vector<float> ch((size_t)3 * D * D), cl((size_t)3 * D * D);
        for (int r = 0; r < 3 * D; ++r)
            for (int j = 0; j < D; ++j) {
                const int rr = (r < D) ? r : r - D, jj = (r < D) ? D + j : j;
                ch[(size_t)r * D + j] = hi[(size_t)rr * K + jj];
                cl[(size_t)r * D + j] = lo[(size_t)rr * K + jj];
            }
        float* const tc = img + lay.compact;
        packKMajor(ch, 3 * D, D, tc);
        packKMajor(cl, 3 * D, D, tc + (size_t)3 * D * D);
    }
}

// the images of every matrix block of a pass, one layout stride apart
static void buildImage(const FusedPass& pass, float* img, int parts) {
    const size_t stride = imageLayout((int)pass.targets.size(), parts).stride;
    for (size_t b = 0; b < ((size_t)1 << pass.controls.size()); ++b) buildImageBlock(pass, (int)b, img + b * stride, parts);
}

// the image parts the kernels of the current precision and kernel choice read
static int currentParts() {
    const int form = g_tcPrecision == kPrecBF16 ? kPartBF16 : g_tcPrecision == kPrecF16 ? kPartF16 : kPartTF32;
    return form | (g_tcVersion == 1 ? kPartDirect : 0);
}

std::mutex g_stageMutex;
float* g_stage = nullptr;       // page-locked staging of uploadPlanTC
size_t g_stageFloats = 0;

// Operand images of every tensor-core pass (every matrix block of a pass
// with control qubits): only the parts the current precision and kernel
// choice read (tcImagesFit tells when they no longer suffice), laid out by
// imageLayout, built on up to 16 host threads and uploaded in one allocation
// and one copy.  A 6-qubit block holds 96 KB in split-TF32 (72 KB in
// split-BF16); with every part it held 300 KB, whose building and pageable
// copy took ~9 ms of each flush of the 30-qubit circuit.
void* uploadPlanTC(const FusedPlan& plan) {
    DevicePlan* dp = new DevicePlan();
    dp->parts = currentParts();
    if (cudaMalloc(&dp->errFlag, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        delete dp;
        return nullptr;
    }
    cudaMemsetAsync(dp->errFlag, 0, sizeof(int), stream());
    if (cudaMalloc(&dp->norms, 3 * std::max<size_t>(1, plan.passes.size()) * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        dp->norms = nullptr;
    }
    const size_t np = plan.passes.size();
    std::vector<size_t> offset(np + 1, 0);
    for (size_t i = 0; i < np; ++i) {
        const FusedPass& pass = plan.passes[i];
        const int k = (int)pass.targets.size();
        dp->unitary.push_back(pass.unitary ? 1 : 0);
        const bool tc = k >= 4 && k <= 6 && plan.numQubits >= k + 7 + (int)pass.controls.size();
        offset[i + 1] = offset[i] + (tc ? imageLayout(k, dp->parts).stride << pass.controls.size() : 0);
    }
    dp->images.assign(np, nullptr);
    if (offset[np] == 0) return dp;
    if (cudaMalloc(&dp->imageBuf, offset[np] * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        dp->imageBuf = nullptr;
        return dp;                                   // every pass then runs on the SIMT applier
    }
    // built in a page-locked staging buffer kept for the process (a captured
    // 30-qubit circuit re-uploads ~50 MB at every flush), else in pageable memory
    std::lock_guard<std::mutex> lk(g_stageMutex);
    std::vector<float> pageable;
    float* host = nullptr;
    if (g_stageFloats < offset[np]) {
        if (g_stage) cudaFreeHost(g_stage);
        g_stage = nullptr;
        g_stageFloats = 0;
        if (cudaHostAlloc(reinterpret_cast<void**>(&g_stage), offset[np] * sizeof(float), cudaHostAllocDefault) ==
            cudaSuccess)
            g_stageFloats = offset[np];
        else
            cudaGetLastError();
    }
    if (g_stage) {
        host = g_stage;
    } else {
        pageable.resize(offset[np]);
        host = pageable.data();
    }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < np;)
            if (offset[i + 1] > offset[i]) buildImage(plan.passes[i], host + offset[i], dp->parts);
    };
    const unsigned nt = (unsigned)std::min<size_t>({(size_t)16, (size_t)std::max(1u, std::thread::hardware_concurrency()), np});
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
    cudaMemcpy(dp->imageBuf, host, offset[np] * sizeof(float), cudaMemcpyHostToDevice);
    for (size_t i = 0; i < np; ++i)
        if (offset[i + 1] > offset[i]) dp->images[i] = dp->imageBuf + offset[i];
    return dp;
}

// The tensor-core operands of one pass holding `parts`, as uploadPlanTC lays
// them out: the number of floats, and the image itself (a pass without
// control qubits).
size_t tcImageFloats(int k, int parts) { return imageLayout(k, parts).stride; }
void tcBuildImage(const FusedPass& pass, float* img, int parts) { buildImageBlock(pass, 0, img, parts); }
int tcImageParts() { return currentParts(); }
// the host's FP16 rounding of split-FP16 operand images (nearest, ties to even)
void tcRoundHalf(const double* v, uint16_t* out, int count) {
    for (int i = 0; i < count; ++i) out[i] = hostF16RN(v[i]);
}

// Check of the split-FP16 operand images (host, no GPU): for k = 4..6 and
// random matrix blocks scaled by 1e-6 .. 1e4 (one all zero), decode the two
// FP16 parts of every entry of the image's form with the factor after them
// (G = (hi + lo) * 2^-s, 2^-s = factor * 2^14) and compare with the real form
// of G: every entry within 2^-21 of the block's largest, and the largest
// scaled entry at most 2^14.  0 when all hold, else 1.
int tcCheckHalfImages() {
    uint64_t x = 0x9E3779B97F4A7C15ull;
    auto uni = [&x]() {                                  // xorshift64*, uniform in (-1, 1)
        x ^= x >> 12;
        x ^= x << 25;
        x ^= x >> 27;
        return (double)((x * 0x2545F4914F6CDD1Dull) >> 11) * 0x1p-52 - 1.0;
    };
    const double scales[7] = {0.0, 1e-6, 1e-3, 1.0, 7.5, 60.0, 1e4};
    for (int k = 4; k <= 6; ++k)
        for (double sc : scales) {
            const int D = 1 << k;
            FusedPass pass;
            for (int b = 0; b < k; ++b) pass.targets.push_back(b);
            pass.m.resize((size_t)D * D);
            for (auto& g : pass.m) g = cplx(sc * uni(), sc * uni());
            const ImageLayout lay = imageLayout(k, kPartF16);
            std::vector<float> img(lay.stride, 0.f);
            buildImageBlock(pass, 0, img.data(), kPartF16);
            const int bRows = (k == 6) ? 3 * D : 2 * D, bK = (k == 6) ? D : 2 * D;
            const size_t bEntries = (size_t)bRows * bK;
            const uint16_t* fh = reinterpret_cast<const uint16_t*>(img.data() + lay.f16);
            const uint16_t* fl = fh + bEntries;
            const double unscale = (double)img[lay.f16 + bEntries] * std::ldexp(1.0, kF16XExp);
            if (!(unscale > 0.0)) return 1;
            double mx = 0.0;
            for (const cplx& g : pass.m) mx = std::max(mx, std::max(std::fabs(g.real()), std::fabs(g.imag())));
            for (int r = 0; r < bRows; ++r)
                for (int j = 0; j < bK; ++j) {
                    const int rr = (k == 6 && r >= D) ? r - D : r, jj = (k == 6 && r < D) ? D + j : j;
                    const cplx g = pass.m[(size_t)(rr % D) * D + (jj % D)];
                    const double v = (rr < D) ? ((jj < D) ? g.real() : -g.imag()) : ((jj < D) ? g.imag() : g.real());
                    const size_t at = (size_t)(r / 8) * (bK / 8) * 64 + (size_t)(j / 8) * 64 + (r % 8) * 8 + (j % 8);
                    const double hi = f16Value(fh[at]), lo = f16Value(fl[at]);
                    if (std::fabs(hi) > 16384.0) return 1;
                    if (std::fabs((hi + lo) * unscale - v) > std::ldexp(mx, -21)) return 1;
                }
        }
    return 0;
}
// whether a plan's images hold the parts the current precision and kernel
// choice read (else the caller uploads the plan again)
bool tcImagesFit(const void* devPlan) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    return dp && (currentParts() & ~dp->parts) == 0;
}

void freePlanTC(void* h) {
    DevicePlan* dp = reinterpret_cast<DevicePlan*>(h);
    if (!dp) return;
    cudaStreamSynchronize(stream());
    if (dp->imageBuf) cudaFree(dp->imageBuf);
    if (dp->errFlag) cudaFree(dp->errFlag);
    if (dp->norms) cudaFree(dp->norms);
    delete dp;
}

// start of a plan application (pass 0): no previous tensor-core pass
void tcBeginPlan(void* devPlan, size_t numPasses) {
    DevicePlan* dp = reinterpret_cast<DevicePlan*>(devPlan);
    if (!dp) return;
    dp->lastTC = -1;
    dp->chain = false;
    dp->inNorm.assign(numPasses, nullptr);
    dp->target.assign(numPasses, nullptr);
}

// start of every applyPlanF32Range call: the caller may have changed the
// state since the last call, so the next tensor-core pass measures its input;
// entryBound: sum |x|^2 of the state now, on the device, or null
void tcBeginRange(void* devPlan, const double* entryBound) {
    DevicePlan* dp = reinterpret_cast<DevicePlan*>(devPlan);
    if (!dp) return;
    dp->chain = false;
    dp->entryBound = entryBound;
}

// a pass ran on the SIMT applier: a non-unitary one changes the norm
void tcNoteSimtPass(void* devPlan, size_t index) {
    DevicePlan* dp = reinterpret_cast<DevicePlan*>(devPlan);
    if (dp && (index >= dp->unitary.size() || !dp->unitary[index])) {
        dp->chain = false;
        dp->entryBound = nullptr;
    }
}

// Which applier runs a pass on registers of n qubits: 0 = the FP32 SIMT
// applier, 1 = the direct-load tensor-core kernel, 2..5 = the pipelined one
// (2: 2 loader groups on alternate chunks + 1 epilogue group; 3: 1 + 1;
// 4: 1 + 2; 5: 2 loader groups splitting every chunk + 2 epilogue groups).
// Default choice, measured at 30 qubits in ms per pass; "high" means every
// target is at or above qubit 5.  1..3 qubits: the SIMT applier.
// Split-TF32 operands (the default):
//   * 4 qubits: kernel 3 (2.8-3.0, against 2.8-3.1 for kernel 2, 3.1-3.2 SIMT);
//   * 5 qubits: kernel 2 (2.5-2.9, against 2.8-3.0 for kernel 5);
//   * 6 qubits: kernel 5 (2.6-3.0, against 2.8-3.1 for kernel 2).
// Split-BF16 operands (split-FP16 takes the same choices):
//   * 4 qubits, high targets: kernel 2 (2.6-2.8, against SIMT 3.1-3.2);
//   * 4 qubits, other targets: kernel 5 (2.7-3.0);
//   * 5 qubits: kernel 5 (2.7-3.0, against 2.9-3.1 for kernel 2);
//   * 6 qubits: kernel 5 (2.7-3.0).  Kernels 2 and 4 are each a few percent
//     faster on some target sets.  Choosing by target set came to the same
//     total over the 30-qubit circuit (297.4 against 296.3 ms).
// A pass's target layout class for the tuner: 2 when qubits 0 and 1 are both
// targets (the 16-byte column variant), 1 when another target is below qubit
// 5, 0 when every target is at or above qubit 5.
int tuneLayout(const FusedPass& pass) {
    if (pass.targets.size() >= 2 && pass.targets[0] == 0 && pass.targets[1] == 1) return 2;
    return pass.targets[0] < 5 ? 1 : 0;
}
void setTunedKernel(int n, int prec, int k, int layout, int version) {
    if (n >= 0 && n <= kTuneMaxN && prec >= 0 && prec <= 2 && k >= 4 && k <= 6 && layout >= 0 && layout < 3)
        g_tcTuned[n][prec][k][layout] = (version >= 2 && version <= 5) ? version : 0;
}
int tunedKernel(int n, int prec, int k, int layout) {
    if (n < 0 || n > kTuneMaxN || prec < 0 || prec > 2 || k < 4 || k > 6 || layout < 0 || layout > 2) return 0;
    return g_tcTuned[n][prec][k][layout];
}
void setKernelTrial(int version) { g_tcTrial = (version >= 2 && version <= 5) ? version : 0; }
void setKernelTuning(bool on) { g_tcTuning = on; }

// the fixed per-class default of the pipelined kernel (measured choices,
// listed above), by precision, width and target layout class (tuneLayout)
int defaultTcKernel(int prec, int k, int layout) {
    if (prec == kPrecTF32) return k == 4 ? 3 : k == 5 ? 2 : 5;
    if (k == 4) return layout == 0 ? 2 : 5;
    return 5;
}
static int tcKernelChoice(const FusedPass& pass, int n) {
    const int k = (int)pass.targets.size();
    if (g_tcVersion != 0) return g_tcVersion;
    if (g_tcTrial != 0) return g_tcTrial;
    if (g_tcTuning) {
        const int v = tunedKernel(n, g_tcPrecision, k, tuneLayout(pass));
        if (v) return v;
    }
    return defaultTcKernel(g_tcPrecision, k, tuneLayout(pass));
}
int tcKernelFor(const FusedPass& pass, int n) {
    const int k = (int)pass.targets.size(), nc = (int)pass.controls.size();
    if (!g_tcEnabled || k < 4 || k > 6 || n < k + 7 + nc) return 0;
    const int v = tcKernelChoice(pass, n);
    return (nc && v == 1) ? 5 : v;          // the direct-load kernel takes no control qubits
}

// Host model of the global accesses of kApplyTC2 for one pass on one
// register of n qubits, from the same launch parameters and tile walk: every
// CTA (register group, control value), every tile of its sequence (with the
// loaders' step, one tile group, and the epilogue's, two groups), every warp,
// lane, 128-position block m and the 4 amplitudes of a 16-byte access.
// Counts the accesses per amplitude; -1 when an address falls outside the
// register or the pass does not fit.
template <int KQ>
int tc2Coverage(int n, const FusedPass& pass, int groups, std::vector<uint8_t>& count) {
    TC2Params<KQ> p;
    uint64_t numTiles = 0, grid = 0;
    if (!tc2Params<KQ>(n, pass, 1, 0, 0, p, numTiles, grid)) return -1;
    constexpr int V4 = (1 << (KQ + kTileBitsC)) / 512;
    const uint64_t size = 1ull << n;
    count.assign(size, 0);
    for (uint64_t b = 0; b < grid; ++b) {
        const uint64_t cta = b % p.ctasPerInst, u = b / p.ctasPerInst;
        if ((u >> p.ctrlBits) != 0) return -1;
        const uint64_t off = p.ctrlOff[u & ((1u << p.ctrlBits) - 1u)];
        for (int g = 0; g < groups; ++g) {
            TileWalker<KQ> walk;
            for (uint64_t t = cta + (uint64_t)g * p.ctasPerInst; t < numTiles; t += (uint64_t)groups * p.ctasPerInst) {
                const uint64_t base = walk.at(p, t);
                for (int rw = 0; rw < 4; ++rw)
                    for (int lane = 0; lane < 32; ++lane)
                        for (int m = 0; m < V4; ++m)
                            for (int e = 0; e < 4; ++e) {
                                const uint64_t a = off + base + p.laneOff[lane] + p.warpOff[rw][m] + (uint64_t)e;
                                if (a >= size) return -1;
                                if (count[a] < 255) ++count[a];
                            }
            }
        }
    }
    return 0;
}

// Check of imageLayout against what the kernels read (host, no GPU): for
// k = 4..6 and every parts set the library builds (one operand form, with or
// without the direct-load kernel's part), each part a kernel of that set
// reads is present, starts on a 16-byte boundary, lies inside the block and
// overlaps no other part.  0 when all hold, else 1.
int tcCheckImageLayouts() {
    const int sets[6] = {kPartTF32, kPartBF16, kPartF16, kPartTF32 | kPartDirect, kPartBF16 | kPartDirect,
                         kPartF16 | kPartDirect};
    for (int k = 4; k <= 6; ++k)
        for (int parts : sets) {
            const ImageLayout L = imageLayout(k, parts);
            const size_t D = (size_t)1 << k, NK = 4 * D * D, GE = (k == 6) ? 3 * D * D : NK;
            struct Read {
                size_t off, floats;
            };
            std::vector<Read> reads;
            if (parts & kPartTF32) reads.push_back({k == 6 ? L.compact : L.full, 2 * GE});    // hi, lo
            if (parts & kPartBF16) reads.push_back({L.bf16, 3 * GE / 2});                       // three BF16 parts
            if (parts & kPartDirect) reads.push_back({L.full, 2 * NK});                         // direct-load kernel
            if (parts & kPartF16) reads.push_back({L.f16, GE + 1});                             // two FP16 parts, the factor
            if (L.stride % 4) return 1;
            for (const Read& r : reads)
                if (r.off == kNoPart || r.off % 4 || r.off + r.floats > L.stride) return 1;
            // the parts present do not overlap
            std::vector<std::pair<size_t, size_t>> present;
            if (L.full != kNoPart) present.push_back({L.full, L.full + 2 * NK});
            if (L.bf16 != kNoPart) present.push_back({L.bf16, L.bf16 + (3 * GE + 1) / 2});
            if (L.compact != kNoPart) present.push_back({L.compact, L.compact + 6 * D * D});
            if (L.f16 != kNoPart) present.push_back({L.f16, L.f16 + GE + 4});
            for (size_t a = 0; a < present.size(); ++a)
                for (size_t b = a + 1; b < present.size(); ++b)
                    if (present[a].first < present[b].second && present[b].first < present[a].second) return 1;
            for (const auto& r : present)
                if (r.second > L.stride) return 1;
        }
    return 0;
}

// 0 when a pass on `targets` (ascending) with `controls` reads and writes
// every amplitude of an n-qubit register exactly once (both tile walks of
// tc2Coverage), 1 when it does not, -1 when it does not fit or n > 26
int tcCheckCoverage(int n, const std::vector<int>& targets, const std::vector<int>& controls) {
    const int k = (int)targets.size();
    if (n > 26 || k < 4 || k > 6 || controls.size() > 3) return -1;
    FusedPass pass;
    pass.targets = targets;
    pass.controls = controls;
    std::vector<uint8_t> cnt;
    for (int groups = 1; groups <= 2; ++groups) {
        const int rc = k == 4 ? tc2Coverage<4>(n, pass, groups, cnt)
                              : k == 5 ? tc2Coverage<5>(n, pass, groups, cnt) : tc2Coverage<6>(n, pass, groups, cnt);
        if (rc) return -1;
        for (uint8_t v : cnt)
            if (v != 1) return 1;
    }
    return 0;
}

// Launch tensor-core kernel `version` (tcKernelFor) for a pass of k = 4..6
// qubits on one register (batch = 1) or on a batch of registers; false if the
// launch failed.  The direct-load kernel (version 1) takes single registers.
static bool launchPassTC(int version, const FusedPass& pass, float* re, float* im, int n, const float* img, int parts,
                         int* errFlag, const NormLinks& nl, cudaStream_t st, int batch, uint64_t instStride,
                         uint64_t imageStride) {
    const int k = (int)pass.targets.size();
    bool ok = false;
    // the operand part this launch reads; a part that was not built stops the
    // launch (its kernel would read past the image)
    const ImageLayout lay = imageLayout(k, parts);
    const size_t po = version < 2                        ? lay.full
                      : g_tcPrecision == kPrecBF16 ? lay.bf16
                      : g_tcPrecision == kPrecF16  ? lay.f16
                      : k == 6                     ? lay.compact
                                                   : lay.full;
    if (po == kNoPart || lay.stride == 0) return false;
    const size_t bs = lay.stride;
    // the default kernels, when the targets include qubits 0 and 1: the
    // variant with 16-byte column words
    bool done = false;
    if (g_tcVersion == 0 && pass.targets[0] == 0 && pass.targets[1] == 1) {
#define QG_TC2W(KQ, LG, EG, LS, PR)                                                                                    \
    (done = true,                                                                                                       \
     g_tcStaging ? launchTC2<KQ, LG, EG, LS, PR, 4, 1>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride) \
                 : launchTC2<KQ, LG, EG, LS, PR, 4, 0>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride))
// split-FP16 kernels stage with cp.async only
#define QG_TC2F(KQ) \
    (done = true, launchTC2<KQ, 2, 2, 2, kPrecF16, 4, 0>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride))
        const bool tf = g_tcPrecision == kPrecTF32, bf = g_tcPrecision == kPrecBF16;
        if (tf && k == 4 && version == 3) ok = QG_TC2W(4, 1, 1, 1, kPrecTF32);
        else if (tf && k == 5 && version == 2) ok = QG_TC2W(5, 2, 1, 1, kPrecTF32);
        else if (tf && k == 6 && version == 5) ok = QG_TC2W(6, 2, 2, 2, kPrecTF32);
        else if (bf && k == 4 && version == 5) ok = QG_TC2W(4, 2, 2, 2, kPrecBF16);
        else if (bf && k == 5 && version == 5) ok = QG_TC2W(5, 2, 2, 2, kPrecBF16);
        else if (bf && k == 6 && version == 5) ok = QG_TC2W(6, 2, 2, 2, kPrecBF16);
        else if (!tf && !bf && k == 4 && version == 5) ok = QG_TC2F(4);
        else if (!tf && !bf && k == 5 && version == 5) ok = QG_TC2F(5);
        else if (!tf && !bf && k == 6 && version == 5) ok = QG_TC2F(6);
#undef QG_TC2W
#undef QG_TC2F
    }
    if (done) return ok;
    if (version >= 2) {
        // 2: two loader groups (alternate chunks) + one epilogue group; 3: one
        // + one; 4: one + two; 5: two loader groups (each half of every chunk)
        // + two epilogue groups
#define QG_TC2S(KQ, PR, ST)                                                                                                    \
    (version == 2   ? launchTC2<KQ, 2, 1, 1, PR, 1, ST>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride)  \
     : version == 3 ? launchTC2<KQ, 1, 1, 1, PR, 1, ST>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride)  \
     : version == 4 ? launchTC2<KQ, 1, 2, 1, PR, 1, ST>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride)  \
                    : launchTC2<KQ, 2, 2, 2, PR, 1, ST>(re, im, n, pass, img, po, bs, errFlag, nl, st, batch, instStride, imageStride))
#define QG_TC2P(KQ, PR) (g_tcStaging ? QG_TC2S(KQ, PR, 1) : QG_TC2S(KQ, PR, 0))
#define QG_TC2(KQ)                                                                     \
    (g_tcPrecision == kPrecTF32   ? QG_TC2P(KQ, kPrecTF32)                               \
     : g_tcPrecision == kPrecBF16 ? QG_TC2P(KQ, kPrecBF16)                               \
                                  : QG_TC2S(KQ, kPrecF16, 0))
        switch (k) {
            case 4: ok = QG_TC2(4); break;
            case 5: ok = QG_TC2(5); break;
            case 6: ok = QG_TC2(6); break;
            default: return false;
        }
#undef QG_TC2
#undef QG_TC2P
#undef QG_TC2S
        return ok;
    }
    if (batch != 1) return false;
    switch (k) {
        case 4: return launchTC<4>(re, im, n, pass, img + po, errFlag, nl, st);
        case 5: return launchTC<5>(re, im, n, pass, img + po, errFlag, nl, st);
        case 6: return launchTC<6>(re, im, n, pass, img + po, errFlag, nl, st);
        default: return false;
    }
}

// explicit entry used by the FP32 engine with the pass index: 1 = applied on
// the tensor cores, 0 = not a tensor-core pass (the caller runs it on SIMT),
// -1 = the launch failed (already reported)
int applyPassTCIndexed(QuregF32& q, const FusedPass& pass, const void* devPlan, size_t index, cudaStream_t st) {
    DevicePlan* dp = const_cast<DevicePlan*>(reinterpret_cast<const DevicePlan*>(devPlan));
    if (!dp || index >= dp->images.size() || !dp->images[index]) return 0;
    const int k = (int)pass.targets.size();
    float* re = f32re(q);
    float* im = f32im(q);
    const int n = f32n(q);
    const int version = tcKernelFor(pass, n);
    if (version == 0) return 0;
    NormLinks nl{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (dp->norms) {
        if (dp->inNorm.size() != dp->images.size()) dp->inNorm.assign(dp->images.size(), nullptr);
        if (dp->target.size() != dp->images.size()) dp->target.assign(dp->images.size(), nullptr);
        double* mine = dp->norms + 3 * index;            // in, out, scale^2
        cudaMemsetAsync(mine, 0, 3 * sizeof(double), st);
        nl.out = mine + 1;
        nl.scaleSq = mine + 2;
        const bool chained = dp->chain && dp->lastTC >= 0;
        nl.in = chained ? nullptr : mine;
        dp->inNorm[index] = chained ? dp->norms + 3 * dp->lastTC + 1 : mine;
        if (chained) nl.boundSq = dp->norms + 3 * dp->lastTC + 1;
        else if (dp->entryBound) nl.boundSq = dp->entryBound;
        const bool prevUnitary = dp->lastTC >= 0 && dp->unitary[dp->lastTC];
        if (prevUnitary) {
            nl.corrIn = dp->inNorm[dp->lastTC];
            nl.corrOut = dp->norms + 3 * dp->lastTC + 1;
            nl.corrScaleSq = dp->norms + 3 * dp->lastTC + 2;
        }
        // a chain of unitary passes keeps the norm its first pass started from
        const bool continues = chained && prevUnitary && dp->target[dp->lastTC];
        if (continues) nl.corrTarget = dp->target[dp->lastTC];
        dp->target[index] = continues ? dp->target[dp->lastTC] : dp->inNorm[index];
    }
    const bool ok = launchPassTC(version, pass, re, im, n, dp->images[index], dp->parts, dp->errFlag, nl, st, 1, 0, 0);
    if (!ok) return -1;
    dp->lastTC = (int)index;
    dp->chain = true;
    return 1;
}

int tcErrorFlag(const void* devPlan) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    if (!dp || !dp->errFlag) return 0;
    int v = 0;
    cudaMemcpyAsync(&v, dp->errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    if (v) cudaMemsetAsync(dp->errFlag, 0, sizeof(int), stream());   // reported once
    return v;
}

// norm record of pass i of the last application: (input norm, output norm,
// scale^2 applied); 0 if it was not a tensor-core pass or has no record
int tcPassNorms(const void* devPlan, size_t index, double* out3) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    if (!dp || !dp->norms || index >= dp->inNorm.size() || !dp->inNorm[index]) return 0;
    cudaMemcpyAsync(out3, dp->inNorm[index], sizeof(double), cudaMemcpyDeviceToHost, stream());
    cudaMemcpyAsync(out3 + 1, dp->norms + 3 * index + 1, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
    return 1;
}

// the plan's last application ended in a chain of unitary passes whose last
// tensor-core pass left a norm record: the chain's starting norm and that
// pass's output norm (device pointers, valid until the plan runs again)
bool tcFinalNorms(const void* devPlan, const double** target, const double** out) {
    const DevicePlan* dp = reinterpret_cast<const DevicePlan*>(devPlan);
    if (!dp || !dp->norms || !dp->chain || dp->lastTC < 0 || (size_t)dp->lastTC >= dp->target.size()) return false;
    if (!dp->unitary[dp->lastTC] || !dp->target[dp->lastTC]) return false;
    *target = dp->target[dp->lastTC];
    *out = dp->norms + 3 * dp->lastTC + 1;
    return true;
}

void setTensorCoresEnabled(bool on) { g_tcEnabled = on; }
bool setTensorCorePrecision(int mode) {
    if (mode != kPrecTF32 && mode != kPrecBF16 && mode != kPrecF16) return false;
    g_tcPrecision = mode;
    return true;
}
int tensorCorePrecision() { return g_tcPrecision; }
bool setTensorCoreStaging(int mode) {
    if (mode != 0 && mode != 1) return false;
    g_tcStaging = mode;
    return true;
}
int tensorCoreStaging() { return g_tcStaging; }
void setTensorCoreKernel(int version) { g_tcVersion = (version >= 1 && version <= 5) ? version : 0; }
bool tensorCoresEnabled() { return g_tcEnabled; }

// One pass on `batch` registers of n qubits: register b's planes start
// b * 2^n floats into re and im, and its operand image imageStride floats
// after register b - 1's.  One launch; the registers share the SMs.  No norm
// drift correction (the callers normalise per register).  Returns false for a
// pass the tensor cores do not take or a failed launch.
bool applyPassTCBatch(float* re, float* im, int n, const FusedPass& pass, const float* images, size_t imageStride,
                      int parts, int batch, int* errFlag, cudaStream_t st) {
    const int version = tcKernelFor(pass, n);
    if (version < 2 || !images || !pass.controls.empty()) return false;
    const NormLinks nl{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return launchPassTC(version, pass, re, im, n, images, parts, errFlag, nl, st, batch, 1ull << n,
                        (uint64_t)imageStride);
}

}  // namespace qg
