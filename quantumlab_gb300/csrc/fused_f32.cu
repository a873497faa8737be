// fused_f32.cu -- the FP32 fused engine: an FP32 SoA register, the pass
// applier, and FP64-accumulated reductions over it (sm_103a).
//
// No counterpart in the reference.  A compiled plan (fused_plan.cpp) is a
// list of dense 2^k x 2^k complex matrices formed in FP64; each is applied to
// the FP32 state in one streaming pass.  This file holds the SIMT applier
// (FP32 FFMA, matrix rounded to FP32 and held in the kernel's constant
// parameter bank) used for k <= 5; the tensor-core split-TF32 applier lives
// in fused_tc.cu.  Norms, probabilities and the comparison against an FP64
// register accumulate in FP64.
#include "fused_plan.h"
#include "quest_gb300.h"
#include "reduce_kernel.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace qg {

struct QuregF32 {
    int n = 0;
    float* re = nullptr;
    float* im = nullptr;
    double* scratch = nullptr;     // kScratchDoubles, counter kept at 0
    double* host = nullptr;        // pinned result slots
    double* staging = nullptr;     // FP64 device staging for host transfers
    size_t stagingAmps = 0;
    Scratch w() const {
        Scratch s;
        s.partials = scratch;
        s.result = scratch + 2 * kMaxReduceBlocks;
        s.counter = reinterpret_cast<unsigned int*>(scratch + 2 * kMaxReduceBlocks + 64);
        s.host = host;
        return s;
    }
};

// tensor-core applier (fused_tc.cu): 1 applied, 0 not a tensor-core pass, -1 launch failed
int applyPassTCIndexed(QuregF32& q, const FusedPass& p, const void* devPlan, size_t index, cudaStream_t st);
void* uploadPlanTC(const FusedPlan& plan);
bool tcImagesFit(const void* devPlan);
void freePlanTC(void* d);
int tcErrorFlag(const void* devPlan);
int tcPassNorms(const void* devPlan, size_t index, double* out3);
bool tcFinalNorms(const void* devPlan, const double** target, const double** out);
void tcBeginPlan(void* devPlan, size_t numPasses);
void tcBeginRange(void* devPlan, const double* entryBound);
void tcNoteSimtPass(void* devPlan, size_t index);
void setTensorCoresEnabled(bool on);
void setTensorCoreKernel(int version);
bool setTensorCorePrecision(int mode);
int tensorCorePrecision();
bool setTensorCoreStaging(int mode);
int tensorCoreStaging();
int tcCheckCoverage(int n, const std::vector<int>& targets, const std::vector<int>& controls);
int tcCheckImageLayouts();
void tcRoundHalf(const double* v, uint16_t* out, int count);
int tcCheckHalfImages();
bool tensorCoresEnabled();
int tcKernelFor(const FusedPass& pass, int n);
float* f32re(QuregF32& q) { return q.re; }
float* f32im(QuregF32& q) { return q.im; }
int f32n(const QuregF32& q) { return q.n; }

namespace {

constexpr int kApplyThreads = 128;

template <int K>
struct PassParams {
    float mr[1 << K][1 << K];
    float mi[1 << K][1 << K];
    uint64_t off[1 << K];     // address offset of matrix index j (bits on the targets)
    int ins[K];               // ascending target positions (zeros inserted into the group index)
};

// One thread per group of 2^K amplitudes (the non-target bits fixed): load
// the group, multiply by the matrix (constant-bank operands), store.
template <int K>
__global__ void __launch_bounds__(kApplyThreads, (K <= 4 ? 4 : 2)) kApplySimt(float* __restrict__ re, float* __restrict__ im,
                                                           uint64_t nGroups, const __grid_constant__ PassParams<K> p) {
    constexpr int D = 1 << K;
    const uint64_t g = (uint64_t)blockIdx.x * kApplyThreads + threadIdx.x;
    if (g >= nGroups) return;
    uint64_t base = g;
#pragma unroll
    for (int b = 0; b < K; ++b) {
        const int s = p.ins[b];
        base = ((base >> s) << (s + 1)) | (base & ((1ull << s) - 1ull));
    }
    float xr[D], xi[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        xr[j] = re[base + p.off[j]];
        xi[j] = im[base + p.off[j]];
    }
    // rows rolled (uniform index: matrix entries come from the constant bank
    // through the uniform datapath), columns unrolled
#pragma unroll 1
    for (int r = 0; r < D; ++r) {
        float ar = 0.f, ai = 0.f;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            ar = fmaf(p.mr[r][j], xr[j], ar);
            ar = fmaf(-p.mi[r][j], xi[j], ar);
            ai = fmaf(p.mr[r][j], xi[j], ai);
            ai = fmaf(p.mi[r][j], xr[j], ai);
        }
        re[base + p.off[r]] = ar;
        im[base + p.off[r]] = ai;
    }
}

template <int K>
bool launchSimt(QuregF32& q, const FusedPass& pass, cudaStream_t st) {
    constexpr int D = 1 << K;
    PassParams<K> p;
    for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) {
            p.mr[r][c] = (float)pass.m[(size_t)r * D + c].real();
            p.mi[r][c] = (float)pass.m[(size_t)r * D + c].imag();
        }
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
        for (int b = 0; b < K; ++b)
            if (j >> b & 1) o |= 1ull << pass.targets[b];
        p.off[j] = o;
    }
    for (int b = 0; b < K; ++b) p.ins[b] = pass.targets[b];
    const uint64_t nGroups = 1ull << (q.n - K);
    const unsigned blocks = (unsigned)((nGroups + kApplyThreads - 1) / kApplyThreads);
    kApplySimt<K><<<blocks, kApplyThreads, 0, st>>>(q.re, q.im, nGroups, p);
    return !launchFailed("applyPlanF32");
}

bool applyPassSimt(QuregF32& q, const FusedPass& pass, cudaStream_t st) {
    switch (pass.targets.size()) {
        case 1: return launchSimt<1>(q, pass, st);
        case 2: return launchSimt<2>(q, pass, st);
        case 3: return launchSimt<3>(q, pass, st);
        case 4: return launchSimt<4>(q, pass, st);
        case 5: return launchSimt<5>(q, pass, st);
        default: return false;
    }
}

// ------------------------------------------------------------ elementwise
__global__ void kZeroF32(float* __restrict__ re, float* __restrict__ im) {
    re[0] = 1.f;
    (void)im;
}
// FP64 <-> FP32 conversions: four amplitudes per thread with 16-byte accesses
// (the arrays start on 32-byte boundaries); the tail of n % 4 amplitudes is
// converted one by one
constexpr unsigned kConvThreads = 256;
inline unsigned convBlocks(uint64_t n) { return (unsigned)(((n + 3) / 4 + kConvThreads - 1) / kConvThreads); }

__global__ void kF64toF32(const double* __restrict__ sr, const double* __restrict__ si, float* __restrict__ dr,
                          float* __restrict__ di, uint64_t n) {
    const uint64_t i = 4 * ((uint64_t)blockIdx.x * kConvThreads + threadIdx.x);
    if (i + 3 < n) {
        const double2 r0 = *reinterpret_cast<const double2*>(sr + i), r1 = *reinterpret_cast<const double2*>(sr + i + 2);
        const double2 m0 = *reinterpret_cast<const double2*>(si + i), m1 = *reinterpret_cast<const double2*>(si + i + 2);
        *reinterpret_cast<float4*>(dr + i) = make_float4((float)r0.x, (float)r0.y, (float)r1.x, (float)r1.y);
        *reinterpret_cast<float4*>(di + i) = make_float4((float)m0.x, (float)m0.y, (float)m1.x, (float)m1.y);
    } else {
        for (uint64_t j = i; j < n; ++j) {
            dr[j] = (float)sr[j];
            di[j] = (float)si[j];
        }
    }
}
// FP64 -> FP32 as kF64toF32, also adding sum |x|^2 of the FP32 values into
// *normSq (FP32 sums of each thread's 8 values, FP64 across its groups, one
// FP64 atomic per block; grid-stride over one wave of blocks)
__global__ void kF64toF32Norm(const double* __restrict__ sr, const double* __restrict__ si, float* __restrict__ dr,
                              float* __restrict__ di, uint64_t n, double* __restrict__ normSq) {
    double acc = 0.0;
    const uint64_t groups = n / 4;
    for (uint64_t g = (uint64_t)blockIdx.x * kConvThreads + threadIdx.x; g < groups;
         g += (uint64_t)gridDim.x * kConvThreads) {
        const uint64_t i = 4 * g;
        const double2 r0 = *reinterpret_cast<const double2*>(sr + i), r1 = *reinterpret_cast<const double2*>(sr + i + 2);
        const double2 m0 = *reinterpret_cast<const double2*>(si + i), m1 = *reinterpret_cast<const double2*>(si + i + 2);
        const float4 fr = make_float4((float)r0.x, (float)r0.y, (float)r1.x, (float)r1.y);
        const float4 fi = make_float4((float)m0.x, (float)m0.y, (float)m1.x, (float)m1.y);
        *reinterpret_cast<float4*>(dr + i) = fr;
        *reinterpret_cast<float4*>(di + i) = fi;
        float s = fr.x * fr.x;
        s = fmaf(fr.y, fr.y, s);
        s = fmaf(fr.z, fr.z, s);
        s = fmaf(fr.w, fr.w, s);
        s = fmaf(fi.x, fi.x, s);
        s = fmaf(fi.y, fi.y, s);
        s = fmaf(fi.z, fi.z, s);
        s = fmaf(fi.w, fi.w, s);
        acc += (double)s;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (uint64_t j = 4 * groups; j < n; ++j) {
            dr[j] = (float)sr[j];
            di[j] = (float)si[j];
            acc += (double)dr[j] * dr[j] + (double)di[j] * di[j];
        }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[kConvThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(kConvThreads / 32); ++w) b += ws[w];
        atomicAdd(normSq, b);
    }
}
// FP32 -> FP64, each amplitude times *scale when scale is given
// FP32 -> FP64 by moving the fields (exact, as the conversion instruction):
// exponent rebiased by 1023 - 127 = 896, fraction shifted by 52 - 23 = 29.
// Zeros too; subnormals, infinities and NaNs take the conversion
// instruction.  GB300 runs that instruction on its FP64 pipe, which made the
// conversion of a 30-qubit state FP64-bound.
__device__ __forceinline__ double toF64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    if (e != 0u && e != 0xFFu)
        return __longlong_as_double((long long)(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29)));
    if ((u & 0x7FFFFFFFu) == 0u) return __longlong_as_double((long long)sign);
    return (double)f;
}
__global__ void kF32toF64(const float* __restrict__ sr, const float* __restrict__ si, double* __restrict__ dr,
                          double* __restrict__ di, uint64_t n, const double* __restrict__ scale) {
    const uint64_t i = 4 * ((uint64_t)blockIdx.x * kConvThreads + threadIdx.x);
    if (i + 3 < n) {
        const float4 r = *reinterpret_cast<const float4*>(sr + i), m = *reinterpret_cast<const float4*>(si + i);
        double2 a = make_double2(toF64(r.x), toF64(r.y)), b = make_double2(toF64(r.z), toF64(r.w));
        double2 c = make_double2(toF64(m.x), toF64(m.y)), d = make_double2(toF64(m.z), toF64(m.w));
        if (scale) {
            const double s = *scale;
            a.x *= s; a.y *= s; b.x *= s; b.y *= s;
            c.x *= s; c.y *= s; d.x *= s; d.y *= s;
        }
        *reinterpret_cast<double2*>(dr + i) = a;
        *reinterpret_cast<double2*>(dr + i + 2) = b;
        *reinterpret_cast<double2*>(di + i) = c;
        *reinterpret_cast<double2*>(di + i + 2) = d;
    } else {
        const double s = scale ? *scale : 1.0;
        for (uint64_t j = i; j < n; ++j) {
            dr[j] = (double)sr[j] * s;
            di[j] = (double)si[j] * s;
        }
    }
}
// sqrt(*target / *out) into g_planScale (the last norm correction of a plan);
// launched on the library stream right before the conversion that reads it
__device__ double g_planScale;
__global__ void kFinalScale(const double* __restrict__ target, const double* __restrict__ out) {
    const double o = *out;
    g_planScale = (o > 0.0) ? sqrt(*target / o) : 1.0;
}

// Trace of a density matrix of N qubits held as a 2N-qubit vector: the sum of
// the real parts at i (2^N + 1), one block, FP64 accumulation.  Into
// g_trace[slot].
__device__ double g_trace[2];
constexpr int kTraceThreads = 1024;
template <class T>
__global__ void __launch_bounds__(kTraceThreads) kTraceDM(const T* __restrict__ re, int N, int slot) {
    __shared__ double part[kTraceThreads / 32];
    const uint64_t dim = 1ull << N;
    double acc = 0.0;
    for (uint64_t i = threadIdx.x; i < dim; i += kTraceThreads) acc += (double)re[i * (dim + 1)];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = part[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) g_trace[slot] = acc;
    }
}
// g_planScale = trace in / trace out (the correction of a trace-preserving plan)
__global__ void kTraceScale() {
    const double o = g_trace[1];
    g_planScale = (o != 0.0) ? g_trace[0] / o : 1.0;
}

// ------------------------------------------------------------ reductions
struct NormF32 {
    const float *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const float2 r = *reinterpret_cast<const float2*>(re + 2 * i), m = *reinterpret_cast<const float2*>(im + 2 * i);
        return make_double2((double)r.x * r.x + (double)m.x * m.x + (double)r.y * r.y + (double)m.y * m.y, 0.0);
    }
};
// Eight amplitudes per item, squared and summed in FP32, one FP64 addition
// per item.  GB300 runs FP64 at a small fraction of its FP32 rate: the
// conversions and FP64 products of NormF32 made a 30-qubit norm take ~8 ms,
// three times the read of the state.  An FP32 sum of 8 squares is within
// ~8 * 2^-24 of exact and its rounding is unbiased, so over the 2^27 items of
// 30 qubits the total moves by ~1e-11 relative.
struct NormF32x8 {
    const float *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const float4* r4 = reinterpret_cast<const float4*>(re + 8 * i);
        const float4* m4 = reinterpret_cast<const float4*>(im + 8 * i);
        const float4 a = r4[0], b = r4[1], c = m4[0], d = m4[1];
        float s = a.x * a.x;
        s = fmaf(a.y, a.y, s); s = fmaf(a.z, a.z, s); s = fmaf(a.w, a.w, s);
        s = fmaf(b.x, b.x, s); s = fmaf(b.y, b.y, s); s = fmaf(b.z, b.z, s); s = fmaf(b.w, b.w, s);
        float t = c.x * c.x;
        t = fmaf(c.y, c.y, t); t = fmaf(c.z, c.z, t); t = fmaf(c.w, c.w, t);
        t = fmaf(d.x, d.x, t); t = fmaf(d.y, d.y, t); t = fmaf(d.z, d.z, t); t = fmaf(d.w, d.w, t);
        return make_double2((double)(s + t), 0.0);
    }
};
struct ProbZeroF32 {
    const float *re, *im;
    int t;
    __device__ __forceinline__ double2 operator()(uint64_t k) const {
        const uint64_t i = ((k >> t) << (t + 1)) | (k & ((1ull << t) - 1ull));
        const double r = re[i], m = im[i];
        return make_double2(r * r + m * m, 0.0);
    }
};
// <psi64 | psi32> (complex), accumulated in FP64
struct OverlapF32 {
    const double *ar, *ai;
    const float *br, *bi;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double xr = ar[i], xi = ai[i], yr = br[i], yi = bi[i];
        return make_double2(xr * yr + xi * yi, xr * yi - xi * yr);
    }
};
__global__ void kMaxAbsDiff(const double* __restrict__ ar, const double* __restrict__ ai, const float* __restrict__ br,
                            const float* __restrict__ bi, uint64_t n, unsigned long long* __restrict__ out) {
    double m = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double dr = ar[i] - (double)br[i], di = ai[i] - (double)bi[i];
        m = fmax(m, sqrt(dr * dr + di * di));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

bool ensureStaging(QuregF32& q, size_t amps) {
    if (q.stagingAmps >= amps) return true;
    if (q.staging) cudaFree(q.staging);
    q.staging = nullptr;
    q.stagingAmps = 0;
    if (QG_CUDA(cudaMalloc(&q.staging, 2 * amps * sizeof(double)), "createQuregF32")) return false;
    q.stagingAmps = amps;
    return true;
}

QuregF32* Q(void* h) { return reinterpret_cast<QuregF32*>(h); }
}  // namespace
// read the tensor-core error flag after every plan application (one sync)
bool g_checkTC = true;
namespace {

}  // namespace
}  // namespace qg

using qg::QuregF32;

extern "C" {

void* quest_gb300_createQuregF32(int numQubits) {
    if (numQubits < 1 || numQubits > 36) return nullptr;
    QuregF32* q = new QuregF32();
    q->n = numQubits;
    const size_t n = 1ull << numQubits;
    float* base = nullptr;
    if (QG_CUDA(cudaMalloc(&base, 2 * n * sizeof(float)), "createQuregF32")) {
        delete q;
        return nullptr;
    }
    q->re = base;
    q->im = base + n;
    if (QG_CUDA(cudaMalloc(&q->scratch, qg::kScratchDoubles * sizeof(double)), "createQuregF32") ||
        QG_CUDA(cudaMallocHost(&q->host, 64 * sizeof(double)), "createQuregF32")) {
        cudaFree(base);
        delete q;
        return nullptr;
    }
    cudaMemsetAsync(q->scratch, 0, qg::kScratchDoubles * sizeof(double), qg::stream());
    quest_gb300_initZeroStateF32(q);
    return q;
}

void quest_gb300_destroyQuregF32(void* h) {
    QuregF32* q = qg::Q(h);
    if (!q) return;
    cudaStreamSynchronize(qg::stream());
    cudaFree(q->re);
    cudaFree(q->scratch);
    cudaFreeHost(q->host);
    if (q->staging) cudaFree(q->staging);
    delete q;
}

void quest_gb300_initZeroStateF32(void* h) {
    QuregF32* q = qg::Q(h);
    const size_t n = 1ull << q->n;
    cudaStream_t st = qg::stream();
    if (QG_CUDA(cudaMemsetAsync(q->re, 0, 2 * n * sizeof(float), st), "initZeroStateF32")) return;
    qg::kZeroF32<<<1, 1, 0, st>>>(q->re, q->im);
    qg::launchFailed("initZeroStateF32");
}

void quest_gb300_copyFromQureg(void* h, Qureg src) {
    QuregF32* q = qg::Q(h);
    const uint64_t n = 1ull << q->n;
    if (src.numAmpsTotal != (long long)n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "copyFromQureg");
        return;
    }
    qg::kF64toF32<<<qg::convBlocks(n), qg::kConvThreads, 0, qg::stream()>>>(src.deviceStateVec.real, src.deviceStateVec.imag,
                                                                        q->re, q->im, n);
    qg::launchFailed("copyFromQureg");
}

void quest_gb300_copyToQureg(void* h, Qureg dst) {
    QuregF32* q = qg::Q(h);
    const uint64_t n = 1ull << q->n;
    if (dst.numAmpsTotal != (long long)n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "copyToQureg");
        return;
    }
    qg::kF32toF64<<<qg::convBlocks(n), qg::kConvThreads, 0, qg::stream()>>>(q->re, q->im, dst.deviceStateVec.real,
                                                                           dst.deviceStateVec.imag, n, nullptr);
    qg::launchFailed("copyToQureg");
}


// host FP64 amplitudes -> FP32 register, through a bounded FP64 staging
// buffer on the device (chunks of at most 2^26 amplitudes)
void quest_gb300_initStateFromAmpsF32(void* h, const double* re, const double* im) {
    QuregF32* q = qg::Q(h);
    const uint64_t n = 1ull << q->n;
    const uint64_t chunk = std::min<uint64_t>(n, 1ull << 26);
    if (!qg::ensureStaging(*q, chunk)) return;
    cudaStream_t st = qg::stream();
    for (uint64_t s = 0; s < n; s += chunk) {
        const uint64_t c = std::min(chunk, n - s);
        if (QG_CUDA(cudaMemcpyAsync(q->staging, re + s, c * sizeof(double), cudaMemcpyHostToDevice, st), "initStateFromAmpsF32")) return;
        if (QG_CUDA(cudaMemcpyAsync(q->staging + chunk, im + s, c * sizeof(double), cudaMemcpyHostToDevice, st), "initStateFromAmpsF32")) return;
        qg::kF64toF32<<<qg::convBlocks(c), qg::kConvThreads, 0, st>>>(q->staging, q->staging + chunk, q->re + s, q->im + s, c);
        if (qg::launchFailed("initStateFromAmpsF32")) return;
    }
    QG_CUDA(cudaStreamSynchronize(st), "initStateFromAmpsF32");
}

void quest_gb300_copyStateToHostF32(void* h, double* re, double* im) {
    QuregF32* q = qg::Q(h);
    const uint64_t n = 1ull << q->n;
    const uint64_t chunk = std::min<uint64_t>(n, 1ull << 26);
    if (!qg::ensureStaging(*q, chunk)) return;
    cudaStream_t st = qg::stream();
    for (uint64_t s = 0; s < n; s += chunk) {
        const uint64_t c = std::min(chunk, n - s);
        qg::kF32toF64<<<qg::convBlocks(c), qg::kConvThreads, 0, st>>>(q->re + s, q->im + s, q->staging, q->staging + chunk, c,
                                                                       nullptr);
        if (qg::launchFailed("copyStateToHostF32")) return;
        if (QG_CUDA(cudaMemcpyAsync(re + s, q->staging, c * sizeof(double), cudaMemcpyDeviceToHost, st), "copyStateToHostF32")) return;
        if (QG_CUDA(cudaMemcpyAsync(im + s, q->staging + chunk, c * sizeof(double), cudaMemcpyDeviceToHost, st), "copyStateToHostF32")) return;
    }
    QG_CUDA(cudaStreamSynchronize(st), "copyStateToHostF32");
}

// Per-pass timing of plan applications (quest_gb300_setPassEvents): a CUDA
// event pair around every pass of the last application, recorded on the
// library stream from inside the pass loop.
namespace {
bool g_passEvents = false;
std::vector<cudaEvent_t> g_passEv;       // start, end of pass i at 2 i, 2 i + 1
std::vector<char> g_passRecorded;        // pass i of the last application was recorded
}  // namespace

extern "C" void quest_gb300_setPassEvents(int on) { g_passEvents = on != 0; }

extern "C" int quest_gb300_passTimesMs(double* out, int maxPasses) {
    const int n = (int)g_passRecorded.size();
    if (!out) return n;
    for (int i = 0; i < n && i < maxPasses; ++i) {
        float ms = 0.f;
        out[i] = (g_passRecorded[i] && cudaEventElapsedTime(&ms, g_passEv[2 * i], g_passEv[2 * i + 1]) == cudaSuccess)
                     ? (double)ms : -1.0;
    }
    return n;
}

// applyPlanF32Range with, when entryBound is given, sum |x|^2 of the
// register's state on the device (the first tensor-core pass's bound)
static int applyRange(void* h, void* plan, int firstPass, int numPasses, const double* entryBound) {
    QuregF32* q = qg::Q(h);
    qg::FusedPlan* p = reinterpret_cast<qg::FusedPlan*>(plan);
    if (!q || !p || p->numQubits != q->n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "applyPlanF32");
        return -1;
    }
    if (!p->compiled) qg::compilePlan(*p);
    if (!p->compiled) {
        invalidQuESTInputError("The fusion plan could not be compiled.", "applyPlanF32");
        return -1;
    }
    if (p->device && !qg::tcImagesFit(p->device)) {      // built for another precision or kernel
        p->deviceFree(p->device);
        p->device = nullptr;
    }
    if (!p->device) {
        p->device = qg::uploadPlanTC(*p);
        p->deviceFree = qg::freePlanTC;
    }
    const int total = (int)p->passes.size();
    if (firstPass < 0 || numPasses < 0 || firstPass > total) {
        invalidQuESTInputError("Pass range outside the plan.", "applyPlanF32");
        return -1;
    }
    const int last = std::min(total, firstPass + numPasses);
    cudaStream_t st = qg::stream();
    if (firstPass == 0) qg::tcBeginPlan(p->device, p->passes.size());
    qg::tcBeginRange(p->device, entryBound);
    bool usedTC = false;
    if (g_passEvents) {
        while ((int)g_passEv.size() < 2 * total) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) break;
            g_passEv.push_back(e);
        }
        if (firstPass == 0) g_passRecorded.assign(total, 0);
    }
    for (int i = firstPass; i < last; ++i) {
        const qg::FusedPass& pass = p->passes[i];
        const bool timed = g_passEvents && (int)g_passEv.size() >= 2 * total && i < (int)g_passRecorded.size();
        if (timed) cudaEventRecord(g_passEv[2 * i], st);
        const int tc = qg::applyPassTCIndexed(*q, pass, p->device, (size_t)i, st);
        if (tc < 0) return -1;
        if (tc == 0) {
            if (!pass.controls.empty()) {
                invalidQuESTInputError("fused pass with control qubits needs the tensor-core applier", "applyPlanF32");
                return -1;
            }
            if (!qg::applyPassSimt(*q, pass, st)) {
                invalidQuESTInputError("fused pass on more than 5 qubits needs the tensor-core applier", "applyPlanF32");
                return -1;
            }
            qg::tcNoteSimtPass(p->device, (size_t)i);
        } else {
            usedTC = true;
        }
        if (timed) {
            cudaEventRecord(g_passEv[2 * i + 1], st);
            g_passRecorded[i] = 1;
        }
    }
    if (usedTC && qg::g_checkTC && last == total) {
        const int e = qg::tcErrorFlag(p->device);
        if (e) {
            // codes: 1 copy of G (direct-load kernel), 2 its MMAs; pipelined
            // kernel: 3 loaders waiting for a free stage, 4 epilogue waiting for
            // an accumulator, 5 MMA issuer waiting for operands or a free
            // accumulator, 6 a non-finite split-FP16 output
            static const char* const what[] = {
                "", "tensor-core applier: operand staging timed out", "tensor-core applier: MMA completion timed out",
                "tensor-core applier: loaders timed out waiting for a free operand stage",
                "tensor-core applier: epilogue timed out waiting for an accumulator",
                "tensor-core applier: MMA issue timed out waiting for operands or an accumulator",
                "tensor-core applier: split-FP16 operands out of range (an amplitude of modulus 3.99 or more, or a "
                "non-finite state); use split-TF32"};
            invalidQuESTInputError(e >= 1 && e <= 6 ? what[e] : "tensor-core applier: timed out", "applyPlanF32");
            return -1;
        }
    }
    return 0;
}

int quest_gb300_applyPlanF32Range(void* h, void* plan, int firstPass, int numPasses) {
    return applyRange(h, plan, firstPass, numPasses, nullptr);
}

int quest_gb300_applyPlanF32(void* h, void* plan) { return quest_gb300_applyPlanF32Range(h, plan, 0, 1 << 30); }

/* norm record of pass i of the plan's last application on the tensor cores:
   in, out (FP64 sums of |amp|^2) and the square of the scale it applied;
   returns 1, or 0 if pass i has no record */
int quest_gb300_planPassNorms(void* plan, int i, double* inOutScaleSq) {
    qg::FusedPlan* p = reinterpret_cast<qg::FusedPlan*>(plan);
    if (!p || !p->device || i < 0 || !inOutScaleSq) return 0;
    return qg::tcPassNorms(p->device, (size_t)i, inOutScaleSq);
}

/* applier of pass i of the plan for registers of its size (tcKernelFor) */
int quest_gb300_planPassUsesTensorCores(void* plan, int i) {
    qg::FusedPlan* p = reinterpret_cast<qg::FusedPlan*>(plan);
    if (!p || !p->compiled || i < 0 || i >= (int)p->passes.size()) return -1;
    return qg::tcKernelFor(p->passes[i], p->numQubits);
}

void quest_gb300_setTensorCores(int enabled) { qg::setTensorCoresEnabled(enabled != 0); }
void quest_gb300_setTensorCoreKernel(int version) { qg::setTensorCoreKernel(version); }
int quest_gb300_setTensorCorePrecision(int mode) { return qg::setTensorCorePrecision(mode) ? 0 : -1; }
int quest_gb300_getTensorCorePrecision(void) { return qg::tensorCorePrecision(); }
int quest_gb300_setTensorCoreStaging(int mode) { return qg::setTensorCoreStaging(mode) ? 0 : -1; }

int quest_gb300_checkImageLayouts(void) { return qg::tcCheckImageLayouts(); }

int quest_gb300_checkHalfImages(void) { return qg::tcCheckHalfImages(); }

int quest_gb300_roundHalf(const double* values, unsigned short* out, int count) {
    if (count < 0 || (count > 0 && (!values || !out))) return -1;
    qg::tcRoundHalf(values, reinterpret_cast<uint16_t*>(out), count);
    return 0;
}

int quest_gb300_checkTileCoverage(int numQubits, const int* targets, int numTargets, const int* controls, int numControls) {
    if (!targets || numTargets < 4 || numTargets > 6 || numControls < 0 || numControls > 3 || (numControls && !controls))
        return -1;
    std::vector<int> t(targets, targets + numTargets), c(controls, controls + numControls);
    for (size_t i = 1; i < t.size(); ++i)
        if (t[i] <= t[i - 1]) return -1;
    for (size_t i = 1; i < c.size(); ++i)
        if (c[i] <= c[i - 1]) return -1;
    if (t[0] < 0 || t.back() >= numQubits || (numControls && (c[0] < 0 || c.back() >= numQubits))) return -1;
    return qg::tcCheckCoverage(numQubits, t, c);
}
int quest_gb300_getTensorCoreStaging(void) { return qg::tensorCoreStaging(); }

double quest_gb300_calcTotalProbF32(void* h) {
    QuregF32* q = qg::Q(h);
    double v = 0;
    if (q->n >= 3) qg::red::runReduce(qg::NormF32x8{q->re, q->im}, (1ull << q->n) / 8, q->w(), &v, nullptr, "calcTotalProbF32");
    else qg::red::runReduce(qg::NormF32{q->re, q->im}, (1ull << q->n) / 2, q->w(), &v, nullptr, "calcTotalProbF32");
    return v;
}

double quest_gb300_calcProbOfOutcomeF32(void* h, int t, int outcome) {
    QuregF32* q = qg::Q(h);
    if (t < 0 || t >= q->n) {
        invalidQuESTInputError("Invalid target qubit. Must be >=0 and <numQubits.", "calcProbOfOutcomeF32");
        return 0;
    }
    double v = 0;
    qg::red::runReduce(qg::ProbZeroF32{q->re, q->im, t}, (1ull << q->n) / 2, q->w(), &v, nullptr, "calcProbOfOutcomeF32");
    return outcome == 0 ? v : 1 - v;
}

// 1 - |<psi64|psi32>|^2 / (<psi64|psi64> <psi32|psi32>) and max |d amp|
double quest_gb300_compareF32(void* h, Qureg ref, double* maxAmpErr) {
    QuregF32* q = qg::Q(h);
    const uint64_t n = 1ull << q->n;
    if (ref.numAmpsTotal != (long long)n || ref.isDensityMatrix) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "compareF32");
        return -1;
    }
    double orr = 0, oi = 0;
    qg::red::runReduce(qg::OverlapF32{ref.deviceStateVec.real, ref.deviceStateVec.imag, q->re, q->im}, n, q->w(), &orr, &oi,
                       "compareF32");
    const double n32 = quest_gb300_calcTotalProbF32(h);
    const double n64 = calcTotalProb(ref);
    if (maxAmpErr) {
        unsigned long long* d = reinterpret_cast<unsigned long long*>(q->scratch + 2 * qg::kMaxReduceBlocks + 32);
        cudaStream_t st = qg::stream();
        cudaMemsetAsync(d, 0, sizeof(unsigned long long), st);
        qg::kMaxAbsDiff<<<qg::numSMs() * 8, 256, 0, st>>>(ref.deviceStateVec.real, ref.deviceStateVec.imag, q->re, q->im, n, d);
        qg::launchFailed("compareF32");
        cudaMemcpyAsync(q->host + 16, d, sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        memcpy(maxAmpErr, q->host + 16, sizeof(double));
    }
    const double f = (orr * orr + oi * oi) / (n32 * n64);
    return 1.0 - f;
}

}  // extern "C"

namespace qg {
// Trace of the FP64 density matrix (N qubits) about to be converted to FP32,
// recorded on the device for copyToQuregTraceKept
void traceBeforePlan(const double* re, int N) {
    kTraceDM<double><<<1, kTraceThreads, 0, stream()>>>(re, N, 0);
    launchFailed("captureFlush");
}

// FP32 register -> FP64 Qureg after a trace-preserving plan on a density
// matrix of N qubits: the conversion also scales by the trace before the plan
// over the trace after it, which removes the FP32 accumulation's bias (a
// near-uniform shrink of all entries) from trace and purity alike
void copyToQuregTraceKept(void* h, Qureg& dst, int N) {
    QuregF32* q = Q(h);
    const uint64_t n = 1ull << q->n;
    if (dst.numAmpsTotal != (long long)n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "copyToQureg");
        return;
    }
    double* scale = nullptr;
    if (QG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&scale), g_planScale), "copyToQureg")) return;
    kTraceDM<float><<<1, kTraceThreads, 0, stream()>>>(q->re, N, 1);
    kTraceScale<<<1, 1, 0, stream()>>>();
    kF32toF64<<<convBlocks(n), kConvThreads, 0, stream()>>>(q->re, q->im, dst.deviceStateVec.real,
                                                           dst.deviceStateVec.imag, n, scale);
    launchFailed("copyToQureg");
}

// FP64 Qureg -> FP32 register, also summing |x|^2 of the converted state on
// the device; returns where the sum is (in the register's scratch, valid
// until the register changes), or null when the conversion failed
const double* copyFromQuregNorm(void* h, const Qureg& src) {
    QuregF32* q = Q(h);
    const uint64_t n = 1ull << q->n;
    if (src.numAmpsTotal != (long long)n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "copyFromQureg");
        return nullptr;
    }
    double* slot = q->scratch + 2 * kMaxReduceBlocks + 40;
    if (QG_CUDA(cudaMemsetAsync(slot, 0, sizeof(double), stream()), "copyFromQureg")) return nullptr;
    const unsigned blocks = (unsigned)std::min<uint64_t>(convBlocks(n), 8ull * (uint64_t)numSMs());
    kF64toF32Norm<<<blocks, kConvThreads, 0, stream()>>>(src.deviceStateVec.real, src.deviceStateVec.imag, q->re, q->im,
                                                        n, slot);
    return launchFailed("copyFromQureg") ? nullptr : slot;
}

// the whole plan on the register, whose state has sum |x|^2 = *entryBound
// (device), from copyFromQuregNorm
int applyPlanF32Entry(void* h, void* plan, const double* entryBound) { return applyRange(h, plan, 0, 1 << 30, entryBound); }

// FP32 register -> FP64 Qureg after a plan: when the plan ended in a chain of
// unitary passes, the conversion also removes the norm residue of its last
// tensor-core pass (scaled back to the norm the chain started from), which no
// later pass is left to correct
void copyToQuregAfterPlan(void* h, Qureg& dst, void* plan) {
    QuregF32* q = Q(h);
    FusedPlan* p = reinterpret_cast<FusedPlan*>(plan);
    const double *target = nullptr, *out = nullptr;
    if (!q || !p || !p->device || !tcFinalNorms(p->device, &target, &out)) {
        quest_gb300_copyToQureg(h, dst);
        return;
    }
    const uint64_t n = 1ull << q->n;
    if (dst.numAmpsTotal != (long long)n) {
        invalidQuESTInputError("Dimensions of the qubit registers don't match.", "copyToQureg");
        return;
    }
    double* scale = nullptr;
    if (QG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&scale), g_planScale), "copyToQureg")) return;
    kFinalScale<<<1, 1, 0, stream()>>>(target, out);
    kF32toF64<<<convBlocks(n), kConvThreads, 0, stream()>>>(q->re, q->im, dst.deviceStateVec.real,
                                                           dst.deviceStateVec.imag, n, scale);
    launchFailed("copyToQureg");
}
}  // namespace qg

