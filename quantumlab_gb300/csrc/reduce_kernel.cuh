// reduce_kernel.cuh -- single-pass FP64 reduction machinery shared by the
// FP64 engine (reduce.cu) and the FP32 fused engine (fused_f32.cu).
// Each thread keeps FP64 partial sums of two components; warps
// combine with shuffles, blocks through shared memory; the last block to
// finish (ticket counter in the register's scratch) adds the per-block
// partials in a fixed order, so results are deterministic.
#pragma once
#include "qg_internal.h"

#include <algorithm>

namespace qg {
namespace red {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ uint64_t ins0(uint64_t k, int b) { return ((k >> b) << (b + 1)) | (k & ((1ull << b) - 1ull)); }

// Per-thread accumulation: FP64 adds into two independent partial sums.
// GB300 executes FP64 at a small fraction of its FP32 rate, so the sums use
// no compensation terms (a Neumaier step costs ~4 extra FP64 operations per
// addition and made these kernels FP64-bound); accuracy comes from the short
// per-thread chains (about 2^n / (2 * 256 * resident blocks) terms each) and
// the pairwise block / grid combination.
struct Acc {
    double s0 = 0.0, s1 = 0.0;
    __device__ __forceinline__ void add(double x) { s0 += x; }
    __device__ __forceinline__ void add2(double x, double y) {
        s0 += x;
        s1 += y;
    }
    __device__ __forceinline__ double value() const { return s0 + s1; }
};

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// f(i) -> double2 contribution of item i.  4 items are loaded per iteration
// so every thread keeps several loads in flight.
template <class F>
__global__ void __launch_bounds__(kThreads) kReduce(F f, uint64_t nItems, double* __restrict__ partials,
                                                    unsigned int* __restrict__ counter, double* __restrict__ result) {
    __shared__ double sx[kWarps], sy[kWarps];
    __shared__ bool amLast;
    Acc ax, ay;
    const uint64_t stride = (uint64_t)gridDim.x * kThreads;
    uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    for (; i + 3 * stride < nItems; i += 4 * stride) {
        const double2 v0 = f(i), v1 = f(i + stride), v2 = f(i + 2 * stride), v3 = f(i + 3 * stride);
        ax.add2(v0.x + v2.x, v1.x + v3.x);
        ay.add2(v0.y + v2.y, v1.y + v3.y);
    }
    for (; i < nItems; i += stride) {
        const double2 v = f(i);
        ax.add(v.x); ay.add(v.y);
    }
    double x = warpSum(ax.value()), y = warpSum(ay.value());
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sx[w] = x; sy[w] = y; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bx = 0, by = 0;
        for (int k = 0; k < kWarps; ++k) { bx += sx[k]; by += sy[k]; }
        partials[2 * blockIdx.x] = bx;
        partials[2 * blockIdx.x + 1] = by;
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        amLast = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    // last block: fixed-order sum of the partials
    Acc fx, fy;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kThreads) {
        fx.add(__ldcg(partials + 2 * b));
        fy.add(__ldcg(partials + 2 * b + 1));
    }
    x = warpSum(fx.value());
    y = warpSum(fy.value());
    if (lane == 0) { sx[w] = x; sy[w] = y; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bx = 0, by = 0;
        for (int k = 0; k < kWarps; ++k) { bx += sx[k]; by += sy[k]; }
        result[0] = bx;
        result[1] = by;
        *counter = 0u;
    }
}

inline int reduceGrid(uint64_t nItems) {
    // one full wave: 256-thread blocks, 8 resident per SM (the kernel needs
    // well under 32 registers per thread)
    const uint64_t resident = 8ull * (uint64_t)numSMs();
    const uint64_t want = (nItems + kThreads - 1) / kThreads;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, std::min<uint64_t>(resident, kMaxReduceBlocks)));
}

template <class F>
inline bool runReduce(const F& f, uint64_t nItems, const Scratch& w, double* out0, double* out1, const char* caller) {
    cudaStream_t st = stream();
    const int grid = reduceGrid(nItems);
    kReduce<F><<<grid, kThreads, 0, st>>>(f, nItems, w.partials, w.counter, w.result);
    if (launchFailed(caller)) return false;
    if (QG_CUDA(cudaMemcpyAsync(w.host, w.result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st), caller)) return false;
    if (QG_CUDA(cudaStreamSynchronize(st), caller)) return false;
    if (out0) *out0 = w.host[0];
    if (out1) *out1 = w.host[1];
    return true;
}

}  // namespace red
}  // namespace qg
