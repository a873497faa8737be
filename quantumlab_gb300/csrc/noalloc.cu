// noalloc.cu -- total probability of a caller-owned FP64 state vector with
// no allocation at all (include/quest_gb300.h: quest_gb300_calcTotalProbNoAlloc).
//
// Who needs it: code that owns its amplitude arrays and must not allocate
// device memory while it runs -- for example a host callback or a worker in a
// real-time loop that is not allowed to call into the CUDA allocator, a
// process whose GPU memory is fully reserved by another framework's pool, or
// code that only borrows device pointers from its caller.  calcTotalProb()
// needs a Qureg, and creating one allocates the state, a pinned host mirror
// and reduction scratch; this entry point takes bare device pointers.
//
// How: the same single-pass reduction kernel as calcTotalProb() (one partial
// sum per block, the last block adds them in a fixed order), with its scratch
// in a file-scope __device__ array instead of memory from cudaMalloc.  The
// array is kNoAllocBlocks partial pairs plus a result pair and the
// last-block ticket (about 16.5 KB on every GPU that loads the library, held
// until exit).  A block covers at most kAmpsPerBlock amplitudes, so a call
// accepts at most kNoAllocBlocks * kAmpsPerBlock = 2^27 amplitudes (27
// qubits) and rejects larger states with an error.
//
// The kernel reads the arrays two amplitudes at a time with 16-byte loads, so
// both pointers must be 16-byte aligned (any pointer cudaMalloc returned, and
// any even offset into one); a misaligned pointer is rejected on the host
// before anything is queued.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side shadow).  The device address is looked up once per
// device, with that device current, by cudaGetSymbolAddress on the first call
// made on that device (a failed lookup is not remembered: the next call tries
// again); that first call should therefore come before any stream capture.  Every call shares the one array and leaves its contents
// behind: the ticket that must start at zero is cleared on the stream before
// each launch, and calls that overlap on the GPU (other streams, other host
// threads) race on the array -- serialise them.
#include "quest_gb300.h"
#include "reduce_kernel.cuh"

#include <stdint.h>

#include <mutex>

namespace qg {
namespace {

constexpr int kNoAllocBlocks = 1024;
constexpr int kItemsPerThread = 256;                 // items of two amplitudes
constexpr long long kAmpsPerBlock = 2ll * red::kThreads * kItemsPerThread;    // 2^17
constexpr long long kMaxAmps = kAmpsPerBlock * kNoAllocBlocks;                 // 2^27
// [partials 2*kNoAllocBlocks][result 2][ticket + padding 6]
constexpr int kScratchLen = 2 * kNoAllocBlocks + 8;

static __device__ __align__(256) double g_noallocScratch[kScratchLen];

struct NormPairs {             // sum |amp|^2, two consecutive amplitudes per item
    const double *re, *im;
    __device__ __forceinline__ double2 operator()(uint64_t i) const {
        const double2 r = *reinterpret_cast<const double2*>(re + 2 * i);
        const double2 m = *reinterpret_cast<const double2*>(im + 2 * i);
        return make_double2(r.x * r.x + m.x * m.x + r.y * r.y + m.y * m.y, 0.0);
    }
};

constexpr int kMaxDevices = 64;
double* g_scratchAddr[kMaxDevices] = {};
std::mutex g_setupMutex;

// the scratch array's device address on the current device `dev`, looked up
// on first use and kept only once the lookup has succeeded
cudaError_t scratchAddress(int dev, double** out) {
    std::lock_guard<std::mutex> lk(g_setupMutex);
    if (!g_scratchAddr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return e;
        if (!p) return cudaErrorInvalidSymbol;
        g_scratchAddr[dev] = static_cast<double*>(p);
    }
    *out = g_scratchAddr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace qg

extern "C" int quest_gb300_calcTotalProbNoAlloc(const double* deviceReal, const double* deviceImag, long long numAmps,
                                                double* result, void* stream) {
    const char* fn = "quest_gb300_calcTotalProbNoAlloc";
    using namespace qg;
    if (!deviceReal || !deviceImag || !result) {
        invalidQuESTInputError("The amplitude arrays and the result pointer must not be NULL.", fn);
        return 1;
    }
    if (numAmps < 2 || (numAmps & (numAmps - 1)) != 0) {
        invalidQuESTInputError("The number of amplitudes must be a power of two, at least 2.", fn);
        return 1;
    }
    if ((reinterpret_cast<uintptr_t>(deviceReal) & 15u) != 0 || (reinterpret_cast<uintptr_t>(deviceImag) & 15u) != 0) {
        invalidQuESTInputError("The amplitude arrays must start on a 16-byte boundary (two doubles).", fn);
        return 1;
    }
    if (numAmps > kMaxAmps) {
        invalidQuESTInputError("Too many amplitudes: this entry point's fixed scratch holds partial sums for at most "
                               "2^27 amplitudes (27 qubits); use calcTotalProb for larger registers.",
                               fn);
        return 1;
    }
    int dev = 0;
    if (cudaFailed(cudaGetDevice(&dev), "cudaGetDevice", fn)) return 1;
    if (dev < 0 || dev >= kMaxDevices) {
        invalidQuESTInputError("Device ordinal out of range for this entry point.", fn);
        return 1;
    }
    // once per device, with that device current: the array's device address
    double* partials = nullptr;
    if (cudaFailed(scratchAddress(dev, &partials), "cudaGetSymbolAddress", fn)) return 1;
    double* res = partials + 2 * kNoAllocBlocks;
    unsigned int* ticket = reinterpret_cast<unsigned int*>(res + 2);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const uint64_t items = (uint64_t)numAmps / 2;
    const uint64_t perBlock = (uint64_t)red::kThreads * kItemsPerThread;
    const unsigned grid = (unsigned)((items + perBlock - 1) / perBlock);
    if (cudaFailed(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st), "cudaMemsetAsync", fn)) return 1;
    red::kReduce<NormPairs><<<grid, red::kThreads, 0, st>>>(NormPairs{deviceReal, deviceImag}, items, partials, ticket, res);
    if (launchFailed(fn)) return 1;
    if (cudaFailed(cudaMemcpyAsync(result, res, sizeof(double), cudaMemcpyDefault, st), "cudaMemcpyAsync", fn)) return 1;
    if (cudaFailed(cudaStreamSynchronize(st), "cudaStreamSynchronize", fn)) return 1;
    return 0;
}
