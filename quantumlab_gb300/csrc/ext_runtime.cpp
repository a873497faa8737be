// ext_runtime.cpp -- timing / introspection extensions (include/quest_gb300.h).
#include "qg_internal.h"
#include "quest_gb300.h"

#include <atomic>
#include <mutex>

namespace qg {
std::atomic<long long> g_launches{0};
}

namespace {
constexpr int kSlots = 8192;
cudaEvent_t g_events[kSlots] = {};
std::mutex g_eventMutex;
}  // namespace

extern "C" {

void* quest_gb300_stream(void) { return (void*)qg::stream(); }

long long quest_gb300_launchCount(void) { return qg::g_launches.load(); }

int quest_gb300_eventRecord(int slot) {
    if (slot < 0 || slot >= kSlots) return -1;
    {
        std::lock_guard<std::mutex> lk(g_eventMutex);
        if (!g_events[slot] && cudaEventCreate(&g_events[slot]) != cudaSuccess) return -1;
    }
    return cudaEventRecord(g_events[slot], qg::stream()) == cudaSuccess ? 0 : -1;
}

double quest_gb300_eventElapsedMs(int a, int b) {
    if (a < 0 || a >= kSlots || b < 0 || b >= kSlots || !g_events[a] || !g_events[b]) return -1.0;
    if (cudaEventSynchronize(g_events[b]) != cudaSuccess) return -1.0;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, g_events[a], g_events[b]) != cudaSuccess) return -1.0;
    return (double)ms;
}

}  // extern "C"
