// autotune.cpp -- fusion-width autotuner of the FP32 fused engine (host C++).
// No counterpart in the reference.
//
// The cost of a fused pass depends on its width k, on the applier that runs
// it (SIMT for k <= 3, tensor cores for k = 4..6) and on whether one of its
// targets is a low qubit (< 5), which selects the staging tensor-core kernel.
// The tuner times one synthetic pass of every (k, layout) class on a scratch
// FP32 register of the requested size, keeps the table in memory and in a
// small JSON cache file, and picks for a plan the width k in {minK..maxK}
// whose compiled pass list has the lowest predicted time.
#include "fused_plan.h"
#include "qg_internal.h"
#include "quest_gb300.h"

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <vector>

namespace {

struct CostTable {
    // ms per pass, indexed [k][lowTarget]; 0 = not measured
    double ms[7][2] = {};
};

std::mutex g_tuneMutex;
std::map<int, CostTable> g_tables;   // by register size n

std::string cachePath() {
    if (const char* e = getenv("QUEST_GB300_TUNE_CACHE")) return e;
    const char* home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/quest_gb300_tune.json";
}

// cache format: {"n": {"k,low": ms, ...}, ...} -- one flat object per size
void loadCache() {
    FILE* f = fopen(cachePath().c_str(), "r");
    if (!f) return;
    std::string s;
    char buf[4096];
    size_t r;
    while ((r = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, r);
    fclose(f);
    size_t pos = 0;
    while ((pos = s.find('"', pos)) != std::string::npos) {
        const size_t end = s.find('"', pos + 1);
        if (end == std::string::npos) break;
        const std::string key = s.substr(pos + 1, end - pos - 1);
        int n = 0, k = 0, low = 0;
        double ms = 0;
        if (sscanf(key.c_str(), "n%d_k%d_low%d", &n, &k, &low) == 3 && k >= 1 && k <= 6 && (low == 0 || low == 1) &&
            sscanf(s.c_str() + end + 1, " : %lf", &ms) == 1 && ms > 0)
            g_tables[n].ms[k][low] = ms;
        pos = end + 1;
    }
}

void saveCache() {
    const std::string path = cachePath();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {           // create missing parent directories
        const std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') (void)mkdir(dir.substr(0, i).c_str(), 0755);
    }
    FILE* f = fopen(path.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n");
    bool first = true;
    for (auto& kv : g_tables)
        for (int k = 1; k <= 6; ++k)
            for (int low = 0; low < 2; ++low)
                if (kv.second.ms[k][low] > 0) {
                    fprintf(f, "%s  \"n%d_k%d_low%d\": %.6f", first ? "" : ",\n", kv.first, k, low, kv.second.ms[k][low]);
                    first = false;
                }
    fprintf(f, "\n}\n");
    fclose(f);
}

std::once_flag g_loaded;

// time one synthetic pass of width k on targets `t` (median of 3)
double timePass(void* q32, int n, const std::vector<int>& t) {
    const int k = (int)t.size(), D = 1 << k;
    std::mt19937_64 rng(1234 + k);
    std::normal_distribution<double> g;
    std::vector<double> re((size_t)D * D), im((size_t)D * D);
    for (auto& v : re) v = g(rng) / std::sqrt((double)D);
    for (auto& v : im) v = g(rng) / std::sqrt((double)D);
    void* p = quest_gb300_planCreate(n, k);
    if (!p) return 0;
    quest_gb300_planAddGate(p, t.data(), k, re.data(), im.data());
    quest_gb300_planCompile(p);
    quest_gb300_applyPlanF32(q32, p);                 // warm-up (uploads operands)
    std::vector<double> ms;
    for (int r = 0; r < 3; ++r) {
        quest_gb300_eventRecord(8190);
        quest_gb300_applyPlanF32(q32, p);
        quest_gb300_eventRecord(8191);
        ms.push_back(quest_gb300_eventElapsedMs(8190, 8191));
    }
    quest_gb300_planDestroy(p);
    std::sort(ms.begin(), ms.end());
    return ms[1];
}

}  // namespace

extern "C" {

// Measure (or load from the cache) the per-pass cost table for registers of
// numQubits qubits.  Returns 0 on success.
int quest_gb300_autotune(int numQubits) {
    std::lock_guard<std::mutex> lk(g_tuneMutex);
    std::call_once(g_loaded, loadCache);
    CostTable& t = g_tables[numQubits];
    bool missing = false;
    for (int k = 1; k <= 6; ++k)
        for (int low = 0; low < 2; ++low)
            if (k <= numQubits - (low ? 0 : 5) && !(k == 6 && numQubits < 13) && !(t.ms[k][low] > 0)) missing = true;
    if (!missing) return 0;
    void* q32 = quest_gb300_createQuregF32(numQubits);
    if (!q32) return -1;
    for (int k = 1; k <= 6 && k <= numQubits; ++k)
        for (int low = 0; low < 2; ++low) {
            if (t.ms[k][low] > 0) continue;
            if (k == 6 && numQubits < 13) continue;       // 6-qubit passes need the tensor-core applier (n >= k + 7)
            std::vector<int> targ;
            if (low) {
                for (int i = 0; i < k; ++i) targ.push_back(i * 2 < numQubits ? i * 2 : i);    // includes qubit 0
            } else {
                if (numQubits - k < 5) continue;
                for (int i = 0; i < k; ++i) targ.push_back(numQubits - 1 - 2 * i >= 5 ? numQubits - 1 - 2 * i : 5 + i);
            }
            std::sort(targ.begin(), targ.end());
            targ.erase(std::unique(targ.begin(), targ.end()), targ.end());
            if ((int)targ.size() != k) continue;
            t.ms[k][low] = timePass(q32, numQubits, targ);
        }
    quest_gb300_destroyQuregF32(q32);
    saveCache();
    return 0;
}

// Predicted time (ms) of a compiled plan from the cost table (autotune first).
double quest_gb300_planPredictMs(void* plan) {
    qg::FusedPlan* p = reinterpret_cast<qg::FusedPlan*>(plan);
    if (!p || !p->compiled) return -1;
    std::lock_guard<std::mutex> lk(g_tuneMutex);
    auto it = g_tables.find(p->numQubits);
    if (it == g_tables.end()) return -1;
    double total = 0;
    for (const auto& pass : p->passes) {
        const int k = (int)pass.targets.size();
        const int low = pass.targets[0] < 5 ? 1 : 0;
        double c = it->second.ms[k][low];
        if (!(c > 0)) c = it->second.ms[k][1 - low];
        if (!(c > 0)) return -1;
        total += c;
    }
    return total;
}

// Compile the plan at every fusion width in [minK, maxK] and keep the one
// with the lowest predicted time (measuring the cost table if needed).
// Returns the chosen width, or -1.
int quest_gb300_planCompileTuned(void* plan, int minK, int maxK) {
    qg::FusedPlan* p = reinterpret_cast<qg::FusedPlan*>(plan);
    if (!p || minK < 1 || maxK > 6 || minK > maxK) return -1;
    if (quest_gb300_autotune(p->numQubits) != 0) return -1;
    int bestK = -1;
    double best = 0;
    for (int k = minK; k <= std::min(maxK, p->numQubits); ++k) {
        p->maxFused = k;
        qg::compilePlan(*p);
        const double ms = quest_gb300_planPredictMs(plan);
        if (ms > 0 && (bestK < 0 || ms < best)) {
            best = ms;
            bestK = k;
        }
    }
    if (bestK < 0) return -1;
    p->maxFused = bestK;
    quest_gb300_planCompile(plan);
    return bestK;
}

}  // extern "C"
