// capture.cpp -- op-stream capture below the QuEST API (host C++).
//
// QuantumLab issues one QuEST call per gate (Code/QuantumLab/Circuit/QLGate.cpp:
// 652-804, PerformBasicOperation) and reads the state back only at the end of
// a circuit (Code/QuantumLab/Simulator/QLSimulatorVector.cpp:53-65).  With
// capture on for a register, its gate calls are not executed: each becomes a
// dense FP64 matrix on the <= 6 qubits it touches (targets and controls) and
// is queued.  The first call that reads or changes the register in any other
// way -- a reduction, a measurement, a copy, an initialisation, a channel,
// destroyQureg -- flushes the queue: the gates are compiled by the fusion
// planner and applied by the FP32 fused engine (FP64 state -> FP32 -> fused
// passes -> FP64), so the lab gets fusion and the tensor-core passes without a
// source change.  The result carries the FP32 engine's precision
// (1 - fidelity ~1e-11 on a 30-qubit, 20-layer circuit); capture is therefore
// off unless asked for: QUEST_GB300_CAPTURE=fp32 in the environment turns it
// on for every register created afterwards, quest_gb300_setCapture per
// register.  A gate on more than 6 qubits flushes the queue and runs directly.
#include "fused_plan.h"
#include "qg_internal.h"
#include "quest_gb300.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace qg {

struct Capture {
    int n = 0;
    int dmQubits = 0;             // N of a density matrix, 0 for a state vector
    bool tracePreserving = true;  // every queued op is a unitary gate or a channel
    std::vector<FusedGate> gates;
    void* q32 = nullptr;          // FP32 scratch register of the flushes (kept between flushes)
    long long flushes = 0, gatesApplied = 0, passesApplied = 0;
    double compileMs = 0.0;       // host time spent planning the flushes
    // The last searched plan (gates and passes, no device copy).  A flush of
    // the same circuit shape (same qubits gate by gate, at least as diagonal:
    // a repeated circuit, or new angles) takes its passes without a search.
    FusedPlan* shape = nullptr;
    long long shapeReuses = 0;
    long long shapeId = 0;        // counts the shapes searched
    // A search of the current shape with lookahead 8 on a host thread (at
    // most one at a time; registers of 26 qubits or more): a flush plans a
    // new shape without lookahead, which is ~2 % more passes but half the
    // search time, and the flushes after take the better passes once found.
    std::thread better;
    std::atomic<bool> betterDone{false};
    FusedPlan* betterPlan = nullptr;
    long long betterShapeId = -1;
};

namespace {

std::mutex g_capMutex;
std::unordered_map<const double*, Capture*> g_caps;
int g_capDefault = -1;            // -1: not read from the environment yet
int g_capMaxFused = 6;            // 0: the autotuner picks the width per searched plan

// the widest pass a flush of an n-qubit register may fuse
int capWidest(int n) { return g_capMaxFused == 0 ? widestPass(n) : std::min(g_capMaxFused, widestPass(n)); }

int defaultMode() {
    if (g_capDefault < 0) {
        const char* e = getenv("QUEST_GB300_CAPTURE");
        g_capDefault = (e && (!strcmp(e, "fp32") || !strcmp(e, "1"))) ? 1 : 0;
    }
    return g_capDefault;
}

Capture* find(const double* re) {
    auto it = g_caps.find(re);
    return it == g_caps.end() ? nullptr : it->second;
}

// the background search's result, if finished: taken as the shape when it
// is of the current shape and has fewer passes, else dropped
void adoptBetter(Capture* c) {
    if (!c->better.joinable() || !c->betterDone.load()) return;
    c->better.join();
    FusedPlan* bp = c->betterPlan;
    c->betterPlan = nullptr;
    if (bp && bp->compiled && c->shape && c->betterShapeId == c->shapeId && bp->maxFused == c->shape->maxFused &&
        bp->passSets.size() < c->shape->passSets.size()) {
        quest_gb300_planDestroy(c->shape);
        c->shape = bp;
    } else if (bp) {
        quest_gb300_planDestroy(bp);
    }
}

// start the background search of the current shape (none running)
void startBetter(Capture* c) {
    if (c->better.joinable() || !c->shape || c->n < 26) return;
    FusedPlan* bp = new FusedPlan();
    bp->numQubits = c->shape->numQubits;
    bp->maxFused = c->shape->maxFused;
    bp->maxControls = c->shape->maxControls;
    bp->beamWidth = c->shape->beamWidth;
    bp->lookahead = 8;
    bp->searchOnly = true;
    bp->gates = c->shape->gates;
    c->betterPlan = bp;
    c->betterShapeId = c->shapeId;
    c->betterDone.store(false);
    try {
        c->better = std::thread([c, bp]() {
            compilePlan(*bp);
            c->betterDone.store(true);
        });
    } catch (...) {                               // no thread to be had: no background search
        c->betterPlan = nullptr;
        quest_gb300_planDestroy(bp);
    }
}

// position of each touched qubit inside the gate's matrix index
struct Local {
    std::vector<int> qubits;      // ascending
    uint64_t loc(uint64_t mask) const {
        uint64_t r = 0;
        for (size_t b = 0; b < qubits.size(); ++b)
            if (mask >> qubits[b] & 1ull) r |= 1ull << b;
        return r;
    }
};

Local localOf(uint64_t mask) {
    Local l;
    for (int q = 0; q < 64; ++q)
        if (mask >> q & 1ull) l.qubits.push_back(q);
    return l;
}

}  // namespace

void* captureHandle(const double* re) {
    std::lock_guard<std::mutex> lk(g_capMutex);
    return find(re);
}

void captureRegister(const double* re, int n, int dmQubits) {
    std::lock_guard<std::mutex> lk(g_capMutex);
    if (defaultMode() == 1 && !find(re)) {
        Capture* c = new Capture();
        c->n = n;
        c->dmQubits = dmQubits;
        g_caps[re] = c;
    }
}

// apply and clear the queue of a capture record (caller holds no lock)
static void flushRecord(Capture* c, double* re, double* im) {
    if (!c || c->gates.empty()) return;
    if (!c->q32) c->q32 = quest_gb300_createQuregF32(c->n);
    if (!c->q32) {
        invalidQuESTInputError("Could not allocate the FP32 register of the captured gates.", "captureFlush");
        c->gates.clear();
        return;
    }
    Qureg view;
    memset(&view, 0, sizeof view);
    view.numAmpsTotal = 1LL << c->n;
    view.deviceStateVec.real = re;
    view.deviceStateVec.imag = im;
    // density matrix under trace-preserving ops only: the trace is restored
    // after the plan
    const bool keepTrace = c->dmQubits > 0 && c->tracePreserving;
    c->tracePreserving = true;
    if (keepTrace) traceBeforePlan(re, c->dmQubits);
    // the FP64 -> FP32 conversion runs on the device while the host plans;
    // with split-FP16 operands it also sums |x|^2, from which the first
    // tensor-core pass takes its scale (any state then fits FP16's range)
    const double* entryNorm = nullptr;
    if (quest_gb300_getTensorCorePrecision() == 2) entryNorm = copyFromQuregNorm(c->q32, view);
    else quest_gb300_copyFromQureg(c->q32, view);
    FusedPlan* plan = new FusedPlan();
    plan->numQubits = c->n;
    plan->maxControls = defaultMaxControls(c->n);
    const bool tuned = g_capMaxFused == 0;
    plan->maxFused = tuned && c->shape ? c->shape->maxFused : capWidest(c->n);
    plan->gates.swap(c->gates);
    const auto t0 = std::chrono::steady_clock::now();
    // No lookahead: it takes 2-3x the search time for ~2 % fewer passes (12 %
    // on first-order Trotter circuits), a loss when a flush plans a circuit
    // it runs once (a captured 100-step Trotter circuit took 412 ms with it,
    // 88 ms without)
    plan->lookahead = 0;
    adoptBetter(c);
    const bool reused = c->shape && c->shape->maxFused == plan->maxFused && compilePlanLike(*plan, *c->shape);
    if (!reused) {
        // autotuned: the width with the lowest predicted time (the cost table
        // of this register size is measured by the first such flush)
        if (!tuned || quest_gb300_planCompileTuned(plan, std::min(4, capWidest(c->n)), capWidest(c->n)) < 0) {
            plan->maxFused = capWidest(c->n);
            compilePlan(*plan);
        }
    }
    c->compileMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!plan->compiled) {
        invalidQuESTInputError("The captured gates could not be fused.", "captureFlush");
        delete plan;
        return;
    }
    if (entryNorm) applyPlanF32Entry(c->q32, plan, entryNorm);
    else quest_gb300_applyPlanF32(c->q32, plan);
    if (keepTrace) copyToQuregTraceKept(c->q32, view, c->dmQubits);
    else copyToQuregAfterPlan(c->q32, view, plan);
    c->gatesApplied += (long long)plan->gates.size();
    c->passesApplied += (long long)plan->passes.size();
    c->flushes += 1;
    if (reused) {
        c->shapeReuses += 1;
        quest_gb300_planDestroy(plan);
    } else {
        // keep the searched plan as the shape of the next flushes
        if (plan->device && plan->deviceFree) plan->deviceFree(plan->device);
        plan->device = nullptr;
        plan->passes.clear();
        if (c->shape) quest_gb300_planDestroy(c->shape);
        c->shape = plan;
        c->shapeId += 1;
        startBetter(c);
    }
}

void captureFlush(double* re, double* im) {
    Capture* c;
    {
        std::lock_guard<std::mutex> lk(g_capMutex);
        c = find(re);
    }
    flushRecord(c, re, im);
}

void captureDiscard(const double* re) {
    std::lock_guard<std::mutex> lk(g_capMutex);
    if (Capture* c = find(re)) {
        c->gates.clear();
        c->tracePreserving = true;
    }
}

void captureDrop(const double* re) {
    Capture* c = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_capMutex);
        auto it = g_caps.find(re);
        if (it != g_caps.end()) {
            c = it->second;
            g_caps.erase(it);
        }
    }
    if (c) {
        if (c->better.joinable()) c->better.join();
        if (c->betterPlan) quest_gb300_planDestroy(c->betterPlan);
        if (c->q32) quest_gb300_destroyQuregF32(c->q32);
        if (c->shape) quest_gb300_planDestroy(c->shape);
        delete c;
    }
}

// Queue the gate acting on the qubits of `mask` whose effect on a basis state
// is given by `apply` (it maps a 2^k state over the local qubits in place).
// Returns false (after flushing the queue) when the gate is wider than the
// widest pass the fused engine takes on this register: the caller then runs
// it directly.
static bool captureGate(SV s, uint64_t mask, const std::function<void(std::vector<cplx>&, const Local&)>& apply,
                        bool channel = false) {
    Capture* c = reinterpret_cast<Capture*>(s.cap);
    const Local l = localOf(mask);
    const int k = (int)l.qubits.size();
    if (k < 1 || k > capWidest(c->n)) {
        flushRecord(c, s.re, s.im);
        return false;
    }
    const int D = 1 << k;
    FusedGate g;
    g.qubits = l.qubits;
    g.m.assign((size_t)D * D, cplx(0, 0));
    std::vector<cplx> v(D);
    for (int col = 0; col < D; ++col) {
        std::fill(v.begin(), v.end(), cplx(0, 0));
        v[col] = 1;
        apply(v, l);
        for (int r = 0; r < D; ++r) g.m[(size_t)r * D + col] = v[r];
    }
    g.unitary = matrixIsUnitary(g.m, D);
    if (!g.unitary && !channel) c->tracePreserving = false;
    c->gates.push_back(std::move(g));
    return true;
}

// ---- the gate launchers' actions on a small local state -------------------
// (the same semantics as the kernels in sv_gates.cu)
bool capturePair(SV s, int target, uint64_t ctrl, uint64_t flip, const double ur[4], const double ui[4]) {
    const cplx u[4] = {cplx(ur[0], ui[0]), cplx(ur[1], ui[1]), cplx(ur[2], ui[2]), cplx(ur[3], ui[3])};
    return captureGate(s, ctrl | (1ull << target), [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t t = l.loc(1ull << target), cm = l.loc(ctrl), fm = l.loc(flip);
        for (uint64_t i = 0; i < v.size(); ++i)
            if (!(i & t) && (((i ^ fm) & cm) == cm)) {
                const cplx a = v[i], b = v[i | t];
                v[i] = u[0] * a + u[1] * b;
                v[i | t] = u[2] * a + u[3] * b;
            }
    });
}

bool captureNot(SV s, uint64_t ctrl, uint64_t targMask) {
    return captureGate(s, ctrl | targMask, [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t cm = l.loc(ctrl), tm = l.loc(targMask);
        for (uint64_t i = 0; i < v.size(); ++i)
            if ((i & cm) == cm && i < (i ^ tm)) std::swap(v[i], v[i ^ tm]);
    });
}

bool capturePhase(SV s, uint64_t mask, double tr, double ti) {
    return captureGate(s, mask, [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t m = l.loc(mask);
        for (uint64_t i = 0; i < v.size(); ++i)
            if ((i & m) == m) v[i] *= cplx(tr, ti);
    });
}

bool captureRotateZ(SV s, uint64_t ctrl, uint64_t targ, double angle) {
    return captureGate(s, ctrl | targ, [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t cm = l.loc(ctrl), tm = l.loc(targ);
        const cplx even(std::cos(angle / 2), -std::sin(angle / 2)), odd(std::cos(angle / 2), std::sin(angle / 2));
        for (uint64_t i = 0; i < v.size(); ++i)
            if ((i & cm) == cm) v[i] *= (__builtin_popcountll(i & tm) & 1) ? odd : even;
    });
}

// exp(-i angle/2 P) for the Pauli string P with X/Y/Z masks (Y bits are in
// xmask too), on amplitudes whose control bits are set; conj: elementwise
// complex conjugate of that operator.
bool capturePauliRotation(SV s, uint64_t ctrl, uint64_t xmask, uint64_t ymask, uint64_t zmask, double angle, int conj) {
    return captureGate(s, ctrl | xmask | zmask, [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t cm = l.loc(ctrl), xm = l.loc(xmask), ym = l.loc(ymask), zm = l.loc(zmask);
        const int nY = __builtin_popcountll(ym);
        static const cplx ipow[4] = {cplx(1, 0), cplx(0, 1), cplx(-1, 0), cplx(0, -1)};
        std::vector<cplx> out(v.size(), cplx(0, 0));
        const double c = std::cos(angle / 2), sn = std::sin(angle / 2);
        for (uint64_t i = 0; i < v.size(); ++i) {
            if ((i & cm) != cm) {
                out[i] += v[i];
                continue;
            }
            // P|i> = i^nY (-1)^popcount(i & (Y|Z)) |i ^ X>
            cplx ph = ipow[nY & 3] * ((__builtin_popcountll(i & (ym | zm)) & 1) ? -1.0 : 1.0);
            cplx coefDiag(c, 0), coefOff = cplx(0, -sn) * ph;
            if (conj) {
                coefDiag = std::conj(coefDiag);
                coefOff = std::conj(coefOff);
            }
            out[i] += coefDiag * v[i];
            out[i ^ xm] += coefOff * v[i];
        }
        v.swap(out);
    });
}

bool captureSwap(SV s, int q1, int q2) {
    return captureGate(s, (1ull << q1) | (1ull << q2), [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t a = l.loc(1ull << q1), b = l.loc(1ull << q2);
        for (uint64_t i = 0; i < v.size(); ++i)
            if ((i & a) && !(i & b)) std::swap(v[i], v[(i & ~a) | b]);
    });
}

bool captureChannel(SV s, int t, int N, const double S[16]) {
    return captureGate(s, (1ull << t) | (1ull << (t + N)), [&](std::vector<cplx>& v, const Local&) {
        // the two qubits are t < t + N: local bit 0 is the row qubit
        cplx out[4];
        for (int r = 0; r < 4; ++r) {
            out[r] = 0;
            for (int c = 0; c < 4; ++c) out[r] += S[4 * r + c] * v[c];
        }
        for (int r = 0; r < 4; ++r) v[r] = out[r];
    }, true);
}

bool captureChannelN(SV s, uint64_t mask, const double* S) {
    const int D = 1 << __builtin_popcountll(mask);
    return captureGate(s, mask, [&](std::vector<cplx>& v, const Local&) {
        std::vector<cplx> out(D, cplx(0, 0));
        for (int r = 0; r < D; ++r)
            for (int c = 0; c < D; ++c) out[r] += S[(size_t)D * r + c] * v[c];
        v.swap(out);
    }, true);
}

bool captureMatrixN(SV s, uint64_t ctrl, const int* targs, int k, const double* mr, const double* mi) {
    uint64_t tmask = 0;
    for (int i = 0; i < k; ++i) tmask |= 1ull << targs[i];
    return captureGate(s, ctrl | tmask, [&](std::vector<cplx>& v, const Local& l) {
        const uint64_t cm = l.loc(ctrl);
        const int D = 1 << k;
        uint64_t tl[6];
        for (int i = 0; i < k; ++i) tl[i] = l.loc(1ull << targs[i]);
        uint64_t all = 0;
        for (int i = 0; i < k; ++i) all |= tl[i];
        std::vector<cplx> x(D);
        for (uint64_t base = 0; base < v.size(); ++base) {
            if ((base & all) || (base & cm) != cm) continue;
            for (int j = 0; j < D; ++j) {
                uint64_t idx = base;
                for (int b = 0; b < k; ++b)
                    if (j >> b & 1) idx |= tl[b];
                x[j] = v[idx];
            }
            for (int r = 0; r < D; ++r) {
                cplx acc = 0;
                for (int j = 0; j < D; ++j) acc += cplx(mr[(size_t)r * D + j], mi[(size_t)r * D + j]) * x[j];
                uint64_t idx = base;
                for (int b = 0; b < k; ++b)
                    if (r >> b & 1) idx |= tl[b];
                v[idx] = acc;
            }
        }
    });
}

}  // namespace qg

extern "C" {

/* Turn capture on (mode 1: FP32 fused flush) or off (mode 0, flushing what is
 * queued) for a register; returns 0, or -1 for a density matrix or invalid
 * register.  QUEST_GB300_CAPTURE=fp32 sets mode 1 for registers created later. */
int quest_gb300_setCapture(Qureg q, int mode) {
    if (!q.deviceStateVec.real) return -1;
    if (mode == 0) {
        qg::captureFlush(q.deviceStateVec.real, q.deviceStateVec.imag);
        qg::captureDrop(q.deviceStateVec.real);
        return 0;
    }
    std::lock_guard<std::mutex> lk(qg::g_capMutex);
    if (!qg::find(q.deviceStateVec.real)) {
        qg::Capture* c = new qg::Capture();
        c->n = q.numQubitsInStateVec;
        c->dmQubits = q.isDensityMatrix ? q.numQubitsRepresented : 0;
        qg::g_caps[q.deviceStateVec.real] = c;
    }
    return 0;
}

/* Apply the register's queued gates now. */
void quest_gb300_flushCapture(Qureg q) {
    if (q.deviceStateVec.real) qg::captureFlush(q.deviceStateVec.real, q.deviceStateVec.imag);
}

/* Gates queued and not yet applied (0 when capture is off). */
int quest_gb300_capturedGates(Qureg q) {
    std::lock_guard<std::mutex> lk(qg::g_capMutex);
    qg::Capture* c = qg::find(q.deviceStateVec.real);
    return c ? (int)c->gates.size() : 0;
}

/* Totals of the register's flushes since capture was turned on. */
int quest_gb300_captureStats(Qureg q, long long* flushes, long long* gatesApplied, long long* passesApplied,
                             double* compileMs) {
    std::lock_guard<std::mutex> lk(qg::g_capMutex);
    qg::Capture* c = qg::find(q.deviceStateVec.real);
    if (!c) return -1;
    if (flushes) *flushes = c->flushes;
    if (gatesApplied) *gatesApplied = c->gatesApplied;
    if (passesApplied) *passesApplied = c->passesApplied;
    if (compileMs) *compileMs = c->compileMs;
    return 0;
}

/* Largest fused pass width used by flushes (1..6, default 6); 0: the
 * autotuner picks the width of each searched plan. */
void quest_gb300_setCaptureFusion(int maxFusedQubits) {
    if (maxFusedQubits >= 0 && maxFusedQubits <= 6) qg::g_capMaxFused = maxFusedQubits;
}

}  // extern "C"
