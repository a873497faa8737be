// fused_plan.cpp -- gate-fusion planner (host C++) and its C ABI.
//
// Algorithm.  Gates are visited in program order while a set of "open"
// blocks with pairwise-disjoint qubit sets is maintained; each block holds the
// FP64 product of the gates it absorbed.  For a gate g on qubits Q:
//   * the open blocks touching Q are collected, largest first;
//   * while the union of Q and those blocks exceeds kmax, the largest is
//     emitted as a pass (it only holds gates that precede g);
//   * the remaining touched blocks are merged (Kronecker product; they act on
//     disjoint qubits, so they commute) and g is multiplied on.
// At the end every open block is emitted.  Invariant: for two gates sharing a
// qubit, the earlier one's pass is emitted no later than the later one's
// (the earlier gate's block is either already emitted, emitted now, or merged
// with the later gate in order), so the pass sequence equals the circuit.
#include "fused_plan.h"
#include "quest_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <list>
#include <stdexcept>

namespace qg {
namespace {

struct Block {
    uint64_t mask = 0;
    std::vector<int> qubits;   // ascending
    std::vector<cplx> m;       // D x D
    int numGates = 0;
};

// position of each qubit of `sub` inside the ascending list `all`
std::vector<int> positions(const std::vector<int>& sub, const std::vector<int>& all) {
    std::vector<int> pos(sub.size());
    for (size_t i = 0; i < sub.size(); ++i) {
        auto it = std::find(all.begin(), all.end(), sub[i]);
        pos[i] = (int)(it - all.begin());
    }
    return pos;
}

inline int extractBits(int idx, const std::vector<int>& pos) {
    int v = 0;
    for (size_t b = 0; b < pos.size(); ++b) v |= ((idx >> pos[b]) & 1) << b;
    return v;
}

// Kronecker merge of disjoint blocks into one block over the union of qubits.
Block mergeBlocks(const std::vector<const Block*>& bs, const std::vector<int>& extraQubits) {
    Block out;
    for (const Block* b : bs) out.mask |= b->mask;
    for (int q : extraQubits) out.mask |= 1ull << q;
    for (int q = 0; q < 64; ++q)
        if (out.mask >> q & 1ull) out.qubits.push_back(q);
    const int D = 1 << out.qubits.size();
    out.m.assign((size_t)D * D, cplx(0, 0));
    // mask of bits (in the merged index) that belong to no block: identity there
    int freeBits = 0;
    std::vector<std::vector<int>> pos;
    for (const Block* b : bs) {
        pos.push_back(positions(b->qubits, out.qubits));
        out.numGates += b->numGates;
    }
    int covered = 0;
    for (auto& p : pos)
        for (int x : p) covered |= 1 << x;
    freeBits = (D - 1) & ~covered;
    for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) {
            if ((r & freeBits) != (c & freeBits)) continue;
            cplx v(1, 0);
            for (size_t i = 0; i < bs.size(); ++i) {
                const int Db = 1 << bs[i]->qubits.size();
                v *= bs[i]->m[(size_t)extractBits(r, pos[i]) * Db + extractBits(c, pos[i])];
            }
            out.m[(size_t)r * D + c] = v;
        }
    return out;
}

// M <- G (embedded on its qubits) * M
void applyGate(Block& b, const FusedGate& g) {
    const int D = 1 << b.qubits.size();
    const int q = (int)g.qubits.size(), G = 1 << q;
    const std::vector<int> pos = positions(g.qubits, b.qubits);
    int gmask = 0;
    for (int p : pos) gmask |= 1 << p;
    std::vector<cplx> out((size_t)D * D);
    std::vector<int> rowOf(G);
    for (int r = 0; r < D; ++r) {
        const int rg = extractBits(r, pos);
        const int rest = r & ~gmask;
        for (int j = 0; j < G; ++j) {
            int rr = rest;
            for (int t = 0; t < q; ++t)
                if (j >> t & 1) rr |= 1 << pos[t];
            rowOf[j] = rr;
        }
        for (int c = 0; c < D; ++c) {
            cplx acc(0, 0);
            for (int j = 0; j < G; ++j) acc += g.m[(size_t)rg * G + j] * b.m[(size_t)rowOf[j] * D + c];
            out[(size_t)r * D + c] = acc;
        }
    }
    b.m.swap(out);
    b.numGates += 1;
}

void emit(FusedPlan& plan, Block& b) {
    FusedPass p;
    p.targets = b.qubits;
    p.m = std::move(b.m);
    p.numGates = b.numGates;
    plan.passes.push_back(std::move(p));
}

}  // namespace

void compilePlan(FusedPlan& plan) {
    plan.passes.clear();
    std::list<Block> open;
    for (const FusedGate& g : plan.gates) {
        uint64_t gmask = 0;
        for (int q : g.qubits) gmask |= 1ull << q;
        std::vector<std::list<Block>::iterator> touched;
        for (auto it = open.begin(); it != open.end(); ++it)
            if (it->mask & gmask) touched.push_back(it);
        std::sort(touched.begin(), touched.end(),
                  [](const std::list<Block>::iterator& a, const std::list<Block>::iterator& b) {
                      return a->qubits.size() > b->qubits.size();
                  });
        auto unionSize = [&]() {
            uint64_t m = gmask;
            for (auto& it : touched) m |= it->mask;
            return __builtin_popcountll(m);
        };
        size_t drop = 0;
        while (drop < touched.size() && unionSize() > plan.maxFused) {
            emit(plan, *touched[drop]);
            open.erase(touched[drop]);
            touched.erase(touched.begin() + drop);
        }
        std::vector<const Block*> parts;
        uint64_t covered = 0;
        for (auto& it : touched) {
            parts.push_back(&*it);
            covered |= it->mask;
        }
        std::vector<int> extra;
        for (int q : g.qubits)
            if (!(covered >> q & 1ull)) extra.push_back(q);
        Block merged = mergeBlocks(parts, extra);
        for (auto& it : touched) open.erase(it);
        applyGate(merged, g);
        open.push_back(std::move(merged));
    }
    for (Block& b : open) emit(plan, b);
    plan.compiled = true;
}

}  // namespace qg

// ============================================================ C ABI
using qg::cplx;
using qg::FusedGate;
using qg::FusedPlan;

namespace {
FusedPlan* P(void* p) { return reinterpret_cast<FusedPlan*>(p); }
int addGate(void* plan, std::vector<int> qs, std::vector<cplx> m) {
    FusedPlan* p = P(plan);
    if (!p || qs.empty() || (int)qs.size() > p->maxFused) return -1;
    for (int q : qs)
        if (q < 0 || q >= p->numQubits) return -1;
    for (size_t i = 0; i < qs.size(); ++i)
        for (size_t j = i + 1; j < qs.size(); ++j)
            if (qs[i] == qs[j]) return -1;
    p->gates.push_back(FusedGate{std::move(qs), std::move(m)});
    p->compiled = false;
    return 0;
}
}  // namespace

extern "C" {

void* quest_gb300_planCreate(int numQubits, int maxFusedQubits) {
    if (numQubits < 1 || numQubits > 40 || maxFusedQubits < 1 || maxFusedQubits > 6) return nullptr;
    FusedPlan* p = new FusedPlan();
    p->numQubits = numQubits;
    p->maxFused = std::min(maxFusedQubits, numQubits);
    return p;
}

void quest_gb300_planDestroy(void* plan) {
    FusedPlan* p = P(plan);
    if (!p) return;
    if (p->device && p->deviceFree) p->deviceFree(p->device);
    delete p;
}

int quest_gb300_planAddGate(void* plan, const int* targets, int numTargets, const double* re, const double* im) {
    if (numTargets < 1 || numTargets > 6) return -1;
    const int D = 1 << numTargets;
    std::vector<cplx> m((size_t)D * D);
    for (int i = 0; i < D * D; ++i) m[i] = cplx(re[i], im[i]);
    return addGate(plan, std::vector<int>(targets, targets + numTargets), std::move(m));
}

int quest_gb300_planAddCompactUnitary(void* plan, int t, double ar, double ai, double br, double bi) {
    // [alpha, -conj(beta); beta, conj(alpha)]
    return addGate(plan, {t}, {cplx(ar, ai), cplx(-br, bi), cplx(br, bi), cplx(ar, -ai)});
}

int quest_gb300_planAddUnitary(void* plan, int t, const double* re4, const double* im4) {
    return addGate(plan, {t}, {cplx(re4[0], im4[0]), cplx(re4[1], im4[1]), cplx(re4[2], im4[2]), cplx(re4[3], im4[3])});
}

int quest_gb300_planAddHadamard(void* plan, int t) {
    const double f = 1.0 / std::sqrt(2.0);
    return addGate(plan, {t}, {cplx(f, 0), cplx(f, 0), cplx(f, 0), cplx(-f, 0)});
}

int quest_gb300_planAddControlledNot(void* plan, int c, int t) {
    // bit 0 = control, bit 1 = target: swap |01> (c=1,t=0) and |11>
    std::vector<cplx> m(16, cplx(0, 0));
    m[0 * 4 + 0] = 1; m[2 * 4 + 2] = 1;
    m[1 * 4 + 3] = 1; m[3 * 4 + 1] = 1;
    return addGate(plan, {c, t}, std::move(m));
}

int quest_gb300_planAddControlledPhaseShift(void* plan, int a, int b, double theta) {
    std::vector<cplx> m(16, cplx(0, 0));
    m[0] = 1; m[5] = 1; m[10] = 1;
    m[15] = cplx(std::cos(theta), std::sin(theta));
    return addGate(plan, {a, b}, std::move(m));
}

int quest_gb300_planCompile(void* plan) {
    FusedPlan* p = P(plan);
    if (!p) return -1;
    if (p->device && p->deviceFree) p->deviceFree(p->device);
    p->device = nullptr;
    qg::compilePlan(*p);
    return (int)p->passes.size();
}

int quest_gb300_planNumGates(void* plan) { return P(plan) ? (int)P(plan)->gates.size() : -1; }

int quest_gb300_planPass(void* plan, int i, int* targets, double* re, double* im) {
    FusedPlan* p = P(plan);
    if (!p || !p->compiled || i < 0 || i >= (int)p->passes.size()) return -1;
    const qg::FusedPass& s = p->passes[i];
    const int k = (int)s.targets.size();
    if (targets)
        for (int b = 0; b < k; ++b) targets[b] = s.targets[b];
    if (re && im)
        for (size_t e = 0; e < s.m.size(); ++e) {
            re[e] = s.m[e].real();
            im[e] = s.m[e].imag();
        }
    return k;
}

}  // extern "C"
