// fused_plan.cpp -- gate-fusion planner (host C++) and its C ABI.
//
// A plan is a sequence of passes.  A pass is a set S of at most kmax qubits
// and the FP64 product of the gates it absorbs.  Every pass costs one sweep of
// the state, whatever it holds, so the planner minimises the number of passes.
//
// Order constraints.  A gate is "diagonal on qubit q" when its matrix has no
// entry that changes the value of q.  Examples are a phase gate, either qubit
// of a controlled phase, and the control of a CNOT.  Two gates that meet only
// on qubits where both are diagonal commute.  For each qubit, the gates on it
// are cut into segments: a maximal run of consecutive gates that are all
// diagonal on it, or a single gate that is not.  A gate may run once all gates
// of the earlier segments of each of its qubits have run.  Gates that this
// rule leaves unordered share only qubits where both are diagonal, so they
// commute.  Every order the rule allows therefore gives the same product.
//
// Search.  Passes are chosen one at a time from the front of the remaining
// circuit.  The closure of a qubit set S is every remaining gate that can run,
// in some allowed order, using only the qubits of S.
//   * The beam starts from the single live qubits.
//   * Each level grows each set by whole gates: by the qubits of the next
//     multi-qubit gate on one of its members, all at once.  A 3-qubit gate
//     added one qubit at a time would pass through sets that absorb nothing
//     new, which tie and crowd the beam.  When no member has such a gate,
//     the set grows by any one live qubit.
//   * Each level keeps the `beam` best sets, ranked by multi-qubit gates
//     absorbed, then by gates absorbed, then by least advanced qubits first.
//   * The best set found becomes the pass and its closure is applied.  With
//     lookahead L (default 4), the L best distinct sets of the search are
//     each applied on a copy of the search state and followed by one more
//     search; the set whose two passes absorb the most multi-qubit gates,
//     then gates, becomes the pass.  On 30-qubit random circuits this saves
//     ~2 % of the passes (65 -> 64 at seed 2; 730 -> 713 over 12 circuits of
//     26-30 qubits); on the first-order Hubbard circuit, 58 -> 51 passes.
// The search repeats until every gate is absorbed.  Take 30-qubit random
// circuits of Haar one-qubit gates, random-matching controlled phases and CNOT
// brickwork, at kmax = 6.  Merging gates into open blocks in program order
// takes ~130 passes for 20 layers; this search takes ~100.  On 10 first-order
// Trotter steps of the 12-site Fermi-Hubbard chain (24 qubits, 2- and 3-qubit
// Pauli rotations) it takes 58 passes; growing by one qubit per level took 96.
//
// Products.  A pass matrix is built in split real/imaginary planes.  Each
// absorbed gate multiplies on from the left, using only its nonzero entries.
// The inner loop runs over the D matrix columns.  Once the search has fixed
// the passes, their products are independent and are shared among up to 16
// host threads.
#include "fused_plan.h"
#include "quest_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_set>

namespace qg {
namespace {

constexpr int kDepth = 1;   // multi-qubit gates per member looked at for candidates

struct GateInfo {
    uint64_t mask = 0;
    uint64_t diag = 0;      // qubits on which the gate is diagonal
    int nq = 0;
    int q[6];
    int seg[6];             // segment of the gate on q[t]
};

// qubits of g on which its matrix is block-diagonal (exact zeros elsewhere)
uint64_t diagonalQubits(const FusedGate& g) {
    const int m = (int)g.qubits.size(), G = 1 << m;
    uint64_t d = 0;
    for (int b = 0; b < m; ++b) {
        bool ok = true;
        for (int r = 0; r < G && ok; ++r)
            for (int c = 0; c < G; ++c)
                if (((r ^ c) >> b & 1) && g.m[(size_t)r * G + c] != cplx(0, 0)) {
                    ok = false;
                    break;
                }
        if (ok) d |= 1ull << g.qubits[b];
    }
    return d;
}

struct Scored {
    uint64_t set = 0;
    int multi = 0, all = 0, lag = 0;
    // growth candidates: the qubits outside the set of the next multi-qubit
    // gate on each member (whole gates, so a 3-qubit gate is not split over
    // levels at which nothing new is absorbed)
    uint64_t ext[8] = {};
    int next = 0;
};

bool better(const Scored& a, const Scored& b) {
    if (a.multi != b.multi) return a.multi > b.multi;
    if (a.all != b.all) return a.all > b.all;
    if (a.lag != b.lag) return a.lag < b.lag;
    return a.set < b.set;
}

class Search {
  public:
    Search(const std::vector<FusedGate>& gates, int numQubits, int kmax, int beam, int maxCtl, int look)
        : nq_(numQubits), kmax_(kmax), beam_(std::max(1, beam)), maxCtl_(maxCtl), look_(look), g_(gates.size()),
          byq_(numQubits),
          segStart_(numQubits), cur_(numQubits, 0), rem_(numQubits, 0), applied_(gates.size(), 0),
          stamp_(gates.size(), 0), remaining_((int)gates.size()) {
        std::vector<int> lastDiag(numQubits, 0);
        for (size_t i = 0; i < gates.size(); ++i) {
            const FusedGate& fg = gates[i];
            GateInfo& gi = g_[i];
            const uint64_t diag = diagonalQubits(fg);
            gi.diag = diag;
            gi.nq = (int)fg.qubits.size();
            for (int t = 0; t < gi.nq; ++t) {
                const int q = fg.qubits[t];
                gi.q[t] = q;
                gi.mask |= 1ull << q;
                const int d = (int)(diag >> q & 1);
                // a new segment unless this gate and the previous one on q are both diagonal on q
                if (!(d && lastDiag[q] && !byq_[q].empty())) segStart_[q].push_back((int)byq_[q].size());
                gi.seg[t] = (int)segStart_[q].size() - 1;
                byq_[q].push_back((int)i);
                lastDiag[q] = d;
            }
        }
        for (int q = 0; q < nq_; ++q) {
            segStart_[q].push_back((int)byq_[q].size());
            rem_[q] = nseg(q) > 0 ? segSize(q, 0) : 0;
            if (nseg(q) > 0) live_ |= 1ull << q;
        }
    }

    bool done() const { return remaining_ == 0; }

    // choose the next pass, apply its closure; returns its qubit set (0 on
    // failure), the absorbed gates in an allowed order and the pass's
    // control qubits
    uint64_t next(std::vector<int>& absorbed, uint64_t& controls) {
        const int look = look_;
        std::vector<Scored> finalists;
        Scored best;
        bool have = search(best, look > 0 ? &finalists : nullptr);
        if (look > 0 && have && finalists.size() > 1) {
            std::sort(finalists.begin(), finalists.end(), better);
            std::vector<uint64_t> uniq;
            int bestTotal = -1, bestMulti = -1;
            for (const Scored& f : finalists) {
                if (std::find(uniq.begin(), uniq.end(), f.set) != uniq.end()) continue;
                uniq.push_back(f.set);
                if ((int)uniq.size() > look) break;
                Search copy(*this);
                std::vector<int> abs;
                copy.closure(f.set, &abs, nullptr, true);
                Scored nb;
                const bool h2 = !copy.done() && copy.search(nb, nullptr);
                const int tm = f.multi + (h2 ? nb.multi : 0), ta = f.all + (h2 ? nb.all : 0);
                if (tm > bestMulti || (tm == bestMulti && ta > bestTotal)) {
                    bestMulti = tm;
                    bestTotal = ta;
                    best = f;
                }
            }
        }
        uint64_t S = best.set;
        if (!have || best.all == 0) {
            // the earliest remaining gate can always run: every gate before it has run
            while (applied_[first_]) ++first_;
            S = g_[first_].mask;
        }
        absorbed.clear();
        controls = closure(S, &absorbed, nullptr, true);
        return absorbed.empty() ? 0 : S;     // 0: no progress (cannot happen, see above)
    }

    // the beam search of one pass; false when no set was scored
    bool search(Scored& best, std::vector<Scored>* finalists) {
        std::vector<Scored> beam, cand;
        std::unordered_set<uint64_t> seen;
        for (int q = 0; q < nq_; ++q)
            if (live_ >> q & 1) cand.push_back(eval(1ull << q));
        bool have = false;
        for (int level = 1;; ++level) {
            if (cand.empty()) break;
            const size_t keep = std::min(cand.size(), (size_t)beam_);
            std::partial_sort(cand.begin(), cand.begin() + keep, cand.end(), better);
            cand.resize(keep);
            beam.swap(cand);
            if (finalists) finalists->insert(finalists->end(), beam.begin(), beam.end());
            if (!have || better(beam[0], best)) best = beam[0];
            have = true;
            if (level >= kmax_) break;
            cand.clear();
            seen.clear();
            for (const Scored& b : beam) {
                if (b.next > 0) {
                    for (int e = 0; e < b.next; ++e) {
                        const uint64_t t = b.set | b.ext[e];
                        if (__builtin_popcountll(t) <= kmax_ && seen.insert(t).second) cand.push_back(eval(t));
                    }
                } else if (__builtin_popcountll(b.set) < kmax_) {
                    for (uint64_t pm = live_ & ~b.set; pm; pm &= pm - 1) {
                        const uint64_t t = b.set | (pm & (~pm + 1));
                        if (seen.insert(t).second) cand.push_back(eval(t));
                    }
                }
            }
        }
        return have;
    }

  private:
    int nseg(int q) const { return (int)segStart_[q].size() - 1; }
    int segSize(int q, int s) const { return segStart_[q][s + 1] - segStart_[q][s]; }

    Scored eval(uint64_t S) {
        Scored s;
        s.set = S;
        closure(S, nullptr, &s, false);
        return s;
    }

    // Closure of S from the current front.  With `commit` the absorbed gates
    // are marked as run and the front moves past them.  With maxCtl > 0 and
    // at least four qubits in S, a gate may also use up to maxCtl qubits
    // outside S on which it is diagonal ("controls"): each must lie outside
    // the pass's tile (at least 7 qubits outside S below it), so that it is
    // constant over every tile and the pass applies one of 2^controls
    // matrices per tile.  Returns the controls used.
    uint64_t closure(uint64_t S, std::vector<int>* out, Scored* sc, bool commit) {
        if (++stampId_ == 0) {
            std::fill(stamp_.begin(), stamp_.end(), 0u);
            stampId_ = 1;
        }
        const uint32_t id = stampId_;
        int qs[64], nS = 0;
        int lcur[64], lrem[64];
        for (uint64_t m = S; m; m &= m - 1) {
            const int q = __builtin_ctzll(m);
            qs[nS++] = q;
            lcur[q] = cur_[q];
            lrem[q] = rem_[q];
        }
        int multi = 0, all = 0;
        uint64_t ctl = 0, touched = S;
        const bool allowCtl = maxCtl_ > 0 && nS >= 4;
        auto validCtl = [&](int c) { return c - __builtin_popcountll(S & ((1ull << c) - 1ull)) >= 7; };
        bool changed = true;
        while (changed) {
            changed = false;
            for (int a = 0; a < nS; ++a) {
                const int q = qs[a];
                bool advanced = true;
                while (advanced && lcur[q] < nseg(q)) {
                    advanced = false;
                    const int s = lcur[q];
                    for (int j = segStart_[q][s]; j < segStart_[q][s + 1] && !advanced; ++j) {
                        const int i = byq_[q][j];
                        if (applied_[i] || stamp_[i] == id) continue;
                        const GateInfo& gi = g_[i];
                        const uint64_t outside = gi.mask & ~S;
                        if (outside) {
                            if (!allowCtl || (outside & ~gi.diag) ||
                                __builtin_popcountll(ctl | outside) > maxCtl_)
                                continue;
                            bool ok = true;
                            for (uint64_t m = outside; m && ok; m &= m - 1) ok = validCtl(__builtin_ctzll(m));
                            if (!ok) continue;
                            for (uint64_t m = outside & ~touched; m; m &= m - 1) {
                                const int c = __builtin_ctzll(m);
                                lcur[c] = cur_[c];
                                lrem[c] = rem_[c];
                            }
                            touched |= outside;
                        }
                        bool ready = true;
                        for (int t = 0; t < gi.nq && ready; ++t) ready = gi.seg[t] == lcur[gi.q[t]];
                        if (!ready) continue;
                        stamp_[i] = id;
                        if (out) out->push_back(i);
                        ++all;
                        multi += gi.nq > 1;
                        ctl |= outside;
                        changed = true;
                        for (int t = 0; t < gi.nq; ++t) {
                            const int x = gi.q[t];
                            if (--lrem[x] == 0) {
                                ++lcur[x];
                                lrem[x] = lcur[x] < nseg(x) ? segSize(x, lcur[x]) : 0;
                                if (x == q) advanced = true;
                            }
                        }
                    }
                }
            }
        }
        if (sc) {
            sc->multi = multi;
            sc->all = all;
            int lag = 0;
            sc->next = 0;
            for (int a = 0; a < nS; ++a) {
                const int q = qs[a];
                lag += cur_[q];
                int found = 0;
                if (lcur[q] >= nseg(q)) continue;
                for (int j = segStart_[q][lcur[q]]; j < (int)byq_[q].size() && found < kDepth; ++j) {
                    const int i = byq_[q][j];
                    if (applied_[i] || stamp_[i] == id || g_[i].nq < 2) continue;
                    ++found;
                    const uint64_t e = g_[i].mask & ~S;
                    bool dup = (e == 0);
                    for (int x = 0; x < sc->next && !dup; ++x) dup = sc->ext[x] == e;
                    if (!dup && sc->next < 8) sc->ext[sc->next++] = e;
                }
            }
            sc->lag = lag;
        }
        if (commit) {
            for (int i : *out) applied_[i] = 1;
            for (uint64_t m = S | ctl; m; m &= m - 1) {
                const int q = __builtin_ctzll(m);
                cur_[q] = lcur[q];
                rem_[q] = lrem[q];
                if (cur_[q] >= nseg(q)) live_ &= ~(1ull << q);
            }
            remaining_ -= all;
        }
        return ctl;
    }

    int nq_, kmax_, beam_, maxCtl_, look_;
    std::vector<GateInfo> g_;
    std::vector<std::vector<int>> byq_;       // gates on each qubit, program order
    std::vector<std::vector<int>> segStart_;  // per qubit: first index in byq_ of each segment, then byq_.size()
    std::vector<int> cur_, rem_;              // per qubit: current segment and its gates not yet run
    std::vector<uint8_t> applied_;
    std::vector<uint32_t> stamp_;
    uint32_t stampId_ = 0;
    uint64_t live_ = 0;                       // qubits with gates left
    int remaining_;
    size_t first_ = 0;
};

// M <- G M, G embedded on bit positions pos[] of the pass index; M is D x D
// (row-major, split planes); tr/ti hold the 2^m rows of one group
void mulGate(double* __restrict Mr, double* __restrict Mi, int D, const FusedGate& g, const int* pos,
             double* __restrict tr, double* __restrict ti) {
    const int m = (int)g.qubits.size(), G = 1 << m;
    int off[64];
    int gmask = 0;
    for (int b = 0; b < m; ++b) gmask |= 1 << pos[b];
    for (int a = 0; a < G; ++a) {
        off[a] = 0;
        for (int b = 0; b < m; ++b)
            if (a >> b & 1) off[a] |= 1 << pos[b];
    }
    // nonzero entries of each row of G
    std::vector<int> nzStart(G + 1, 0), nzCol;
    std::vector<double> nzRe, nzIm;
    for (int a = 0; a < G; ++a) {
        for (int b = 0; b < G; ++b) {
            const cplx v = g.m[(size_t)a * G + b];
            if (v == cplx(0, 0)) continue;
            nzCol.push_back(b);
            nzRe.push_back(v.real());
            nzIm.push_back(v.imag());
        }
        nzStart[a + 1] = (int)nzCol.size();
    }
    for (int r0 = 0; r0 < D; ++r0) {
        if (r0 & gmask) continue;
        for (int a = 0; a < G; ++a) {
            memcpy(tr + (size_t)a * D, Mr + (size_t)(r0 | off[a]) * D, sizeof(double) * D);
            memcpy(ti + (size_t)a * D, Mi + (size_t)(r0 | off[a]) * D, sizeof(double) * D);
        }
        for (int a = 0; a < G; ++a) {
            double* __restrict orow = Mr + (size_t)(r0 | off[a]) * D;
            double* __restrict oirow = Mi + (size_t)(r0 | off[a]) * D;
            for (int c = 0; c < D; ++c) orow[c] = oirow[c] = 0;
            for (int e = nzStart[a]; e < nzStart[a + 1]; ++e) {
                const double gr = nzRe[e], gi = nzIm[e];
                const double* __restrict sr = tr + (size_t)nzCol[e] * D;
                const double* __restrict si = ti + (size_t)nzCol[e] * D;
                for (int c = 0; c < D; ++c) {
                    orow[c] += gr * sr[c] - gi * si[c];
                    oirow[c] += gr * si[c] + gi * sr[c];
                }
            }
        }
    }
}

}  // namespace

bool tensorCoresEnabled();   // fused_tc.cu
int defaultMaxControls(int n) { return (n >= 26 && tensorCoresEnabled()) ? 3 : 0; }

bool matrixIsUnitary(const std::vector<cplx>& m, int D) {
    for (int r = 0; r < D; ++r)
        for (int c = r; c < D; ++c) {
            double ar = 0, ai = 0;
            for (int j = 0; j < D; ++j) {
                const cplx a = m[(size_t)r * D + j], b = m[(size_t)c * D + j];
                ar += a.real() * b.real() + a.imag() * b.imag();     // a conj(b)
                ai += a.imag() * b.real() - a.real() * b.imag();
            }
            if (std::fabs(ar - (r == c ? 1.0 : 0.0)) > 1e-12 || std::fabs(ai) > 1e-12) return false;
        }
    return true;
}

// The block of g (diagonal on the qubits of `ctl` it touches) for the values
// `val` of those qubits (bit j of val <-> the j-th qubit of ctl): a gate on
// g's other qubits.
FusedGate controlBlock(const FusedGate& g, uint64_t ctl, uint32_t val) {
    FusedGate sub;
    const int m = (int)g.qubits.size();
    uint32_t fixedVal = 0;
    int keep[6], nk = 0;
    for (int b = 0; b < m; ++b) {
        const int q = g.qubits[b];
        if (ctl >> q & 1ull) {
            const int j = __builtin_popcountll(ctl & ((1ull << q) - 1ull));
            if (val >> j & 1u) fixedVal |= 1u << b;
        } else {
            keep[nk++] = b;
            sub.qubits.push_back(q);
        }
    }
    const int G = 1 << m, Gs = 1 << nk;
    auto expand = [&](int r) {
        int x = (int)fixedVal;
        for (int t = 0; t < nk; ++t)
            if (r >> t & 1) x |= 1 << keep[t];
        return x;
    };
    sub.m.resize((size_t)Gs * Gs);
    for (int r = 0; r < Gs; ++r)
        for (int c = 0; c < Gs; ++c) sub.m[(size_t)r * Gs + c] = g.m[(size_t)expand(r) * G + expand(c)];
    sub.unitary = g.unitary;
    return sub;
}

// products of the absorbed gates of one pass on its qubit set S, one per
// value of its control qubits `ctl`
void buildPass(const FusedPlan& plan, uint64_t S, uint64_t ctl, const std::vector<int>& absorbed, FusedPass& p) {
    p.targets.clear();
    p.controls.clear();
    for (int q = 0; q < 64; ++q) {
        if (S >> q & 1) p.targets.push_back(q);
        if (ctl >> q & 1) p.controls.push_back(q);
    }
    const int k = (int)p.targets.size(), D = 1 << k;
    const uint32_t nv = 1u << p.controls.size();
    int posOf[64];
    for (int b = 0; b < k; ++b) posOf[p.targets[b]] = b;
    std::vector<double> Mr((size_t)D * D), Mi((size_t)D * D), tr((size_t)64 * D), ti((size_t)64 * D);
    p.m.resize((size_t)nv * D * D);
    for (uint32_t v = 0; v < nv; ++v) {
        std::fill(Mr.begin(), Mr.end(), 0.0);
        std::fill(Mi.begin(), Mi.end(), 0.0);
        for (int r = 0; r < D; ++r) Mr[(size_t)r * D + r] = 1.0;
        for (int i : absorbed) {
            const FusedGate& g0 = plan.gates[i];
            uint64_t gm = 0;
            for (int q : g0.qubits) gm |= 1ull << q;
            const FusedGate sub = (gm & ctl) ? controlBlock(g0, ctl, v) : FusedGate{};
            const FusedGate& g = (gm & ctl) ? sub : g0;
            int pos[6];
            for (size_t t = 0; t < g.qubits.size(); ++t) pos[t] = posOf[g.qubits[t]];
            mulGate(Mr.data(), Mi.data(), D, g, pos, tr.data(), ti.data());
        }
        cplx* blk = p.m.data() + (size_t)v * D * D;
        for (size_t e = 0; e < (size_t)D * D; ++e) blk[e] = cplx(Mr[e], Mi[e]);
    }
    p.numGates = (int)absorbed.size();
    p.unitary = true;
    for (int i : absorbed) p.unitary = p.unitary && plan.gates[i].unitary;
}

void compilePlan(FusedPlan& plan) {
    plan.passes.clear();
    std::vector<uint64_t> sets, ctls;
    std::vector<std::vector<int>> members;
    {
        Search search(plan.gates, plan.numQubits, plan.maxFused, plan.beamWidth, plan.maxControls, plan.lookahead);
        std::vector<int> absorbed;
        uint64_t ctl = 0;
        while (!search.done()) {
            sets.push_back(search.next(absorbed, ctl));
            if (!sets.back()) {
                plan.compiled = false;
                return;
            }
            ctls.push_back(ctl);
            members.push_back(absorbed);
        }
    }
    plan.passSets = sets;
    plan.passControls = ctls;
    plan.passMembers = members;
    if (plan.searchOnly) {
        plan.compiled = true;                 // a structure for compilePlanLike
        return;
    }
    // the pass products are independent: a few host threads share them
    const size_t np = sets.size();
    plan.passes.resize(np);
    std::atomic<size_t> nextPass{0};
    auto work = [&]() {
        for (size_t i; (i = nextPass.fetch_add(1)) < np;) buildPass(plan, sets[i], ctls[i], members[i], plan.passes[i]);
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::min<size_t>({(size_t)std::min(hw, 16u), np, 1 + plan.gates.size() / 64});
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
    plan.compiled = true;
}

bool compilePlanLike(FusedPlan& plan, const FusedPlan& structure) {
    plan.compiled = false;
    plan.passes.clear();
    if (!structure.compiled || plan.gates.size() != structure.gates.size() || plan.numQubits != structure.numQubits)
        return false;
    for (size_t i = 0; i < plan.gates.size(); ++i) {
        const FusedGate &a = plan.gates[i], &b = structure.gates[i];
        if (a.qubits != b.qubits) return false;
        const uint64_t da = diagonalQubits(a), db = diagonalQubits(b);
        if ((db & ~da) != 0) return false;
    }
    plan.passSets = structure.passSets;
    plan.passControls = structure.passControls;
    plan.passMembers = structure.passMembers;
    const size_t np = plan.passSets.size();
    plan.passes.resize(np);
    std::atomic<size_t> nextPass{0};
    auto work = [&]() {
        for (size_t i; (i = nextPass.fetch_add(1)) < np;)
            buildPass(plan, plan.passSets[i], plan.passControls[i], plan.passMembers[i], plan.passes[i]);
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::min<size_t>({(size_t)std::min(hw, 16u), np, 1 + plan.gates.size() / 64});
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
    plan.compiled = true;
    return true;
}

FusedGate pauliRotationGate(uint64_t x, uint64_t y, uint64_t z, double angle) {
    FusedGate g;
    const uint64_t mask = x | z;
    for (uint64_t m = mask; m; m &= m - 1) g.qubits.push_back(__builtin_ctzll(m));
    const int k = (int)g.qubits.size();
    const uint64_t D = 1ull << k;
    // the masks on the gate's local qubits (bit b <-> qubits[b])
    auto local = [&](uint64_t v) {
        uint64_t r = 0;
        for (int b = 0; b < k; ++b)
            if (v >> g.qubits[b] & 1ull) r |= 1ull << b;
        return r;
    };
    const uint64_t xm = local(x), ym = local(y), zm = local(z);
    static const cplx ipow[4] = {cplx(1, 0), cplx(0, 1), cplx(-1, 0), cplx(0, -1)};
    const cplx iy = ipow[__builtin_popcountll(ym) & 3];
    const double c = std::cos(angle / 2), sn = std::sin(angle / 2);
    g.m.assign(D * D, cplx(0, 0));
    for (uint64_t i = 0; i < D; ++i) {
        // P|i> = i^nY (-1)^popcount(i & (Y|Z)) |i ^ X>
        const cplx ph = iy * ((__builtin_popcountll(i & (ym | zm)) & 1) ? -1.0 : 1.0);
        g.m[i * D + i] += c;
        g.m[(i ^ xm) * D + i] += cplx(0, -sn) * ph;
    }
    g.unitary = matrixIsUnitary(g.m, (int)D);
    return g;
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
    const bool u = qg::matrixIsUnitary(m, 1 << (int)qs.size());
    p->gates.push_back(FusedGate{std::move(qs), std::move(m), u});
    p->compiled = false;
    return 0;
}
}  // namespace

extern "C" {

void* quest_gb300_planCreate(int numQubits, int maxFusedQubits) {
    if (numQubits < 1 || numQubits > 40 || maxFusedQubits < 1 || maxFusedQubits > 6) return nullptr;
    FusedPlan* p = new FusedPlan();
    p->numQubits = numQubits;
    p->maxFused = std::min(maxFusedQubits, qg::widestPass(numQubits));
    p->maxControls = qg::defaultMaxControls(numQubits);
    // from 28 qubits a pass costs ~0.7-2.8 ms: 8 candidates (about 1.5x the
    // search time of 4) save ~1 more pass on the 30-qubit random circuit
    p->lookahead = numQubits >= 28 ? 8 : 4;
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

int quest_gb300_planSetBeamWidth(void* plan, int width) {
    FusedPlan* p = P(plan);
    if (!p || width < 1 || width > 256) return -1;
    p->beamWidth = width;
    p->compiled = false;
    return 0;
}

int quest_gb300_planSetLookahead(void* plan, int candidates) {
    FusedPlan* p = P(plan);
    if (!p || candidates < 0 || candidates > 16) return -1;
    p->lookahead = candidates;
    p->compiled = false;
    return 0;
}

int quest_gb300_planSetMaxControls(void* plan, int maxControls) {
    FusedPlan* p = P(plan);
    if (!p || maxControls < 0 || maxControls > 3) return -1;
    p->maxControls = maxControls;
    p->compiled = false;
    return 0;
}

int quest_gb300_planPassControls(void* plan, int i, int* controls) {
    FusedPlan* p = P(plan);
    if (!p || !p->compiled || i < 0 || i >= (int)p->passes.size()) return -1;
    const qg::FusedPass& s = p->passes[i];
    if (controls)
        for (size_t j = 0; j < s.controls.size(); ++j) controls[j] = s.controls[j];
    return (int)s.controls.size();
}

int quest_gb300_planCompile(void* plan) {
    FusedPlan* p = P(plan);
    if (!p) return -1;
    if (p->device && p->deviceFree) p->deviceFree(p->device);
    p->device = nullptr;
    qg::compilePlan(*p);
    return p->compiled ? (int)p->passes.size() : -1;
}

int quest_gb300_planCompileLike(void* plan, void* structure) {
    FusedPlan* p = P(plan);
    const FusedPlan* s = P(structure);
    if (!p || !s || p == s) return -1;
    if (p->device && p->deviceFree) p->deviceFree(p->device);
    p->device = nullptr;
    return qg::compilePlanLike(*p, *s) ? (int)p->passes.size() : -1;
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
        for (size_t e = 0; e < ((size_t)1 << (2 * k)); ++e) {     // block 0 (all control bits 0)
            re[e] = s.m[e].real();
            im[e] = s.m[e].imag();
        }
    return k;
}

int quest_gb300_planPassBlock(void* plan, int i, int block, double* re, double* im) {
    FusedPlan* p = P(plan);
    if (!p || !p->compiled || i < 0 || i >= (int)p->passes.size() || !re || !im) return -1;
    const qg::FusedPass& s = p->passes[i];
    const size_t DD = (size_t)1 << (2 * s.targets.size());
    if (block < 0 || (size_t)block >= ((size_t)1 << s.controls.size())) return -1;
    for (size_t e = 0; e < DD; ++e) {
        re[e] = s.m[block * DD + e].real();
        im[e] = s.m[block * DD + e].imag();
    }
    return (int)s.targets.size();
}

}  // extern "C"
