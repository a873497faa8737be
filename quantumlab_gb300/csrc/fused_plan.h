// fused_plan.h -- gate-fusion planner of the FP32 fused engine (host C++).
//
// No counterpart in the reference (QuEST applies one kernel per gate).  A
// plan records a gate stream and groups it into "passes": dense
// 2^k x 2^k complex matrices on k <= kmax qubits, each formed as the FP64
// product of the gates it absorbs.  Each pass is one streaming sweep of the
// FP32 state on the device.
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

namespace qg {

using cplx = std::complex<double>;

struct FusedGate {
    std::vector<int> qubits;   // matrix bit b <-> qubits[b]
    std::vector<cplx> m;       // row-major 2^q x 2^q
    bool unitary = false;      // m m^+ = I to 1e-12 (matrixIsUnitary)
};

struct FusedPass {
    std::vector<int> targets;  // ascending; matrix bit b <-> targets[b]
    // Control qubits (ascending; none unless the plan allows them): qubits
    // outside the targets on which every absorbed gate that touches them is
    // diagonal.  The pass applies, to each amplitude, the matrix of the value
    // c of its control bits (bit j of c <-> controls[j]).
    std::vector<int> controls;
    std::vector<cplx> m;       // 2^controls.size() row-major D x D blocks (block c), D = 2^targets.size()
    int numGates = 0;
    bool unitary = false;      // every absorbed gate is unitary
};

struct FusedPlan {
    int numQubits = 0;
    int maxFused = 4;
    int beamWidth = 16;         // sets kept per level of the pass search
    int maxControls = 0;        // control qubits a pass may use (0..3; see FusedPass)
    int lookahead = 4;          // candidate sets tried one pass ahead (0: the best set at once)
    bool searchOnly = false;    // compilePlan finds the passes (passSets...) without their products
    std::vector<FusedGate> gates;
    std::vector<FusedPass> passes;
    // the search's result: per pass its qubit set and the indices of the
    // gates it absorbs, in an allowed order (compilePlanLike reuses them)
    std::vector<uint64_t> passSets;
    std::vector<uint64_t> passControls;
    std::vector<std::vector<int>> passMembers;
    bool compiled = false;
    // device copy of the per-pass FP32 (and split-TF32) operands, built on
    // first use by the FP32 engine; owned by the engine
    void* device = nullptr;
    void (*deviceFree)(void*) = nullptr;
};

// Widest pass the FP32 appliers take on registers of n qubits: six qubits
// need the tensor-core applier (n >= 13: a tile is 2^(6+7) amplitudes), the
// SIMT applier takes up to five.
inline int widestPass(int n) { return n >= 13 ? 6 : (n < 5 ? n : 5); }

// Control qubits a new plan on n qubits may use: 3 from 26 qubits up while
// the tensor cores are enabled (controlled passes run only there; on a
// 25-qubit register a captured 7,040-gate circuit took 36 ms with controls
// against 32 without: a pass is ~90 us there, and the extra operand images
// cost more host time than the passes they save), else 0.
int defaultMaxControls(int n);

// |m m^+ - I| <= 1e-12 entrywise for a row-major D x D matrix.
bool matrixIsUnitary(const std::vector<cplx>& m, int D);

// Beam search over qubit sets at the circuit front (see fused_plan.cpp).
// Leaves plan.compiled false if it fails.
void compilePlan(FusedPlan& plan);

// Compile `plan` with the passes `structure` found, without a search: the
// gate lists must match gate by gate in qubits, and every gate of `plan` must
// be diagonal on at least the qubits where `structure`'s gate is (so that the
// structure's reordering stays valid).  Gates of the same circuit with other
// angles qualify.  Returns false (plan not compiled) otherwise.
bool compilePlanLike(FusedPlan& plan, const FusedPlan& structure);

// exp(-i angle/2 P) as a dense gate on the qubits of the Pauli string with
// X/Y/Z masks x, y, z (Y bits also in x); the operator QuEST's
// multiRotatePauli applies (QuEST_common.c:411-448).
FusedGate pauliRotationGate(uint64_t x, uint64_t y, uint64_t z, double angle);

}  // namespace qg
