// qg_internal.h -- internal interface between the QuEST-ABI front-end
// (api.cpp) and the sm_103a engines (*.cu).  Not installed, not part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <stddef.h>
#include <vector>

#include "QuEST.h"

namespace qg {

typedef long long idx_t;

// ---- runtime -------------------------------------------------------------
// All device work of the library is queued on one stream created with the
// default (blocking) flags, so it also orders against legacy-stream work that
// callers issue on the same device.
cudaStream_t stream();
// Report a CUDA failure through invalidQuESTInputError; returns true on error.
bool cudaFailed(cudaError_t e, const char* what, const char* caller);
#define QG_CUDA(call, caller) ::qg::cudaFailed((call), #call, caller)
// Check the last launch; returns true on error.
bool launchFailed(const char* caller);

int numSMs();
// kernels launched by the library (quest_gb300_launchCount)
extern std::atomic<long long> g_launches;

// Per-register reduction workspace held in Qureg.firstLevelReduction.
// Layout (doubles): [partials: 2*kMaxReduceBlocks][result: 64][counter word]
constexpr int kMaxReduceBlocks = 2048;
constexpr size_t kScratchDoubles = 2 * kMaxReduceBlocks + 64 + 8;
struct Scratch {
    double* partials;          // 2*kMaxReduceBlocks doubles (double2 per block)
    double* result;            // device result slots
    unsigned int* counter;     // last-block-done ticket, kept at 0 between calls
    double* host;              // pinned host slots (Qureg.secondLevelReduction)
};
Scratch scratchOf(const Qureg& q);

// ---- state-vector gates (sv_gates.cu) ------------------------------------
// Every launcher acts on the FP64 SoA arrays (re, im) of 2^n amplitudes.
struct SV {
    double* re;
    double* im;
    int n;                      // qubits in the state vector (2N for a density matrix)
    void* cap = nullptr;        // capture record: gate launchers queue the gate instead (capture.cpp)
};
inline SV svOf(const Qureg& q) { return SV{q.deviceStateVec.real, q.deviceStateVec.imag, q.numQubitsInStateVec}; }

// ---- op-stream capture (capture.cpp) ----------------------------------------
void* captureHandle(const double* re);            // the register's capture record, or null
// at creation: capture on if QUEST_GB300_CAPTURE=fp32; dmQubits = N for a
// density matrix of N qubits (a 2N-qubit vector), 0 for a state vector
void captureRegister(const double* re, int n, int dmQubits);
void captureFlush(double* re, double* im);        // apply the queued gates (FP32 fused engine)
// FP32 register -> FP64 Qureg after applying `plan`, with the plan's last norm
// correction folded in (fused_f32.cu)
void copyToQuregAfterPlan(void* qureg32, Qureg& dst, void* plan);
// the same for a trace-preserving plan on a density matrix of N qubits: the
// trace recorded by traceBeforePlan is restored (fused_f32.cu)
void traceBeforePlan(const double* re, int N);
void copyToQuregTraceKept(void* qureg32, Qureg& dst, int N);
// FP64 Qureg -> FP32 register with sum |x|^2 of the result summed on the
// device (returned; null on failure), and a whole plan applied to a register
// whose sum |x|^2 the device holds at entryBound (fused_f32.cu)
const double* copyFromQuregNorm(void* qureg32, const Qureg& src);
int applyPlanF32Entry(void* qureg32, void* plan, const double* entryBound);
void captureDiscard(const double* re);            // drop the queued gates (the state is overwritten next)
void captureDrop(const double* re);               // at destruction
// launcher hooks: queue the gate and return true, or return false (after a
// flush) when it touches more than 6 qubits
bool capturePair(SV s, int target, uint64_t ctrl, uint64_t flip, const double ur[4], const double ui[4]);
bool captureNot(SV s, uint64_t ctrl, uint64_t targMask);
bool capturePhase(SV s, uint64_t mask, double tr, double ti);
bool captureRotateZ(SV s, uint64_t ctrl, uint64_t targ, double angle);
bool capturePauliRotation(SV s, uint64_t ctrl, uint64_t xmask, uint64_t ymask, uint64_t zmask, double angle, int conj);
bool captureSwap(SV s, int q1, int q2);
bool captureMatrixN(SV s, uint64_t ctrl, const int* targs, int k, const double* mr, const double* mi);
// a one-qubit decoherence channel on a density matrix of N qubits, as the
// real 4 x 4 superoperator S on (row qubit t, column qubit t + N): local index
// = row bit + 2 column bit, out = S in
bool captureChannel(SV s, int t, int N, const double S[16]);
// a channel on the qubits of `mask` (k of them, k <= 6) as its real
// 2^k x 2^k superoperator S (row-major), local bit i = the i-th lowest qubit
bool captureChannelN(SV s, uint64_t mask, const double* S);

struct Mat2 { double r[2][2], i[2][2]; };

// U on target for amplitudes whose control bits match: ((idx ^ flip) & ctrl) == ctrl.
void gateMatrix2(SV s, int target, uint64_t ctrl, uint64_t flip, const Mat2& u);
// [alpha, -conj(beta); beta, conj(alpha)] (QuEST compactUnitary form).
void gateCompact(SV s, int target, uint64_t ctrl, double ar, double ai, double br, double bi);
void gateHadamard(SV s, int target);
// amp <-> amp ^ targMask where ctrl bits are set (X, CNOT, multi-qubit NOT).
void gateNot(SV s, uint64_t ctrl, uint64_t targMask);
// Y (conjFac=+1) or conj(Y) (conjFac=-1) on target, where ctrl bits are set.
void gatePauliY(SV s, int target, uint64_t ctrl, double conjFac);
// amp *= (tr + i ti) where all bits of mask are 1.
void gatePhase(SV s, uint64_t mask, double tr, double ti);
// amp *= exp(-i angle/2 * (+1 even parity of idx&targ, -1 odd)), where ctrl bits set.
void gateRotateZ(SV s, uint64_t ctrl, uint64_t targ, double angle);
// exp(-i angle/2 P) with P a Pauli string given by x/y/z masks, where ctrl bits set;
// conj!=0 applies the elementwise conjugate operator.
void gatePauliRotation(SV s, uint64_t ctrl, uint64_t xmask, uint64_t ymask, uint64_t zmask, double angle, int conj);
void gateSwap(SV s, int q1, int q2);
// plain-path arithmetic of the general 2 x 2 gates: 0 FP64, 1 double-float
bool setPlainArithmetic(int mode);
int plainArithmetic();
// Dense 2^k x 2^k (k <= 6) on targets (targs[0] = least significant matrix bit).
// mr/mi row-major host arrays.
void gateMatrixN(SV s, uint64_t ctrl, const int* targs, int k, const double* mr, const double* mi);

// ---- initialisation / elementwise (state_ops.cu) --------------------------
void stateFill(SV s, double re, double im);
void stateSetOne(SV s, idx_t index, double re, double im);   // one element, others untouched
void stateDebug(SV s);
// product of unit vectors on consecutive qubit ranges from qubit 0 (<= 16 registers)
void stateProduct(SV s, int numRegs, const int* regBits, const double* vr, const double* vi);
void statePlusDM(SV s, int nRep);
void statePureDM(SV rho, const double* psiRe, const double* psiIm, int nRep);
void stateWeighted(SV out, double f1r, double f1i, SV a, double f2r, double f2i, SV b, double for_, double foi);
void stateMixDM(SV a, double p, SV b);
void collapseSV(SV s, int target, int outcome, double renorm);
void collapseDM(SV s, int target, int nRep, int outcome, double renorm);
// density-matrix channels (QuEST.c:1259-1322 semantics)
void dmDephase(SV s, int target, int nRep, double retain);
void dmDepolarise(SV s, int target, int nRep, double level);
void dmDamp(SV s, int target, int nRep, double prob);
void dmPauli(SV s, int target, int nRep, double pX, double pY, double pZ);
// q1 < q2 (QuEST.c:1269, 1300: ensureIndsIncrease)
void dmTwoQubitDephase(SV s, int q1, int q2, int nRep, double retain);
void dmTwoQubitDepolarise(SV s, int q1, int q2, int nRep, double level);

// ---- reductions (reduce.cu) -------------------------------------------------
// All return their value through the pinned host slot after a stream sync.
double reduceTotalProbSV(SV s, const Scratch& w);
double reduceTotalProbDM(SV s, int nRep, const Scratch& w);
double reduceProbZeroSV(SV s, int target, const Scratch& w);
double reduceProbZeroDM(SV s, int target, int nRep, const Scratch& w);
void reduceInnerProduct(SV bra, SV ket, const Scratch& w, double* outRe, double* outIm);
double reduceDotReal(SV a, SV b, const Scratch& w);          // sum re*re' + im*im'
double reduceNormSq(SV s, const Scratch& w);                 // sum |amp|^2 (no Kahan split)
double reduceDistSq(SV a, SV b, const Scratch& w);
double reduceFidelityDM(SV rho, SV psi, int nRep, const Scratch& w);
// Expectation sum_t coeff_t <psi|P_t|psi> (SV) or Tr(P_t rho) (DM) of Pauli
// strings grouped by their X/Y mask (one read of the state per group); yz/nY
// per term.  Every group's reduction is queued before one synchronisation.
struct PauliTerm { uint64_t yz; int nY; double coeff; };
struct PauliTermGroup { uint64_t xmask; std::vector<PauliTerm> terms; };
double reduceExpecPauliGroups(SV s, int isDM, int nRep, const std::vector<PauliTermGroup>& groups, const Scratch& w);
// State vector, X/Y mask x != 0: each pair (j, j ^ x) adds Re(conj(psi_j)
// psi_k) A(j) + Im(conj(psi_j) psi_k) B(j), A and B sums of +-c over these
// lists of (yz mask, c): the terms whose pair contributions do not cancel.
void pauliPairTerms(uint64_t x, const std::vector<PauliTerm>& terms, std::vector<std::pair<uint64_t, double>>& A,
                    std::vector<std::pair<uint64_t, double>>& B);
void reduceProbAllOutcomes(SV s, int isDM, int nRep, const int* qubits, int numQubits, double* hostOut, const Scratch& w);

}  // namespace qg
