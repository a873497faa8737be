/*
 * quest_gb300.h -- extensions of the GB300 library beyond the QuEST API.
 *
 * None of these has a counterpart in the reference (Code/QuEST340 has no
 * timing, no fused FP32 engine and no batched engine); they are additions
 * required to measure and to run the fused / batched paths.  C ABI, plain
 * pointers and sizes only.
 */
#ifndef QUEST_GB300_H
#define QUEST_GB300_H

#include "QuEST.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- runtime introspection and timing ---------------------------------- */
/* The cudaStream_t on which every kernel of the library is queued. */
void* quest_gb300_stream(void);
/* Number of kernels this library has launched since load. */
long long quest_gb300_launchCount(void);
/* Record CUDA event `slot` (0..8191) on the library stream. Returns 0 on success. */
int quest_gb300_eventRecord(int slot);
/* Milliseconds between two recorded events (waits for `slotB`); -1 on error. */
double quest_gb300_eventElapsedMs(int slotA, int slotB);
/* 1 when the register's host mirror is page-locked (cudaMallocHost), 0 when
 * that failed and it fell back to pageable memory, -1 for an unknown register.
 * Host <-> device copies of a pageable mirror run several times slower. */
int quest_gb300_hostMirrorPinned(Qureg qureg);

/* ---- gate-fusion plans ---------------------------------------------------
 * A plan records a gate stream on numQubits qubits and compiles it into
 * passes: dense 2^k x 2^k complex matrices on k <= maxFusedQubits (<= 6)
 * qubits, formed as FP64 products of the absorbed gates.  maxFusedQubits is
 * capped at the widest pass the FP32 appliers take on numQubits qubits: 6
 * from 13 qubits up, else 5 (or numQubits).  Matrices are row-major with
 * matrix bit b on targets[b]; compactUnitary and friends keep the QuEST
 * conventions.  Add functions return 0, or -1 on invalid input (a gate wider
 * than the capped width included).                                          */
void* quest_gb300_planCreate(int numQubits, int maxFusedQubits);
void quest_gb300_planDestroy(void* plan);
int quest_gb300_planAddGate(void* plan, const int* targets, int numTargets, const double* re, const double* im);
int quest_gb300_planAddCompactUnitary(void* plan, int target, double alphaRe, double alphaIm, double betaRe, double betaIm);
int quest_gb300_planAddUnitary(void* plan, int target, const double* re4, const double* im4);
int quest_gb300_planAddHadamard(void* plan, int target);
int quest_gb300_planAddControlledNot(void* plan, int control, int target);
int quest_gb300_planAddControlledPhaseShift(void* plan, int qubit1, int qubit2, double angle);
/* Sets kept per level of the pass search (1..256, default 16); wider finds
 * fewer passes on some circuits at more host time.  Returns 0 or -1. */
int quest_gb300_planSetBeamWidth(void* plan, int width);
/* Lookahead of the pass search (0..16 candidate sets; default 4, and 8 for
 * plans on 28 qubits or more): the best
 * candidates of each pass are tried with the pass that would follow them, and
 * the pair that absorbs the most gates decides (~2 % fewer passes on random
 * circuits, ~12 % on first-order Trotter circuits, for ~2x the search time).
 * 0 takes the best set at once; op-stream capture plans without lookahead.
 * Returns 0 or -1. */
int quest_gb300_planSetLookahead(void* plan, int candidates);
/* Control qubits a pass may use (0..3; a new plan gets 3 on registers of 26
 * qubits or more while the tensor cores are enabled, else 0; op-stream
 * capture uses the same rule).  A pass of at least four
 * qubits may then absorb gates that also act on qubits outside its targets,
 * when each gate is diagonal on those qubits and each such qubit lies above
 * the pass's tile (at least 7 non-target qubits below it): the pass applies,
 * per amplitude, the matrix of the value of its control bits (2^controls
 * FP64 products).  A controlled controlledPhaseShift, for instance, no longer
 * needs both its qubits in one pass.  Controlled passes run on the
 * tensor-core applier only.  Returns 0 or -1. */
int quest_gb300_planSetMaxControls(void* plan, int maxControls);
/* Compile; returns the number of passes, or -1. */
int quest_gb300_planCompile(void* plan);
/* Compile `plan` with the passes of the compiled plan `structure`, without a
 * search: the same circuit with other angles (a variational loop, another
 * Hamiltonian instance).  The gate lists must match gate by gate in qubits,
 * and each gate of `plan` must be diagonal on at least the qubits where the
 * structure's gate is.  Returns the number of passes, or -1. */
int quest_gb300_planCompileLike(void* plan, void* structure);
int quest_gb300_planNumGates(void* plan);
/* Copy pass i (targets ascending, FP64 matrix; for a controlled pass the
 * matrix of control value 0); returns k or -1. */
int quest_gb300_planPass(void* plan, int i, int* targets, double* re, double* im);
/* Control qubits of pass i (ascending) into controls (may be NULL); returns
 * their number or -1. */
int quest_gb300_planPassControls(void* plan, int i, int* controls);
/* The matrix of pass i for control value `block` (bit j <-> the j-th control
 * qubit); returns k or -1. */
int quest_gb300_planPassBlock(void* plan, int i, int block, double* re, double* im);

/* Per-pass timing: with setPassEvents(1), applyPlanF32 records a CUDA event
 * pair on the library stream around each pass; passTimesMs writes the
 * durations (ms) of the passes of the last application (-1 for a pass not
 * recorded) once the stream has passed them, and returns the number of
 * passes. */
void quest_gb300_setPassEvents(int on);
int quest_gb300_passTimesMs(double* out, int maxPasses);

/* ---- arithmetic of the plain path ------------------------------------------
 * No counterpart in the reference.  GB300 runs FP64 fused multiply-adds at
 * about 1/70 of its FP32 rate, so the plain path's general 2 x 2 gates
 * (compactUnitary and the rotations, unitary and its controlled forms,
 * hadamard) are bound by the FP64 pipe, not by HBM.  Mode 1 computes them in
 * double-float arithmetic on the FP32 and integer pipes: each double is split
 * into two floats by integer field operations (2^-47 relative), products are
 * exact through FMA, sums compensated (TwoSum), and the result is packed back
 * into the double's fields; the state stays FP64 in memory.  A gate's result
 * is then within a few 2^-47 of FP64, relative to its largest term.  Doubles
 * below 2^-126 in magnitude are flushed to 0 and those of 2^128 and above
 * are not representable.  Mode 0, exact FP64, is the default.  Returns 0, or
 * -1 for an unknown mode. */
int quest_gb300_setPlainArithmetic(int mode);
int quest_gb300_getPlainArithmetic(void);

/* ---- autotuner -------------------------------------------------------------
 * No counterpart in the reference.  autotune measures, for registers of
 * numQubits qubits at the current tensor-core precision, the time of one pass
 * of every width k = 1..6 in every target layout class (0: every target at or
 * above qubit 5; 1: a target below 5; 2: qubits 0 and 1 both targets) on a
 * scratch FP32 register.  Each class that runs on the tensor cores is timed
 * with every pipelined kernel variant (2: two loader groups on alternate
 * chunks + one epilogue group; 3: one + one; 4: one + two; 5: two loader
 * groups splitting each chunk + two epilogue groups) and the fastest is used
 * for that class from then on, unless it beats the class's fixed default by
 * 3 % or less (then the default stays; setKernelTuning(0) returns to the
 * fixed defaults).  The table is cached as JSON ($QUEST_GB300_TUNE_CACHE, default
 * ~/.cache/quest_gb300_tune.json) and loaded by the first autotune call.
 * planCompileTuned compiles the plan at every width in [minK, maxK] and keeps
 * the fastest predicted one.  tunedKernel returns the chosen variant of a
 * class (0 if untuned) and its measured time per pass.                      */
int quest_gb300_autotune(int numQubits);
double quest_gb300_planPredictMs(void* plan);
int quest_gb300_planCompileTuned(void* plan, int minK, int maxK);
int quest_gb300_tunedKernel(int numQubits, int k, int layout, double* msPerPass);
void quest_gb300_setKernelTuning(int on);

/* ---- FP32 registers of the fused engine ----------------------------------
 * A state vector of 2^numQubits FP32 complex amplitudes (SoA) on the
 * device.  Reductions accumulate in FP64.                                    */
void* quest_gb300_createQuregF32(int numQubits);
void quest_gb300_destroyQuregF32(void* qureg32);
void quest_gb300_initZeroStateF32(void* qureg32);
/* host FP64 amplitudes (like initStateFromAmps), rounded to FP32 on the device */
void quest_gb300_initStateFromAmpsF32(void* qureg32, const double* reals, const double* imags);
/* all amplitudes to host FP64 arrays */
void quest_gb300_copyStateToHostF32(void* qureg32, double* reals, double* imags);
/* device-side conversion from / to an FP64 state-vector Qureg of equal size */
void quest_gb300_copyFromQureg(void* qureg32, Qureg source);
void quest_gb300_copyToQureg(void* qureg32, Qureg destination);
/* apply every pass of the plan (compiling it first if needed); 0 on success */
int quest_gb300_applyPlanF32(void* qureg32, void* plan);
/* Norm record of pass i of the plan's last application, if it ran on the
 * tensor cores: {sum |x|^2 in, sum |y|^2 out, square of the drift-correction
 * scale it applied}.  Returns 1, or 0 if there is no record. */
int quest_gb300_planPassNorms(void* plan, int i, double* inOutScaleSq);
/* apply passes [firstPass, firstPass + numPasses) only (timing, stepping) */
int quest_gb300_applyPlanF32Range(void* qureg32, void* plan, int firstPass, int numPasses);
/* applier of pass i: 0 = SIMT, 1 = direct-load tensor-core kernel, 2..5 =
 * pipelined tensor-core kernel (as setTensorCoreKernel); -1 if invalid */
int quest_gb300_planPassUsesTensorCores(void* plan, int i);
/* passes on 4..6 qubits run on the tensor cores (split-TF32) unless disabled
 * here (1 = enabled, the default; 0 = FP32 SIMT applier for k <= 5) */
void quest_gb300_setTensorCores(int enabled);
/* tensor-core kernel: 0 = chosen per pass (default), 1 = always the
 * direct-load kernel, 2..5 = always the pipelined kernel with 2 loader + 1
 * epilogue warp groups (2), 1 + 1 (3), 1 + 2 (4), or 2 + 2 with the loader
 * groups splitting every chunk (5) */
void quest_gb300_setTensorCoreKernel(int version);
/* Operands of the pipelined tensor-core kernel: 0 = 3-term split-TF32
 * (X, G in two TF32 parts; Xh.Gh + Xl.Gh + Xh.Gl), the default; 1 = 4-term
 * split-BF16 (X in two BF16 parts, G in three; Xh.Gh + Xl.Gh + Xh.Gl +
 * Xh.Gll); 2 = 3-term split-FP16 (as split-TF32, with FP16 parts of the same
 * 11-bit precision at twice the MMA rate; X and each matrix block are scaled
 * by powers of two before the split, X's from the norm the previous pass of
 * a plan application measured, or, at the first pass, the norm a capture
 * flush sums while converting the state, else 2^14: so the first tensor-core
 * pass of quest_gb300_applyPlanF32 needs amplitudes of modulus below 3.99; a
 * non-finite output is reported as an error, the state is then lost).  All
 * accumulate in FP32.
 * Returns 0, or -1 for another mode. */
int quest_gb300_setTensorCorePrecision(int mode);
int quest_gb300_getTensorCorePrecision(void);
/* How the pipelined tensor-core kernels stage state tiles in shared memory:
 * 0 = 16-byte cp.async copies by every loader lane (the default); 1 = TMA
 * bulk copies (cp.async.bulk), one 128-byte row of a tile per copy, completing
 * on an mbarrier.  Both give identical results; on the 30-qubit random
 * circuit a 6-qubit pass takes 2.83 ms with 0 and 3.77 ms with 1 (split-TF32),
 * because 128-byte copies keep the TMA unit far below the HBM rate.  Returns
 * 0, or -1 for another mode. */
int quest_gb300_setTensorCoreStaging(int mode);
int quest_gb300_getTensorCoreStaging(void);
/* Host check of the pipelined tensor-core kernel's addressing (no GPU): from
 * the launch parameters of a pass on `targets` (ascending, 4..6) with
 * `controls` (ascending, 0..3) on a register of numQubits <= 26 qubits, walk
 * every CTA, tile, warp and lane as the kernel does.  Returns 0 when every
 * amplitude is read and written exactly once, 1 when not, -1 when the pass
 * does not fit (controls inside the tile, too few qubits). */
int quest_gb300_checkTileCoverage(int numQubits, const int* targets, int numTargets, const int* controls, int numControls);
/* Host check of the tensor-core operand images (no GPU): for every pass width
 * and image layout the library builds, the part each kernel reads is present,
 * 16-byte aligned, inside the image block and disjoint from the other parts.
 * Returns 0 when all hold, else 1. */
int quest_gb300_checkImageLayouts(void);
/* Host check of the split-FP16 operand images (no GPU): for pass widths 4..6
 * and random matrix blocks from zero to 1e4 in size, the two FP16 parts of
 * every entry, times the factor stored after them, give the entry to 2^-21
 * of the block's largest, with every scaled entry at most 2^14.  Returns 0
 * when all hold, else 1. */
int quest_gb300_checkHalfImages(void);
/* The host rounding that builds split-FP16 operand images: each value to the
 * nearest IEEE binary16 (ties to even; infinity beyond 65504), as bit
 * patterns.  Returns 0, or -1 for a negative count or a missing array. */
int quest_gb300_roundHalf(const double* values, unsigned short* out, int count);
double quest_gb300_calcTotalProbF32(void* qureg32);
double quest_gb300_calcProbOfOutcomeF32(void* qureg32, int measureQubit, int outcome);
/* 1 - |<ref|q>|^2 / (<ref|ref><q|q>) against an FP64 state vector; writes the
 * largest |amplitude difference| to *maxAmpErr when it is not NULL */
double quest_gb300_compareF32(void* qureg32, Qureg reference, double* maxAmpErr);

/* ---- batched swap tests (QKMeans distances) --------------------------------
 * For each test t, P(ancilla = 0) of the (2d+1)-qubit swap-test circuit
 * |0>|v>|u> -> H(anc) -> CSWAP(anc; u_i, v_i) for i < d -> H(anc), with
 * u = vector idxA[t], v = vector idxB[t] (real, length 2^d, 1 <= d <= 10).
 * The distance estimate is 2 P0 - 1 = |<u|v>|^2.  Vectors are concatenated
 * in `vectors` (host, FP64) at offsets[i] with length 2^dimLog2[i].  Create
 * uploads the data and captures one persistent kernel into a CUDA graph;
 * Run replays it (FP32 state vectors, FP64-combined probabilities) and writes
 * numTests values to p0Out (host) in the caller's order.                    */
void* quest_gb300_swapTestBatchCreate(const double* vectors, const long long* offsets, const int* dimLog2,
                                      int numVectors, const int* idxA, const int* idxB, int numTests);
int quest_gb300_swapTestBatchRun(void* batch, double* p0Out);
/* Autotune the batch's kernel: time every pairing of CTAs per SM (2, 3, 4)
 * and shared-memory threshold (states of up to 2^9, 2^11 or 2^13 amplitudes
 * kept in shared memory, larger ones in a global arena), keep the fastest and
 * capture the graph again with it.  Writes the choice, its time per run and
 * the default's (4 CTAs per SM, 2^13) in ms; returns 0 or -1. */
int quest_gb300_swapTestBatchTune(void* batch, int* ctasPerSM, int* smemAmps, double* msBest, double* msDefault);
void quest_gb300_swapTestBatchDestroy(void* batch);

/* ---- op-stream capture ------------------------------------------------------
 * No counterpart in the reference.  With capture on for a register, its gate
 * calls (every unitary/matrix/rotation/phase/NOT/swap/Pauli-rotation call and
 * applyTrotterCircuit) are queued as dense FP64 matrices on the <= 6 qubits
 * they touch instead of running; the first other call on the register (a
 * reduction, measurement, copy, amplitude read, channel, ...) applies the
 * queue through the fusion planner and the FP32 fused engine; calls that
 * overwrite the whole state (init*, initStateFromAmps, copyStateToGPU, a
 * cloneQureg target) drop it.  Results then carry the FP32 engine's precision.
 * QUEST_GB300_CAPTURE=fp32 turns capture on for registers created afterwards. */
/* mode 1: capture with FP32 fused flushes; 0: off (flushes what is queued).
 * Returns 0, or -1 for an unallocated register. */
int quest_gb300_setCapture(Qureg qureg, int mode);
void quest_gb300_flushCapture(Qureg qureg);
/* gates queued and not yet applied */
int quest_gb300_capturedGates(Qureg qureg);
/* Totals of the register's flushes since capture was turned on: flushes,
 * gates applied, fused passes applied and host milliseconds spent planning
 * them (any pointer may be null).  Returns 0, or -1 when capture is off. */
int quest_gb300_captureStats(Qureg qureg, long long* flushes, long long* gatesApplied, long long* passesApplied,
                             double* compileMs);
/* widest fused pass of the flushes, 1..6 (default 6); 0: the autotuner picks
 * the width of each searched plan (planCompileTuned over 4..6; the first such
 * flush of a register size measures its cost table) */
void quest_gb300_setCaptureFusion(int maxFusedQubits);

/* ---- amplitude-encoded product states ------------------------------------------
 * No counterpart in the reference; it replaces the lab's amplitude-encoding
 * circuits (Code/QuantumLab/Circuit/Gates/AmplitudeEncodeCuda.cu:691-776) for
 * state preparation.  Sets a state-vector register to v_{R-1} (x) ... (x) v_0:
 * register r holds v_r / |v_r| on the next regQubits[r] qubits, starting at
 * qubit 0; the qubits above are |0>.  re / im hold the R vectors one after
 * another (lengths 2^regQubits[r]); im may be NULL for real vectors.
 * 1 <= R <= 16.  Returns 0, or -1 after reporting an invalid argument
 * through invalidQuESTInputError. */
int quest_gb300_initProductState(Qureg qureg, int numRegs, const int* regQubits, const double* re, const double* im);

/* ---- repeated measurement ------------------------------------------------------
 * No counterpart in the reference; it replaces the lab's shot loop "measure
 * each listed qubit in order, then copyStateToGPU to restore the state"
 * (Code/QuantumLab/Simulator/QLSimulatorMeasure.cpp:70-109) by one call.
 * Writes numShots outcome codes (bit j = outcome of qubits[j]) drawn from the
 * same global MT19937 stream, with the same rule and the same number of draws
 * as that loop (QuEST_common.c:165-180), so a seeded run gives the loop's
 * outcomes.  The register is left unchanged (the loop leaves the last shot's
 * collapse).  1 <= numQubits <= 24.  Returns 0, or -1 after reporting an
 * invalid argument through invalidQuESTInputError. */
int quest_gb300_sampleMeasurements(Qureg qureg, const int* qubits, int numQubits, int numShots, int* outcomes);

/* ---- batched Trotter instances ----------------------------------------------
 * B Hamiltonian instances of 11..numQubits qubits (numQubits <= 34) evolve
 * together as FP32 states.  Instances that share register size, Pauli
 * strings, Trotter order and repetitions form a class (coefficients, time and
 * the classical start state may differ): one fusion plan per class (searched
 * on one member, reused with each member's FP64 products) and one
 * tensor-core launch per fused pass over all the class's states.  Classes of
 * different step counts, orders, sizes or Hamiltonians run one after another
 * in the same run, and after the first run the whole batch is a CUDA graph
 * that later runs replay.  The gates are QuEST's applyTrotterCircuit(hamil,
 * time, order, reps) from initClassicalState(init).  Energies are
 * <H> / <psi|psi> of each final FP32 state (FP32 products, FP64 sums).
 * Errors go through invalidQuESTInputError; functions return 0 or -1.       */
void* quest_gb300_trotterBatchCreate(int numQubits, int numInstances);
int quest_gb300_trotterBatchSetInstance(void* batch, int instance, PauliHamil hamil, double time, int order, int reps,
                                        long long initClassicalState);
/* Set instance `instance` to an explicit circuit instead: the gates recorded
 * in `plan` (planCreate(numQubits, ...) + planAdd*; 11 <= numQubits <= the
 * batch's), applied from initClassicalState(init); its "energy" is the
 * expectation of `hamil` (numSumTerms = 0: none, reported as 0).  Instances
 * with the same register size, gate qubits gate by gate and Hamiltonian
 * strings share a class (one search, one launch per pass); an instance whose
 * gates cannot take its class's passes is given its own. */
int quest_gb300_trotterBatchSetCircuit(void* batch, int instance, void* plan, PauliHamil hamil,
                                       long long initClassicalState);
/* Evolve every instance; energies (may be null): B doubles. */
int quest_gb300_trotterBatchRun(void* batch, double* energies);
/* Copy instance `instance`'s final state into an FP64 register of n qubits,
 * scaled to norm 1 (the start state's) by the norm the last run measured. */
int quest_gb300_trotterBatchCopyState(void* batch, int instance, Qureg dst);
/* Fused-pass launches per run, summed over the classes (after the first
 * run), else -1. */
int quest_gb300_trotterBatchNumPasses(void* batch);
/* Classes of the batch (after the first run), else -1. */
int quest_gb300_trotterBatchNumClasses(void* batch);
void quest_gb300_trotterBatchDestroy(void* batch);

/* ---- total probability without allocating ---------------------------------
 * No counterpart in the reference.  For callers that hold their own FP64
 * state arrays and must not allocate while they run (a host callback or
 * real-time worker kept out of the CUDA allocator, a process whose device
 * memory is reserved by another framework's pool, a library that only borrows
 * device pointers): sum |amp|^2 of deviceReal/deviceImag[numAmps] with no
 * cudaMalloc, cudaFree or allocating library call.  Scratch is a fixed
 * __device__ array of about 16.5 KB per GPU, so numAmps must be a power of two
 * in [2, 2^27]; larger states are rejected with an error (use calcTotalProb).
 * Both arrays must start on a 16-byte boundary (they are read two doubles at
 * a time); a misaligned pointer is rejected before anything is queued.
 * The result is written to *result (host or device memory) and the call
 * returns after `stream` (a cudaStream_t; NULL = legacy default stream) has
 * finished it.  The first call on a device looks up the scratch address (a
 * failed lookup is retried by the next call) and should come before any
 * stream capture.  All calls share the scratch: calls
 * that overlap on the GPU race.  Returns 0 on success, nonzero after
 * reporting the error through invalidQuESTInputError.                       */
int quest_gb300_calcTotalProbNoAlloc(const double* deviceReal, const double* deviceImag, long long numAmps,
                                     double* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QUEST_GB300_H */
