/*
 * QuEST.h -- C ABI of the GB300 state-vector / density-matrix library.
 *
 * This header is the drop-in boundary below QuantumLab: every type keeps the
 * byte layout and every function keeps the name, argument meaning and error
 * behaviour of the QuEST 3.4 API that QuantumLab calls
 * (Code/QuEST340/QuEST/include/QuEST.h in the reference).  Only the subset on
 * the simulation hot path is declared; each group cites the reference
 * declaration and front-end implementation (Code/QuEST340/QuEST/src/QuEST.c)
 * it replaces.
 *
 * Precision: qreal is double (the reference's QuEST_PREC=2 build).  The plain
 * engine computes every gate in FP64 on the device; the FP32 fused engine is
 * a separate extension API (quest_gb300.h).
 *
 * Errors: invalid input calls invalidQuESTInputError(msg, func).  The default
 * definition is weak; it forwards to the function pointer __other_input_error
 * when that is set, otherwise prints the message and exits (reference
 * QuEST_validation.c:216-243, QuEST.h:72-73).  Unlike the reference, an API
 * call whose validation failed returns immediately if the handler returns,
 * so a handler that records the error and returns is safe.
 */
#ifndef QUEST_H
#define QUEST_H

#include "QuEST_precision.h"

#ifndef M_PI
#define M_PI 3.1415926535897932384626433832795028841971
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error hook (reference QuEST.h:72-73, QuEST_validation.c:216-243) ---- */
typedef void (*pfinvalidQuESTInputError)(const char* errMsg, const char* errFunc);
extern pfinvalidQuESTInputError __other_input_error;
void invalidQuESTInputError(const char* errMsg, const char* errFunc);

/* ---- value types (reference QuEST.h:87-400; layouts must match) ---- */
enum phaseGateType {SIGMA_Z = 0, S_GATE = 1, T_GATE = 2};
enum pauliOpType {PAULI_I = 0, PAULI_X = 1, PAULI_Y = 2, PAULI_Z = 3};
enum phaseFunc {
    NORM = 0, SCALED_NORM = 1, INVERSE_NORM = 2, SCALED_INVERSE_NORM = 3, SCALED_INVERSE_SHIFTED_NORM = 4,
    PRODUCT = 5, SCALED_PRODUCT = 6, INVERSE_PRODUCT = 7, SCALED_INVERSE_PRODUCT = 8,
    DISTANCE = 9, SCALED_DISTANCE = 10, INVERSE_DISTANCE = 11, SCALED_INVERSE_DISTANCE = 12,
    SCALED_INVERSE_SHIFTED_DISTANCE = 13};
enum bitEncoding {UNSIGNED = 0, TWOS_COMPLEMENT = 1};

typedef struct {
    char* buffer;
    int bufferSize;
    int bufferFill;
    int isLogging;
} QASMLogger;

typedef struct ComplexArray { qreal* real; qreal* imag; } ComplexArray;
typedef struct Complex { qreal real; qreal imag; } Complex;
typedef struct ComplexMatrix2 { qreal real[2][2]; qreal imag[2][2]; } ComplexMatrix2;
typedef struct ComplexMatrix4 { qreal real[4][4]; qreal imag[4][4]; } ComplexMatrix4;
typedef struct ComplexMatrixN { int numQubits; qreal** real; qreal** imag; } ComplexMatrixN;
typedef struct Vector { qreal x, y, z; } Vector;

typedef struct PauliHamil {
    enum pauliOpType* pauliCodes;   /* numSumTerms * numQubits codes, term-major */
    qreal* termCoeffs;              /* numSumTerms coefficients */
    int numSumTerms;
    int numQubits;
} PauliHamil;

typedef struct DiagonalOp {
    int numQubits;
    long long int numElemsPerChunk;
    int numChunks;
    int chunkId;
    qreal* real;
    qreal* imag;
    ComplexArray deviceOperator;
} DiagonalOp;

/* A register.  stateVec is the host mirror (pinned host memory here),
 * deviceStateVec the authoritative FP64 SoA device arrays.  A density matrix
 * of N qubits is a 2N-qubit vector, element (r, c) at index r + c * 2^N. */
typedef struct Qureg {
    int isDensityMatrix;
    int numQubitsRepresented;
    int numQubitsInStateVec;
    long long int numAmpsPerChunk;
    long long int numAmpsTotal;
    int chunkId;
    int numChunks;
    ComplexArray stateVec;
    ComplexArray pairStateVec;      /* unused on one GPU (NULL) */
    ComplexArray deviceStateVec;
    qreal* firstLevelReduction;     /* device reduction scratch of this register */
    qreal* secondLevelReduction;    /* pinned host slot for reduction results */
    QASMLogger* qasmLog;
} Qureg;

typedef struct QuESTEnv {
    int rank;
    int numRanks;
    unsigned long int* seeds;
    int numSeeds;
} QuESTEnv;

/* ---- environment (reference QuEST.h:1922-1983, QuEST_gpu.cu:447-498) ---- */
QuESTEnv createQuESTEnv(void);
void destroyQuESTEnv(QuESTEnv env);
void syncQuESTEnv(QuESTEnv env);
int syncQuESTSuccess(int successCode);
void reportQuESTEnv(QuESTEnv env);
void getEnvironmentString(QuESTEnv env, char str[200]);
void seedQuEST(QuESTEnv* env, unsigned long int* seedArray, int numSeeds);   /* QuEST.c seedQuEST via QuEST_gpu.cu:3970 */
void seedQuESTDefault(QuESTEnv* env);                                        /* QuEST.c:1653 */
void getQuESTSeeds(QuESTEnv env, unsigned long int** seeds, int* numSeeds);  /* QuEST.c:1661 */
int getQuEST_PREC(void);                                                      /* QuEST.c:1649 */

/* ---- registers (QuEST.c:42-86; QuEST_gpu.cu:277-326, 500-519) ---- */
Qureg createQureg(int numQubits, QuESTEnv env);
Qureg createDensityQureg(int numQubits, QuESTEnv env);
Qureg createCloneQureg(Qureg qureg, QuESTEnv env);
void destroyQureg(Qureg qureg, QuESTEnv env);
void copyStateToGPU(Qureg qureg);
void copyStateFromGPU(Qureg qureg);
void copySubstateToGPU(Qureg qureg, long long int startInd, long long int numAmps);
void copySubstateFromGPU(Qureg qureg, long long int startInd, long long int numAmps);
int getNumQubits(Qureg qureg);
long long int getNumAmps(Qureg qureg);
ComplexMatrixN createComplexMatrixN(int numQubits);
void destroyComplexMatrixN(ComplexMatrixN matr);
PauliHamil createPauliHamil(int numQubits, int numSumTerms);
void destroyPauliHamil(PauliHamil hamil);
void initPauliHamil(PauliHamil hamil, qreal* coeffs, enum pauliOpType* codes);

/* ---- initialisation (QuEST.c:119-176) ---- */
void initBlankState(Qureg qureg);
void initZeroState(Qureg qureg);
void initPlusState(Qureg qureg);
void initClassicalState(Qureg qureg, long long int stateInd);
void initPureState(Qureg qureg, Qureg pure);
void initDebugState(Qureg qureg);
void initStateFromAmps(Qureg qureg, qreal* reals, qreal* imags);
void setAmps(Qureg qureg, long long int startInd, qreal* reals, qreal* imags, long long int numAmps);
void setDensityAmps(Qureg qureg, long long int startRow, long long int startCol, qreal* reals, qreal* imags, long long int numAmps);
void cloneQureg(Qureg targetQureg, Qureg copyQureg);
void setWeightedQureg(Complex fac1, Qureg qureg1, Complex fac2, Qureg qureg2, Complex facOut, Qureg out);

/* ---- amplitude access (QuEST.c:940-970) ---- */
Complex getAmp(Qureg qureg, long long int index);
qreal getRealAmp(Qureg qureg, long long int index);
qreal getImagAmp(Qureg qureg, long long int index);
qreal getProbAmp(Qureg qureg, long long int index);
Complex getDensityAmp(Qureg qureg, long long int row, long long int col);

/* ---- one-qubit gates (QuEST.c:178-430) ---- */
void hadamard(Qureg qureg, int targetQubit);
void pauliX(Qureg qureg, int targetQubit);
void pauliY(Qureg qureg, int targetQubit);
void pauliZ(Qureg qureg, int targetQubit);
void sGate(Qureg qureg, int targetQubit);
void tGate(Qureg qureg, int targetQubit);
void phaseShift(Qureg qureg, int targetQubit, qreal angle);
void rotateX(Qureg qureg, int rotQubit, qreal angle);
void rotateY(Qureg qureg, int rotQubit, qreal angle);
void rotateZ(Qureg qureg, int rotQubit, qreal angle);
void rotateAroundAxis(Qureg qureg, int rotQubit, qreal angle, Vector axis);
void compactUnitary(Qureg qureg, int targetQubit, Complex alpha, Complex beta);
void unitary(Qureg qureg, int targetQubit, ComplexMatrix2 u);
void applyMatrix2(Qureg qureg, int targetQubit, ComplexMatrix2 u);

/* ---- controlled gates (QuEST.c:366-660) ---- */
void controlledNot(Qureg qureg, int controlQubit, int targetQubit);
void controlledPauliY(Qureg qureg, int controlQubit, int targetQubit);
void controlledPhaseShift(Qureg qureg, int idQubit1, int idQubit2, qreal angle);
void controlledPhaseFlip(Qureg qureg, int idQubit1, int idQubit2);
void controlledRotateX(Qureg qureg, int controlQubit, int targetQubit, qreal angle);
void controlledRotateY(Qureg qureg, int controlQubit, int targetQubit, qreal angle);
void controlledRotateZ(Qureg qureg, int controlQubit, int targetQubit, qreal angle);
void controlledRotateAroundAxis(Qureg qureg, int controlQubit, int targetQubit, qreal angle, Vector axis);
void controlledCompactUnitary(Qureg qureg, int controlQubit, int targetQubit, Complex alpha, Complex beta);
void controlledUnitary(Qureg qureg, int controlQubit, int targetQubit, ComplexMatrix2 u);
void multiControlledUnitary(Qureg qureg, int* controlQubits, int numControlQubits, int targetQubit, ComplexMatrix2 u);
void multiStateControlledUnitary(Qureg qureg, int* controlQubits, int* controlState, int numControlQubits, int targetQubit, ComplexMatrix2 u);
void multiControlledPhaseShift(Qureg qureg, int* controlQubits, int numControlQubits, qreal angle);
void multiControlledPhaseFlip(Qureg qureg, int* controlQubits, int numControlQubits);
void multiQubitNot(Qureg qureg, int* targs, int numTargs);
void multiControlledMultiQubitNot(Qureg qureg, int* ctrls, int numCtrls, int* targs, int numTargs);
void swapGate(Qureg qureg, int qubit1, int qubit2);
void sqrtSwapGate(Qureg qureg, int qb1, int qb2);

/* ---- multi-qubit gates (QuEST.c:300-352, 640-760, 1116-1140) ---- */
void twoQubitUnitary(Qureg qureg, int targetQubit1, int targetQubit2, ComplexMatrix4 u);
void controlledTwoQubitUnitary(Qureg qureg, int controlQubit, int targetQubit1, int targetQubit2, ComplexMatrix4 u);
void multiControlledTwoQubitUnitary(Qureg qureg, int* controlQubits, int numControlQubits, int targetQubit1, int targetQubit2, ComplexMatrix4 u);
void multiQubitUnitary(Qureg qureg, int* targs, int numTargs, ComplexMatrixN u);
void controlledMultiQubitUnitary(Qureg qureg, int ctrl, int* targs, int numTargs, ComplexMatrixN u);
void multiControlledMultiQubitUnitary(Qureg qureg, int* ctrls, int numCtrls, int* targs, int numTargs, ComplexMatrixN u);
void applyMatrix4(Qureg qureg, int targetQubit1, int targetQubit2, ComplexMatrix4 u);
void applyMatrixN(Qureg qureg, int* targs, int numTargs, ComplexMatrixN u);
void multiRotateZ(Qureg qureg, int* qubits, int numQubits, qreal angle);
void multiControlledMultiRotateZ(Qureg qureg, int* controlQubits, int numControls, int* targetQubits, int numTargets, qreal angle);
void multiRotatePauli(Qureg qureg, int* targetQubits, enum pauliOpType* targetPaulis, int numTargets, qreal angle);
void multiControlledMultiRotatePauli(Qureg qureg, int* controlQubits, int numControls, int* targetQubits, enum pauliOpType* targetPaulis, int numTargets, qreal angle);
void applyTrotterCircuit(Qureg qureg, PauliHamil hamil, qreal time, int order, int reps);

/* ---- measurement-like operations (QuEST.c:972-1016) ---- */
qreal collapseToOutcome(Qureg qureg, int measureQubit, int outcome);
int measure(Qureg qureg, int measureQubit);
int measureWithStats(Qureg qureg, int measureQubit, qreal* outcomeProb);

/* ---- reductions (QuEST.c:1152-1240) ---- */
qreal calcTotalProb(Qureg qureg);
qreal calcProbOfOutcome(Qureg qureg, int measureQubit, int outcome);
void calcProbOfAllOutcomes(qreal* outcomeProbs, Qureg qureg, int* qubits, int numQubits);
Complex calcInnerProduct(Qureg bra, Qureg ket);
qreal calcDensityInnerProduct(Qureg rho1, Qureg rho2);
qreal calcPurity(Qureg qureg);
qreal calcFidelity(Qureg qureg, Qureg pureState);
qreal calcHilbertSchmidtDistance(Qureg a, Qureg b);
qreal calcExpecPauliProd(Qureg qureg, int* targetQubits, enum pauliOpType* pauliCodes, int numTargets, Qureg workspace);
qreal calcExpecPauliSum(Qureg qureg, enum pauliOpType* allPauliCodes, qreal* termCoeffs, int numSumTerms, Qureg workspace);
qreal calcExpecPauliHamil(Qureg qureg, PauliHamil hamil, Qureg workspace);

/* ---- decoherence (QuEST.c:1259-1322; reference QuEST.h:3620-3850) ---- */
void mixDephasing(Qureg qureg, int targetQubit, qreal prob);
void mixDepolarising(Qureg qureg, int targetQubit, qreal prob);
void mixDamping(Qureg qureg, int targetQubit, qreal prob);
void mixDensityMatrix(Qureg combineQureg, qreal prob, Qureg otherQureg);
void mixTwoQubitDephasing(Qureg qureg, int qubit1, int qubit2, qreal prob);      /* QuEST.c:1269 */
void mixTwoQubitDepolarising(Qureg qureg, int qubit1, int qubit2, qreal prob);   /* QuEST.c:1300 */
void mixPauli(Qureg qureg, int targetQubit, qreal probX, qreal probY, qreal probZ);   /* QuEST.c:1312 */

/* ---- QASM recording: accepted and ignored (QuEST.c:92-113) ---- */
void startRecordingQASM(Qureg qureg);
void stopRecordingQASM(Qureg qureg);
void clearRecordedQASM(Qureg qureg);
void printRecordedQASM(Qureg qureg);
void writeRecordedQASMToFile(Qureg qureg, char* filename);

/* ---- reports (reference QuEST.h:1317-1358; plain-text output) ---- */
void reportState(Qureg qureg);
void reportStateToScreen(Qureg qureg, QuESTEnv env, int reportRank);
void reportQuregParams(Qureg qureg);
void reportPauliHamil(PauliHamil hamil);

/* ---- the rest of the reference API (QuEST.h:800-6900).  These are exported
 * so that any program written against QuEST 3.4 links; QuantumLab calls none
 * of them.  Each reports "unsupported" through invalidQuESTInputError and
 * returns a zeroed value where it has one. ---- */
void mixKrausMap(Qureg qureg, int target, ComplexMatrix2* ops, int numOps);
void mixTwoQubitKrausMap(Qureg qureg, int target1, int target2, ComplexMatrix4* ops, int numOps);
void mixMultiQubitKrausMap(Qureg qureg, int* targets, int numTargets, ComplexMatrixN* ops, int numOps);
void mixNonTPKrausMap(Qureg qureg, int target, ComplexMatrix2* ops, int numOps);
void mixNonTPTwoQubitKrausMap(Qureg qureg, int target1, int target2, ComplexMatrix4* ops, int numOps);
void mixNonTPMultiQubitKrausMap(Qureg qureg, int* targets, int numTargets, ComplexMatrixN* ops, int numOps);
void applyPauliSum(Qureg inQureg, enum pauliOpType* allPauliCodes, qreal* termCoeffs, int numSumTerms, Qureg outQureg);
void applyPauliHamil(Qureg inQureg, PauliHamil hamil, Qureg outQureg);
void applyMultiControlledMatrixN(Qureg qureg, int* ctrls, int numCtrls, int* targs, int numTargs, ComplexMatrixN u);
void applyProjector(Qureg qureg, int qubit, int outcome);
void applyQFT(Qureg qureg, int* qubits, int numQubits);
void applyFullQFT(Qureg qureg);
void applyPhaseFunc(Qureg qureg, int* qubits, int numQubits, enum bitEncoding encoding, qreal* coeffs, qreal* exponents, int numTerms);
void applyPhaseFuncOverrides(Qureg qureg, int* qubits, int numQubits, enum bitEncoding encoding, qreal* coeffs, qreal* exponents, int numTerms, long long int* overrideInds, qreal* overridePhases, int numOverrides);
void applyMultiVarPhaseFunc(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, qreal* coeffs, qreal* exponents, int* numTermsPerReg);
void applyMultiVarPhaseFuncOverrides(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, qreal* coeffs, qreal* exponents, int* numTermsPerReg, long long int* overrideInds, qreal* overridePhases, int numOverrides);
void applyNamedPhaseFunc(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, enum phaseFunc functionNameCode);
void applyNamedPhaseFuncOverrides(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, enum phaseFunc functionNameCode, long long int* overrideInds, qreal* overridePhases, int numOverrides);
void applyParamNamedPhaseFunc(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, enum phaseFunc functionNameCode, qreal* params, int numParams);
void applyParamNamedPhaseFuncOverrides(Qureg qureg, int* qubits, int* numQubitsPerReg, int numRegs, enum bitEncoding encoding, enum phaseFunc functionNameCode, qreal* params, int numParams, long long int* overrideInds, qreal* overridePhases, int numOverrides);
DiagonalOp createDiagonalOp(int numQubits, QuESTEnv env);
DiagonalOp createDiagonalOpFromPauliHamilFile(char* fn, QuESTEnv env);
void destroyDiagonalOp(DiagonalOp op, QuESTEnv env);
void syncDiagonalOp(DiagonalOp op);
void initDiagonalOp(DiagonalOp op, qreal* real, qreal* imag);
void initDiagonalOpFromPauliHamil(DiagonalOp op, PauliHamil hamil);
void setDiagonalOpElems(DiagonalOp op, long long int startInd, qreal* real, qreal* imag, long long int numElems);
void applyDiagonalOp(Qureg qureg, DiagonalOp op);
Complex calcExpecDiagonalOp(Qureg qureg, DiagonalOp op);
PauliHamil createPauliHamilFromFile(char* fn);
#ifndef __cplusplus
/* C only, as in the reference (QuEST.h:776-802, 5687-5733): the matrices are
 * variable-length 2D arrays of 2^numQubits columns.  Implemented. */
void initComplexMatrixN(ComplexMatrixN m, qreal real[][1 << m.numQubits], qreal imag[][1 << m.numQubits]);
ComplexMatrixN bindArraysToStackComplexMatrixN(int numQubits, qreal re[][1 << numQubits], qreal im[][1 << numQubits],
                                               qreal** reStorage, qreal** imStorage);
#endif

#ifdef __cplusplus
}
#endif

#endif /* QUEST_H */
