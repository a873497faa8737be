/*
 * QuEST_precision.h -- the precision definitions of the QuEST ABI.
 *
 * QuantumLab includes this header by name before QuEST.h
 * (Code/QuantumLab/Base/QLSetup.h:23, QuantumLabPCH.h:14 in the reference)
 * and branches on QuEST_PREC; it also calls Ceil() from it.  The names below
 * are the ones the reference's Code/QuEST340/QuEST/include/QuEST_precision.h
 * defines for its QuEST_PREC=2 build, the only precision this library
 * exports: qreal is double.
 */
#ifndef QUEST_PRECISION_H
#define QUEST_PRECISION_H

#include <math.h>

#ifndef QuEST_PREC
#define QuEST_PREC 2
#endif
#if QuEST_PREC != 2
#error "this library is built for QuEST_PREC=2 (qreal = double) only"
#endif

typedef double qreal;

#define REAL_EPS 1e-13
#define REAL_STRING_FORMAT "%.14f"
#define REAL_QASM_FORMAT "%.14g"
#define REAL_SPECIFIER "%lf"
#define absReal(X) fabs(X)
#define MAX_NUM_REGS_APPLY_ARBITRARY_PHASE 100

/* ceil(a / b) for b > 0 */
static inline int Ceil(long long a, long long b) { return (int)(a / b + (a % b != 0)); }

#endif /* QUEST_PRECISION_H */
