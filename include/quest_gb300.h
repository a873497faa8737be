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

#ifdef __cplusplus
}
#endif

#endif /* QUEST_GB300_H */
