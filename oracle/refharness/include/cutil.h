/* cutil.h -- minimal host implementation of the CUDA SDK "cutil" timer
 * helpers that dSim2/src/spinSystem.cpp calls (cutCreateTimer, cutStartTimer,
 * ...).  Test infrastructure for the reference harness in oracle/_ref/;
 * timers measure host wall time. */
#ifndef DSIM_REFHARNESS_CUTIL_H
#define DSIM_REFHARNESS_CUTIL_H
#include <time.h>
#define CUT_SAFE_CALL(call) (call)
#define CUT_CHECK_ERROR(msg) ((void)0)
static double g_cut_start[16], g_cut_acc[16];
static unsigned g_cut_n = 0;
static inline double cut_now_ms() {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}
static inline int cutCreateTimer(unsigned int* t) { *t = (g_cut_n++) & 15u; g_cut_acc[*t] = 0; return 1; }
static inline int cutDeleteTimer(unsigned int) { return 1; }
static inline int cutResetTimer(unsigned int t) { g_cut_acc[t & 15u] = 0; return 1; }
static inline int cutStartTimer(unsigned int t) { g_cut_start[t & 15u] = cut_now_ms(); return 1; }
static inline int cutStopTimer(unsigned int t) { g_cut_acc[t & 15u] += cut_now_ms() - g_cut_start[t & 15u]; return 1; }
static inline float cutGetTimerValue(unsigned int t) { return (float)g_cut_acc[t & 15u]; }
#endif
