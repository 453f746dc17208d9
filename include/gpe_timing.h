/*
 * Host timers of the libcugpe drivers (KKobuszewski/libcugpe dev/gpe_timing.h:36-64),
 * for source compatibility: the reference drivers time blocks of steps with
 *
 *     b_t();  ...  double seconds = e_t(0);
 *
 * b_t() starts a wall-clock and a CPU-time measurement; e_t(0) returns the
 * wall-clock seconds since b_t() and keeps them and the CPU time; e_t(1)
 * returns the kept wall-clock seconds again; e_t(2) the kept CPU seconds.
 * Included by gpe_engine.h, as the reference's engine header includes its
 * timing header.
 */
#ifndef GPE_GB300_TIMING_H
#define GPE_GB300_TIMING_H

#include <time.h>

static double gpe_timing_wall_start_;
static double gpe_timing_wall_;
static clock_t gpe_timing_cpu_start_;
static clock_t gpe_timing_cpu_;

static inline double gpe_timing_now_(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline void b_t(void) {
    gpe_timing_cpu_start_ = clock();
    gpe_timing_wall_start_ = gpe_timing_now_();
}

#ifdef __cplusplus
static inline double e_t(int type = 0)
#else
static inline double e_t(int type)
#endif
{
    if (type == 0) {
        gpe_timing_cpu_ = clock() - gpe_timing_cpu_start_;
        gpe_timing_wall_ = gpe_timing_now_() - gpe_timing_wall_start_;
        return gpe_timing_wall_;
    }
    if (type == 2) return (double)gpe_timing_cpu_ / (double)CLOCKS_PER_SEC;
    return gpe_timing_wall_;
}

#endif
