// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// Lets the reference's test translation unit (tests/test_kinetics.cpp and what
// it includes) compile on aarch64 hosts, where the x86 intrinsic headers do not
// exist. Only the three intrinsics that code calls are provided, portably:
//   __rdtsc      the profiler's and the work queue's spin timer: a monotonic
//                nanosecond clock instead of the TSC (the queue's ~50 us spin
//                before sleeping becomes 150 us);
//   _mm_pause    spin-loop hint: nothing;
//   _mm_getcsr / _mm_setcsr   the NFT code's denormal flush (MXCSR FTZ|DAZ):
//                the value is kept but has no effect on aarch64. None of the
//                chemistry code under test reads or sets it.
// Used only from oracle/Makefile when the host is not x86_64.
#ifndef ORACLE_ARM_COMPAT_X86INTRIN_H
#define ORACLE_ARM_COMPAT_X86INTRIN_H

#include <stdint.h>
#include <time.h>

static inline uint64_t __rdtsc(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

static inline void _mm_pause(void) {}

static unsigned int oracle_arm_compat_csr = 0x1f80u;   // MXCSR's power-on value
static inline unsigned int _mm_getcsr(void) { return oracle_arm_compat_csr; }
static inline void _mm_setcsr(unsigned int v) { oracle_arm_compat_csr = v; }

#endif
