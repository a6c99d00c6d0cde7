/*
 * rdtsc.h -- a portable tick counter for compiling the reference library
 * on hosts without its x86/PowerPC counter instructions: nanoseconds from
 * the monotonic clock (the reference uses ticks only for its own timers).
 */
#ifndef QLL_REF_RDTSC_STUB_H
#define QLL_REF_RDTSC_STUB_H
#include <time.h>
static inline unsigned long long rdtsc(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (unsigned long long)ts.tv_sec*1000000000ULL + (unsigned long long)ts.tv_nsec;
}
#endif
