/* Project-written tick counter for the in-place reference build (test
 * infrastructure only): CLOCK_MONOTONIC nanoseconds. */
#ifndef ORACLE_REF_TICKS_H
#define ORACLE_REF_TICKS_H
#include <time.h>
typedef unsigned long long ticks;
static inline ticks getticks(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (ticks)ts.tv_sec * 1000000000ULL + (ticks)ts.tv_nsec;
}
static inline double elapsed(ticks t1, ticks t0) { return (double)t1 - (double)t0; }
#define HAVE_TICK_COUNTER 1
#define TICKS_PER_SECOND 1000000000.0
#endif
