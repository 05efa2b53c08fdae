/* oracle/ref/fftw_shim.c -- the FFTW entry points the reference NFFT sources
 * call (kernel/nfft/nfft.c:6022-6031 plan, the executes, destroy at
 * 6221-6225; kernel/util/malloc.c:37,54), implemented on the project-written
 * FFT of oracle/fft_cpu.c.  Test infrastructure only: it lets the reference
 * library be built in place as a CPU oracle. */
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"

void orc_fft(int d, const int *n, double *data, int sign);
void orcf_fft(int d, const int *n, float *data, int sign);

#define SHIM(X, R, FFT) \
  struct X##plan_s { int rank; int n[8]; R *in, *out; int sign; }; \
  X##plan X##plan_dft(int rank, const int *n, X##complex *in, X##complex *out, int sign, unsigned flags) \
  { \
    X##plan p = (X##plan)calloc(1, sizeof(*p)); int t; (void)flags; \
    p->rank = rank; for (t = 0; t < rank; t++) p->n[t] = n[t]; \
    p->in = (R*)in; p->out = (R*)out; p->sign = sign; return p; \
  } \
  void X##execute(const X##plan p) \
  { \
    size_t tot = 1; int t; \
    for (t = 0; t < p->rank; t++) tot *= (size_t)p->n[t]; \
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(R) * 2 * tot); \
    FFT(p->rank, p->n, p->out, p->sign); \
  } \
  void X##destroy_plan(X##plan p) { free(p); } \
  void *X##malloc(size_t n) { void *q = NULL; if (posix_memalign(&q, 64, n ? n : 1)) return NULL; return q; } \
  void X##free(void *p) { free(p); } \
  void X##plan_with_nthreads(int nthreads) { (void)nthreads; } \
  int X##init_threads(void) { return 1; } \
  void X##cleanup_threads(void) {} \
  void X##cleanup(void) {}

SHIM(fftw_, double, orc_fft)
SHIM(fftwf_, float, orcf_fft)
