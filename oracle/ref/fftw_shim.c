/* oracle/ref/fftw_shim.c -- the FFTW entry points the reference NFFT sources
 * call (kernel/nfft/nfft.c:6022-6031 plan, the executes, destroy at
 * 6221-6225; kernel/util/malloc.c:37,54), implemented on the project-written
 * FFT of oracle/fft_cpu.c.  Test infrastructure only: it lets the reference
 * library be built in place as a CPU oracle. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"

void orc_fft(int d, const int *n, double *data, int sign);
void orcf_fft(int d, const int *n, float *data, int sign);

/* FFTW's REDFT00 (DCT-I) and RODFT00 (DST-I) of one strided line, by their
 * defining sums in double precision (FFTW documentation, "1d Real-even DFTs"
 * and "1d Real-odd DFTs"): O(n^2), enough for the oracle's small cases. */
static void r2r_line(double *v, int n, int kind, double *tmp)
{
  int j, k;
  for (k = 0; k < n; k++) {
    double s = 0;
    if (kind == 3) {
      s = v[0] + ((k & 1) ? -v[n - 1] : v[n - 1]);
      for (j = 1; j < n - 1; j++) s += 2.0 * v[j] * cos(M_PI * (double)j * k / (n - 1));
    } else {
      for (j = 0; j < n; j++) s += 2.0 * v[j] * sin(M_PI * (double)(j + 1) * (k + 1) / (n + 1));
    }
    tmp[k] = s;
  }
  for (k = 0; k < n; k++) v[k] = tmp[k];
}

#define SHIM(X, R, FFT) \
  struct X##plan_s { int rank; int n[8]; R *in, *out; int sign; int r2r; int kind[8]; }; \
  X##plan X##plan_dft(int rank, const int *n, X##complex *in, X##complex *out, int sign, unsigned flags) \
  { \
    X##plan p = (X##plan)calloc(1, sizeof(*p)); int t; (void)flags; \
    p->rank = rank; for (t = 0; t < rank; t++) p->n[t] = n[t]; \
    p->in = (R*)in; p->out = (R*)out; p->sign = sign; return p; \
  } \
  X##plan X##plan_r2r(int rank, const int *n, R *in, R *out, const X##r2r_kind *kind, unsigned flags) \
  { \
    X##plan p = (X##plan)calloc(1, sizeof(*p)); int t; (void)flags; \
    p->rank = rank; for (t = 0; t < rank; t++) { p->n[t] = n[t]; p->kind[t] = kind[t]; } \
    p->in = in; p->out = out; p->r2r = 1; return p; \
  } \
  static void X##r2r_exec(const X##plan p) \
  { \
    size_t tot = 1, inner, outer, a, b; int t, k, nmax = 1; double *line, *tmp; \
    for (t = 0; t < p->rank; t++) { tot *= (size_t)p->n[t]; if (p->n[t] > nmax) nmax = p->n[t]; } \
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(R) * tot); \
    line = (double*)malloc(sizeof(double) * (size_t)nmax); tmp = (double*)malloc(sizeof(double) * (size_t)nmax); \
    for (t = 0; t < p->rank; t++) { \
      inner = 1; for (k = t + 1; k < p->rank; k++) inner *= (size_t)p->n[k]; \
      outer = tot / (inner * (size_t)p->n[t]); \
      for (a = 0; a < outer; a++) for (b = 0; b < inner; b++) { \
        R *base = p->out + a * (size_t)p->n[t] * inner + b; \
        for (k = 0; k < p->n[t]; k++) line[k] = (double)base[(size_t)k * inner]; \
        r2r_line(line, p->n[t], p->kind[t], tmp); \
        for (k = 0; k < p->n[t]; k++) base[(size_t)k * inner] = (R)line[k]; \
      } \
    } \
    free(line); free(tmp); \
  } \
  void X##execute(const X##plan p) \
  { \
    size_t tot = 1; int t; \
    if (p->r2r) { X##r2r_exec(p); return; } \
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
