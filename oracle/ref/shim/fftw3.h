/* Project-written stand-in for the few FFTW3 declarations the reference NFFT
 * sources use (test infrastructure only; FFTW is not installed).  The FFTs
 * themselves come from oracle/fft_cpu.c through oracle/ref/fftw_shim.c. */
#ifndef ORACLE_REF_FFTW3_H
#define ORACLE_REF_FFTW3_H
#include <stddef.h>
#include <complex.h>
#ifdef __cplusplus
extern "C" {
#endif
#define FFTW_CONCAT(prefix, name) prefix ## name
#define FFTW_MANGLE_DOUBLE(name) FFTW_CONCAT(fftw_, name)
#define FFTW_MANGLE_FLOAT(name) FFTW_CONCAT(fftwf_, name)
#define FFTW_MANGLE_LONG_DOUBLE(name) FFTW_CONCAT(fftwl_, name)
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)
/* real-to-real kinds the reference's NFCT / NFST plan (FFTW's numbering) */
#define FFTW_REDFT00 3
#define FFTW_RODFT00 7
#define ORACLE_FFTW_DECLARE(X, R) \
  typedef R _Complex X##complex; \
  typedef struct X##plan_s *X##plan; \
  typedef enum { X##R2HC_kind_ = 0 } X##r2r_kind_do_not_use; \
  typedef int X##r2r_kind; \
  X##plan X##plan_dft(int rank, const int *n, X##complex *in, X##complex *out, int sign, unsigned flags); \
  X##plan X##plan_r2r(int rank, const int *n, R *in, R *out, const X##r2r_kind *kind, unsigned flags); \
  void X##execute(const X##plan p); \
  void X##destroy_plan(X##plan p); \
  void *X##malloc(size_t n); \
  void X##free(void *p); \
  void X##plan_with_nthreads(int nthreads); \
  int X##init_threads(void); \
  void X##cleanup_threads(void); \
  void X##cleanup(void);
ORACLE_FFTW_DECLARE(fftw_, double)
ORACLE_FFTW_DECLARE(fftwf_, float)
ORACLE_FFTW_DECLARE(fftwl_, long double)
#ifdef __cplusplus
}
#endif
#endif
