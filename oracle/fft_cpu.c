/*
 * oracle/fft_cpu.c -- project-written CPU FFT used by the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is part of the CPU oracle that the
 * tests and the CPU-baseline leg of the benchmark use to check and time the
 * GPU library.  Nothing in the product path links or calls it.
 *
 * The reference NFFT library delegates its oversampled FFT to FFTW
 * (kernel/nfft/nfft.c:6030-6031 plans a d-dimensional complex DFT with
 * FFTW_FORWARD for the trafo and FFTW_BACKWARD for the adjoint; the executes are
 * at nfft.c:2834, 2871, 3900, 3938, 5516, 5557, 5690, 5738).  FFTW is not
 * available here, so this file restates the unnormalised d-dimensional
 * complex DFT
 *
 *     out[l] = sum_k in[k] * exp(sign * 2*pi*i * <k, l/n>)
 *
 * with an iterative radix-2 Cooley-Tukey transform along each axis for
 * power-of-two lengths and a direct O(n^2) DFT for any other length.  Each
 * precision computes in its own precision; twiddles come from the math
 * library in double and are rounded once.
 *
 * Compiled twice: plain (double, prefix orc_) and with -DORC_SINGLE (float,
 * prefix orcf_).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORC_SINGLE
typedef float R;
#define P(name) orcf_##name
#else
typedef double R;
#define P(name) orc_##name
#endif

static const double ORC_TWO_PI = 6.2831853071795864769252867665590057683943;

static int is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

/* In-place radix-2 DIT FFT of one contiguous line of n complex values
 * (interleaved re/im).  tw holds n/2 twiddles exp(sign*2*pi*i*k/n). */
static void fft_line_pow2(R *a, long n, const R *tw)
{
  long i, j, len;
  /* bit reversal */
  for (i = 1, j = 0; i < n; i++) {
    long bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      R tr = a[2 * i], ti = a[2 * i + 1];
      a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
      a[2 * j] = tr; a[2 * j + 1] = ti;
    }
  }
  for (len = 2; len <= n; len <<= 1) {
    long half = len >> 1, step = n / len, s, k;
    for (s = 0; s < n; s += len) {
      for (k = 0; k < half; k++) {
        R wr = tw[2 * (k * step)], wi = tw[2 * (k * step) + 1];
        R *u = a + 2 * (s + k), *v = a + 2 * (s + k + half);
        R vr = v[0] * wr - v[1] * wi;
        R vi = v[0] * wi + v[1] * wr;
        v[0] = u[0] - vr; v[1] = u[1] - vi;
        u[0] = u[0] + vr; u[1] = u[1] + vi;
      }
    }
  }
}

/* Direct DFT of one line (any n), out-of-place into tmp then copied back. */
static void dft_line(R *a, long n, int sign, R *tmp)
{
  long k, l;
  for (l = 0; l < n; l++) {
    double sr = 0.0, si = 0.0;
    for (k = 0; k < n; k++) {
      double ang = sign * ORC_TWO_PI * (double)((k * l) % n) / (double)n;
      double c = cos(ang), s = sin(ang);
      sr += a[2 * k] * c - a[2 * k + 1] * s;
      si += a[2 * k] * s + a[2 * k + 1] * c;
    }
    tmp[2 * l] = (R)sr; tmp[2 * l + 1] = (R)si;
  }
  memcpy(a, tmp, sizeof(R) * 2 * (size_t)n);
}

/* Unnormalised d-dimensional complex DFT, row-major (last index fastest),
 * in place on interleaved data.  sign = -1 (forward) or +1 (backward). */
void P(fft)(int d, const int *n, R *data, int sign)
{
  long total = 1;
  int t;
  for (t = 0; t < d; t++) total *= n[t];
  for (t = 0; t < d; t++) {
    long nt = n[t], stride = 1, outer, lines;
    int u;
    R *tw = NULL;
    for (u = t + 1; u < d; u++) stride *= n[u];
    outer = total / (nt * stride);
    lines = outer * stride;
    if (is_pow2(nt)) {
      long k;
      tw = (R*)malloc(sizeof(R) * 2 * (size_t)(nt / 2 + 1));
      for (k = 0; k < nt / 2; k++) {
        double ang = sign * ORC_TWO_PI * (double)k / (double)nt;
        tw[2 * k] = (R)cos(ang);
        tw[2 * k + 1] = (R)sin(ang);
      }
    }
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
      R *line = (R*)malloc(sizeof(R) * 2 * (size_t)nt);
      R *tmp = (R*)malloc(sizeof(R) * 2 * (size_t)nt);
      long L;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (L = 0; L < lines; L++) {
        long o = L / stride, s = L % stride, k;
        R *base = data + 2 * (o * nt * stride + s);
        if (stride == 1) {
          if (tw) fft_line_pow2(base, nt, tw); else dft_line(base, nt, sign, tmp);
          continue;
        }
        for (k = 0; k < nt; k++) {
          line[2 * k] = base[2 * k * stride];
          line[2 * k + 1] = base[2 * k * stride + 1];
        }
        if (tw) fft_line_pow2(line, nt, tw); else dft_line(line, nt, sign, tmp);
        for (k = 0; k < nt; k++) {
          base[2 * k * stride] = line[2 * k];
          base[2 * k * stride + 1] = line[2 * k + 1];
        }
      }
      free(line);
      free(tmp);
    }
    free(tw);
  }
}
