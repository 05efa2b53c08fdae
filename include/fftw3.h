/*
 * fftw3.h -- the FFTW 3 type names that the NFFT 3 C API mentions, for
 * systems without FFTW.
 *
 * The NFFT header includes <fftw3.h> only for fftw_complex / fftwf_complex,
 * the opaque plan pointer types and the planner flag values (reference
 * include/nfft3.h:23, 108-161).  The GPU library computes its FFTs with cuFFT
 * and never calls FFTW, so this header declares types only.  When a real
 * FFTW 3 header is found first on the include path it is used instead; its
 * types are layout-identical.
 *
 * As in FFTW 3, the complex types are C99 `double _Complex` when <complex.h>
 * was included before this header, and `double[2]` otherwise.
 */
#ifndef FFTW3_H
#define FFTW3_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_CONCAT(prefix, name) prefix ## name
#define FFTW_MANGLE_DOUBLE(name) FFTW_CONCAT(fftw_, name)
#define FFTW_MANGLE_FLOAT(name) FFTW_CONCAT(fftwf_, name)
#define FFTW_MANGLE_LONG_DOUBLE(name) FFTW_CONCAT(fftwl_, name)

#if defined(_Complex_I) && defined(complex) && defined(I)
#define FFTW_DEFINE_COMPLEX(R, C) typedef R _Complex C
#else
#define FFTW_DEFINE_COMPLEX(R, C) typedef R C[2]
#endif

FFTW_DEFINE_COMPLEX(double, fftw_complex);
FFTW_DEFINE_COMPLEX(float, fftwf_complex);
FFTW_DEFINE_COMPLEX(long double, fftwl_complex);

typedef struct fftw_plan_s *fftw_plan;
typedef struct fftwf_plan_s *fftwf_plan;
typedef struct fftwl_plan_s *fftwl_plan;

typedef int fftw_r2r_kind;
typedef int fftwf_r2r_kind;
typedef int fftwl_r2r_kind;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)

/* planner flags (values as in FFTW 3; accepted and ignored by cuFFT) */
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

#ifdef __cplusplus
}
#endif

#endif /* FFTW3_H */
