/* Project-written configuration for compiling the reference NFFT sources in
 * place as a CPU oracle (test infrastructure only).  Selects the default
 * Kaiser-Bessel window and the C99/POSIX facilities of gcc on Linux. */
#ifndef ORACLE_REF_CONFIG_H
#define ORACLE_REF_CONFIG_H
#define KAISER_BESSEL 1
#define WINDOW_NAME "KAISER_BESSEL"
#define STDC_HEADERS 1
#define HAVE_COMPLEX_H 1
#define HAVE_STDINT_H 1
#define HAVE_INTTYPES_H 1
#define HAVE_SYS_TYPES_H 1
#define HAVE_STDLIB_H 1
#define HAVE_STRING_H 1
#define HAVE_MALLOC_H 1
#define HAVE_ALLOCA 1
#define HAVE_ALLOCA_H 1
#define HAVE_DRAND48 1
#define HAVE_SRAND48 1
#define HAVE_CLOCK_GETTIME 1
#define SIZEOF_PTRDIFF_T 8
#define NFFT_VERSION_MAJOR 3
#define NFFT_VERSION_MINOR 5
#define NFFT_VERSION_PATCH 4
#define NFFT_VERSION_TYPE 0
#define PACKAGE_VERSION "3.5.4-oracle"
#define NFFT_PRECISION_DOUBLE 1
#endif
