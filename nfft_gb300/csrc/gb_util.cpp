// gb_util.cpp -- the utility part of the NFFT 3 C API (host functions).
//
// Reference: kernel/util/malloc.c:21-64 (allocation hooks, die), rand.c:20-61,
// int.c:21-133 (exp2i, next_power_of_2), window.c:37-60 (m2K, default cut-off,
// window name), thread.c:25-57, time.c, error.c:120-168, vector1.c:22-57,
// vector3.c:22-178 (upd_axpy, fftshift), version.c.
//
// nfft_malloc hands out page-locked (pinned) host memory for large blocks so
// that the plan's x / f_hat / f arrays, which the library allocates with it
// under MALLOC_X / MALLOC_F_HAT / MALLOC_F, move to and from the GPU by DMA
// at full link bandwidth.  Small blocks and hosts without a usable GPU get
// ordinary aligned memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <mutex>
#include <map>
#include <string>
#include <unordered_set>
#include <utility>

#include "../../include/nfft3.h"
#include "gb_common.cuh"
#include "gb_internal.h"

namespace {

std::mutex g_pin_mu;
std::unordered_set<void *> g_pinned;
constexpr size_t PIN_MIN_BYTES = 64 * 1024;

void *alloc_block(size_t n)
{
  if (n == 0) n = 1;
  void *p = nullptr;
  if (n >= PIN_MIN_BYTES) {
    if (cudaHostAlloc(&p, n, cudaHostAllocPortable) == cudaSuccess && p) {
      std::lock_guard<std::mutex> lk(g_pin_mu);
      g_pinned.insert(p);
      return p;
    }
    cudaGetLastError();  // no GPU here: fall through to pageable memory
    p = nullptr;
  }
  if (posix_memalign(&p, 64, n) != 0) return nullptr;
  return p;
}

void free_block(void *p)
{
  bool pinned = false;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pinned.find(p);
    if (it != g_pinned.end()) {
      pinned = true;
      g_pinned.erase(it);
    }
  }
  if (pinned) cudaFreeHost(p);
  else free(p);
}

std::mutex g_err_mu;
std::string g_last_error;

}  // namespace

namespace gb {

void record_error(const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = buf;
}

void fatal(const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_last_error = buf;
  }
  std::string msg = std::string("nfft_gb300: ") + buf + "\n";
  nfft_die(msg.c_str());
}

void check_cuda(cudaError_t e, const char *what, const char *file, int line)
{
  if (e != cudaSuccess) fatal("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

void check_launch(const char *what, const char *file, int line)
{
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fatal("launch of %s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

void set_smem_limit(const void *kernel, size_t bytes)
{
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> done;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice", __FILE__, __LINE__);
  std::lock_guard<std::mutex> lk(mu);
  size_t &have = done[std::make_pair(dev, kernel)];
  if (have >= bytes) return;
  check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
             "cudaFuncSetAttribute", __FILE__, __LINE__);
  have = bytes;
}

}  // namespace gb

extern "C" {

// ------------------------------------------------ allocation hooks and die
#define GB_MALLOC_API(X, NAME)                                                         \
  X##malloc_type_function X##malloc_hook = 0;                                          \
  X##free_type_function X##free_hook = 0;                                              \
  X##die_type_function X##die_hook = 0;                                                \
  void *X##malloc(size_t n)                                                            \
  {                                                                                    \
    if (X##malloc_hook) return X##malloc_hook(n);                                      \
    void *p = alloc_block(n);                                                          \
    if (!p) X##die(NAME ": out of memory\n");                                          \
    return p;                                                                          \
  }                                                                                    \
  void X##free(void *p)                                                                \
  {                                                                                    \
    if (!p) return;                                                                    \
    if (X##free_hook) {                                                                \
      X##free_hook(p);                                                                 \
      return;                                                                          \
    }                                                                                  \
    free_block(p);                                                                     \
  }                                                                                    \
  void X##die(const char *s)                                                           \
  {                                                                                    \
    if (X##die_hook) X##die_hook(s);                                                   \
    else fputs(s, stderr);                                                             \
    exit(EXIT_FAILURE);                                                                \
  }

GB_MALLOC_API(nfft_, "nfft_malloc")
GB_MALLOC_API(nfftf_, "nfftf_malloc")

unsigned long long nfft_gb_tma_wait_timeouts(void)
{
  return gb::read_wait_timeouts() + gb::read_wait_timeouts_2d();
}

const char *nfft_gb_last_error(void)
{
  static thread_local std::string copy;
  std::lock_guard<std::mutex> lk(g_err_mu);
  copy = g_last_error;
  return copy.c_str();
}

void nfft_gb_clear_error(void)
{
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error.clear();
}

int nfft_gb_device_ok(void)
{
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (prop.major == 10 && prop.minor == 3) ? 1 : 0;
}

// ------------------------------------------------ utilities per precision
#define GB_UTIL_API(Y, R, CX)                                                          \
  R Y##drand48(void) { return (R)drand48(); }                                          \
  void Y##srand48(long int seed) { srand48(seed); }                                    \
  void Y##vrand_unit_complex(CX *x, const NFFT_INT n)                                  \
  {                                                                                    \
    for (NFFT_INT k = 0; k < n; k++) {                                                 \
      R re = Y##drand48();                                                             \
      R im = Y##drand48();                                                             \
      ((R *)x)[2 * k] = re;                                                            \
      ((R *)x)[2 * k + 1] = im;                                                        \
    }                                                                                  \
  }                                                                                    \
  void Y##vrand_shifted_unit_double(R *x, const NFFT_INT n)                            \
  {                                                                                    \
    for (NFFT_INT k = 0; k < n; k++) x[k] = Y##drand48() - (R)0.5;                     \
  }                                                                                    \
  void Y##vrand_real(R *x, const NFFT_INT n, const R a, const R b)                     \
  {                                                                                    \
    for (NFFT_INT k = 0; k < n; k++) x[k] = a + Y##drand48() * (b - a);                \
  }                                                                                    \
  void Y##vpr_double(R *x, const NFFT_INT n, const char *text)                         \
  {                                                                                    \
    if (text) printf("\n %s, adr=%p\n", text, (void *)x);                              \
    for (NFFT_INT k = 0; k < n; k++) {                                                 \
      if (k % 8 == 0) printf("%6td.\t", k);                                            \
      printf("%+.1E,", (double)x[k]);                                                  \
      if (k % 8 == 7) printf("\n");                                                    \
    }                                                                                  \
    if (n % 8 != 0) printf("\n");                                                      \
    fflush(stdout);                                                                    \
  }                                                                                    \
  void Y##vpr_complex(CX *x, const NFFT_INT n, const char *text)                       \
  {                                                                                    \
    const R *v = (const R *)x;                                                         \
    if (text) printf("\n %s, adr=%p\n", text, (void *)x);                              \
    for (NFFT_INT k = 0; k < n; k++) {                                                 \
      if (k % 4 == 0) printf("%6td.\t", k);                                            \
      printf("%+.1E%+.1Ei,", (double)v[2 * k], (double)v[2 * k + 1]);                  \
      if (k % 4 == 3) printf("\n");                                                    \
    }                                                                                  \
    if (n % 4 != 0) printf("\n");                                                      \
    fflush(stdout);                                                                    \
  }                                                                                    \
  NFFT_INT Y##get_num_threads(void) { return 1; }                                      \
  void Y##set_num_threads(NFFT_INT nthreads) { (void)nthreads; }                       \
  NFFT_INT Y##has_threads_enabled(void) { return 0; }                                  \
  R Y##clock_gettime_seconds(void)                                                     \
  {                                                                                    \
    struct timespec ts;                                                                \
    clock_gettime(CLOCK_MONOTONIC, &ts);                                               \
    return (R)ts.tv_sec + (R)ts.tv_nsec * (R)1e-9;                                     \
  }                                                                                    \
  R Y##error_l_infty_complex(const CX *x, const CX *y, const NFFT_INT n)               \
  {                                                                                    \
    const R *a = (const R *)x, *b = (const R *)y;                                      \
    R num = 0, den = 0;                                                                \
    for (NFFT_INT k = 0; k < n; k++) {                                                 \
      R t = std::hypot(a[2 * k] - b[2 * k], a[2 * k + 1] - b[2 * k + 1]);              \
      num = t > num ? t : num;                                                         \
      t = std::hypot(a[2 * k], a[2 * k + 1]);                                          \
      den = t > den ? t : den;                                                         \
    }                                                                                  \
    return num / den;                                                                  \
  }                                                                                    \
  R Y##error_l_infty_1_complex(const CX *x, const CX *y, const NFFT_INT n,             \
                               const CX *z, const NFFT_INT m)                          \
  {                                                                                    \
    const R *a = (const R *)x, *b = (const R *)y, *c = (const R *)z;                   \
    R num = 0, den = 0;                                                                \
    for (NFFT_INT k = 0; k < n; k++) {                                                 \
      R t = std::hypot(a[2 * k] - b[2 * k], a[2 * k + 1] - b[2 * k + 1]);              \
      num = t > num ? t : num;                                                         \
    }                                                                                  \
    for (NFFT_INT k = 0; k < m; k++) den += std::hypot(c[2 * k], c[2 * k + 1]);        \
    return num / den;                                                                  \
  }                                                                                    \
  NFFT_INT Y##exp2i(const NFFT_INT a) { return (NFFT_INT)(1U << a); }                  \
  NFFT_INT Y##next_power_of_2(const NFFT_INT x)                                        \
  {                                                                                    \
    if (x < 0) return -1;                                                              \
    if (x < 2) return x + 1;                                                           \
    uint64_t v = (uint64_t)x - 1;                                                      \
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16; v |= v >> 32;   \
    return (NFFT_INT)(v + 1);                                                          \
  }                                                                                    \
  R Y##dot_complex(CX *x, NFFT_INT n)                                                  \
  {                                                                                    \
    const R *a = (const R *)x;                                                         \
    R s = 0;                                                                           \
    for (NFFT_INT k = 0; k < n; k++) s += a[2 * k] * a[2 * k] + a[2 * k + 1] * a[2 * k + 1]; \
    return s;                                                                          \
  }                                                                                    \
  void Y##upd_axpy_complex(CX *x, R a, CX *y, NFFT_INT n)                              \
  {                                                                                    \
    R *u = (R *)x;                                                                     \
    const R *v = (const R *)y;                                                         \
    for (NFFT_INT k = 0; k < 2 * n; k++) u[k] = a * u[k] + v[k];                       \
  }                                                                                    \
  void Y##fftshift_complex(CX *x, NFFT_INT d, NFFT_INT *N)                             \
  {                                                                                    \
    R *v = (R *)x;                                                                     \
    for (NFFT_INT da = 0; da < d; da++) {                                              \
      NFFT_INT Npre = 1, Npost = 1, Nact = N[da];                                      \
      for (NFFT_INT t = 0; t < da; t++) Npre *= N[t];                                  \
      for (NFFT_INT t = da + 1; t < d; t++) Npost *= N[t];                             \
      for (NFFT_INT kp = 0; kp < Npre; kp++)                                           \
        for (NFFT_INT ka = 0; ka < Nact / 2; ka++)                                     \
          for (NFFT_INT kq = 0; kq < Npost; kq++) {                                    \
            NFFT_INT k = (kp * Nact + ka) * Npost + kq;                                \
            NFFT_INT ks = (kp * Nact + ka + Nact / 2) * Npost + kq;                    \
            R t0 = v[2 * k], t1 = v[2 * k + 1];                                        \
            v[2 * k] = v[2 * ks]; v[2 * k + 1] = v[2 * ks + 1];                        \
            v[2 * ks] = t0; v[2 * ks + 1] = t1;                                        \
          }                                                                            \
    }                                                                                  \
  }                                                                                    \
  void Y##fftshift_complex_int(CX *x, int d, int *N)                                   \
  {                                                                                    \
    NFFT_INT NN[GB_MAXD];                                                              \
    for (int t = 0; t < d && t < GB_MAXD; t++) NN[t] = N[t];                           \
    Y##fftshift_complex(x, d, NN);                                                     \
  }                                                                                    \
  void Y##get_version(unsigned *major, unsigned *minor, unsigned *patch)               \
  {                                                                                    \
    *major = 3; *minor = 5; *patch = 4;                                                \
  }                                                                                    \
  const char *Y##get_window_name(void) { return "KAISER_BESSEL"; }

GB_UTIL_API(nfft_, double, fftw_complex)
GB_UTIL_API(nfftf_, float, fftwf_complex)

// default cut-off of the Kaiser-Bessel window (reference include/infft.h:224-230)
NFFT_INT nfft_get_default_window_cut_off(void) { return 8; }
NFFT_INT nfftf_get_default_window_cut_off(void) { return 4; }

}  // extern "C"
