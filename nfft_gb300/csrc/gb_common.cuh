// gb_common.cuh -- shared types and device helpers of the GB300 NFFT library.
//
// Conventions (matching the reference NFFT 3):
//  * x is node-major, x[j*d + t] in [-1/2, 1/2) (reference nfft.c:6185-6191);
//  * f_hat is row-major over k_t = -N_t/2 .. N_t/2-1, last dimension fastest;
//  * the oversampled grid g has n_t points per dimension in FFT order;
//  * node j's window covers grid indices u_t .. u_t + 2m + 1 (mod n_t) with
//    u_t = floor(x_t n_t) - m (reference nfft.c:324-340), and the window
//    argument uses the unwrapped index (reference nfft.c:5838-5840).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#define GB_MAXD 8          // largest dimension d the library accepts
#define GB_MAXW 66         // largest window width 2m+2 (m <= 32)

namespace gb {

template <typename R> struct Cx;
template <> struct Cx<float> { typedef float2 T; };
template <> struct Cx<double> { typedef double2 T; };

// ---------------------------------------------------------------- errors
void record_error(const char *fmt, ...);
void fatal(const char *fmt, ...);  // records, then calls nfft_die (exits)
// Raises `kernel`'s dynamic shared-memory limit to at least `bytes` on the
// current device.  The attribute is per device, so this keeps one record per
// (device, kernel) and sets it where it is still lower; a mutex makes first
// calls from several host threads safe.
void set_smem_limit(const void *kernel, size_t bytes);
void check_cuda(cudaError_t e, const char *what, const char *file, int line);
void check_launch(const char *what, const char *file, int line);

#define GB_CUDA(call) ::gb::check_cuda((call), #call, __FILE__, __LINE__)
#define GB_LAUNCHED(name) ::gb::check_launch(name, __FILE__, __LINE__)

// ---------------------------------------------------------------- geometry
// Everything a transform kernel needs about the plan, passed by value.
template <typename R>
struct Geom {
  int d;
  int m;
  int w;                 // 2m+2
  int n[GB_MAXD];        // grid lengths
  int N[GB_MAXD];        // bandwidths
  R nR[GB_MAXD];         // (R) n_t
  R b[GB_MAXD];          // KB shape parameter per dim, pi (2 - 1/sigma_t)
  R mm;                  // (R) m * (R) m
  long long M;           // nodes
  long long n_total;
  long long N_total;
  // tiling of the grid for the shared-memory kernels
  int T[GB_MAXD];        // tile edge per dim
  int ntile[GB_MAXD];    // tiles per dim (n_t / T_t, rounded up)
  int ext[GB_MAXD];      // padded subgrid edge T_t + w - 1
  int cs;                // sub-cell edge of the 3-D group kernels (1 = off)
  int csz;               // sub-cell edge along the last dimension (z-column kernels: 1)
  int sub;               // sub-cells per tile ((T/cs)^(d-1) (T/csz), 1 = off)
  int sx, sy;            // shared-memory plane strides of the group kernels (x, y)
};

// Polynomial form of the Kaiser-Bessel window (single-precision 3-D
// kernels): tap l of a node is sum_k c[t][l][k] s^k with s = 2 frac(n x) - 1.
#define KB_POLY_DP 10    // coefficients per tap (degree 9)
#define KB_POLY_WMAX 16  // widest window with a polynomial form
struct WinPoly {
  float c[3][KB_POLY_WMAX][KB_POLY_DP];  // per dimension, tap, increasing power of s
  int same;                              // every dimension has the same b (c[0] serves all)
};
// fills coef[l * KB_POLY_DP + k] for the w taps of the window with cut-off m
// and shape b (host, double precision)
void kb_poly_fit(int m, double b, int w, float *coef);
// The same in double precision for the 2-D double-precision kernels: degree
// 16, interpolated in extended precision, within 5e-15 of the window's peak.
#define KB_POLYD_DP 17
struct WinPolyD {
  double c[2][KB_POLY_WMAX][KB_POLYD_DP];  // per dimension, tap, increasing power of s
};
void kb_polyd_fit(int m, double b, int w, double *coef);

struct WorkItem {
  int tile;    // linear tile id (row-major over ntile)
  int start;   // first sorted node
  int end;     // one past last sorted node
  int pad;
};

#ifdef __CUDACC__
// ---------------------------------------------------------------- window
template <typename R> __device__ __forceinline__ R gb_pi();
template <> __device__ __forceinline__ float gb_pi<float>() { return 3.14159265358979323846f; }
template <> __device__ __forceinline__ double gb_pi<double>() { return 3.14159265358979323846; }

__device__ __forceinline__ float gb_sqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double gb_sqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float gb_sinh(float v) { return sinhf(v); }
__device__ __forceinline__ double gb_sinh(double v) { return sinh(v); }
__device__ __forceinline__ float gb_sin(float v) { return sinf(v); }
__device__ __forceinline__ double gb_sin(double v) { return sin(v); }
__device__ __forceinline__ float gb_floor(float v) { return floorf(v); }
__device__ __forceinline__ double gb_floor(double v) { return floor(v); }

// Kaiser-Bessel window phi(xl) for grid length n, where xl = x - l/n
// (reference include/infft.h:209-215): sinh(b s)/(pi s) with
// s = sqrt(m^2 - (n xl)^2) inside the support, sin(b s)/(pi s) with
// s = sqrt((n xl)^2 - m^2) outside, b/pi on the boundary.
template <typename R>
__device__ __forceinline__ R kb_phi(R xl, R nR, R mm, R b)
{
  const R t = xl * nR;
  const R t2 = t * t;
  const R arg = mm - t2;
  if (arg > R(0)) {
    const R s = gb_sqrt(arg);
    return gb_sinh(b * s) / (gb_pi<R>() * s);
  } else if (arg < R(0)) {
    const R s = gb_sqrt(t2 - mm);
    return gb_sin(b * s) / (gb_pi<R>() * s);
  }
  return b / gb_pi<R>();
}

// The same window as a function of t = n (x - l/n) (the argument the macro
// forms first); kb_phi_t is the accurate form, kb_phi_t_fast the single
// precision form of the 3-D group kernels: rsqrt instead of sqrt and a
// division, sinh from one accurate expf and an approximate reciprocal (the
// e^{-y} term matters only where the weight is near its smallest, b/pi, far
// below the window's peak), and the approximate sine on the two outer taps,
// whose weights are of order b/pi against a peak of sinh(b m)/(pi m).
template <typename R>
__device__ __forceinline__ R kb_phi_t(R t, R mm, R b)
{
  const R t2 = t * t;
  const R arg = mm - t2;
  if (arg > R(0)) {
    const R s = gb_sqrt(arg);
    return gb_sinh(b * s) / (gb_pi<R>() * s);
  } else if (arg < R(0)) {
    const R s = gb_sqrt(t2 - mm);
    return gb_sin(b * s) / (gb_pi<R>() * s);
  }
  return b / gb_pi<R>();
}

__device__ __forceinline__ float kb_phi_t_fast(float t, float mm, float b)
{
  const float inv_pi = 0.318309886183790671538f;
  const float arg = mm - t * t;
  if (arg > 0.f) {
    const float r = rsqrtf(arg);
    const float e = expf(b * (arg * r));
    return 0.5f * (e - __fdividef(1.f, e)) * (r * inv_pi);
  } else if (arg < 0.f) {
    const float r = rsqrtf(-arg);
    return __sinf(b * (-arg * r)) * (r * inv_pi);
  }
  return b * inv_pi;
}

__device__ __forceinline__ float kb_window_t(float t, float mm, float b) { return kb_phi_t_fast(t, mm, b); }

// the W taps of a node from its polynomial form, s = 2 frac(n x) - 1
template <int W>
__device__ __forceinline__ void kb_poly_taps_s(float s, const float (&c)[KB_POLY_WMAX][KB_POLY_DP], float (&v)[W])
{
  static_assert(W <= KB_POLY_WMAX, "no polynomial form for this width");
#pragma unroll
  for (int l = 0; l < W; ++l) {
    float a = c[l][KB_POLY_DP - 1];
#pragma unroll
    for (int k = KB_POLY_DP - 2; k >= 0; --k) a = fmaf(a, s, c[l][k]);
    v[l] = a;
  }
}

// The same W taps from the window's symmetry: tap W-1-l at s equals tap l at
// -s (the Kaiser-Bessel window is even and the taps are symmetric about the
// window centre), so with P_l(s) = E_l(s^2) + s O_l(s^2) split into its even
// and odd powers, taps l and W-1-l are E_l + s O_l and E_l - s O_l: two
// degree-4 Horner chains in s^2 per pair of taps (10 multiply-adds instead of
// 18), from the coefficients of the first W/2 taps only.
template <int W>
__device__ __forceinline__ void kb_poly_taps_sym(float s, const float (&c)[KB_POLY_WMAX][KB_POLY_DP], float (&v)[W])
{
  static_assert(W <= KB_POLY_WMAX && W % 2 == 0, "even width with a polynomial form");
  static_assert(KB_POLY_DP == 10, "degree-9 form: five even and five odd coefficients");
  const float t = s * s;
#pragma unroll
  for (int l = 0; l < W / 2; ++l) {
    float e = c[l][8], o = c[l][9];
    e = fmaf(e, t, c[l][6]);
    o = fmaf(o, t, c[l][7]);
    e = fmaf(e, t, c[l][4]);
    o = fmaf(o, t, c[l][5]);
    e = fmaf(e, t, c[l][2]);
    o = fmaf(o, t, c[l][3]);
    e = fmaf(e, t, c[l][0]);
    o = fmaf(o, t, c[l][1]);
    v[l] = fmaf(s, o, e);
    v[W - 1 - l] = fmaf(-s, o, e);
  }
}

// double precision: the W taps of a node from the degree-16 form
template <int W>
__device__ __forceinline__ void kb_polyd_taps_s(double s, const double (&c)[KB_POLY_WMAX][KB_POLYD_DP],
                                                double (&v)[W])
{
  static_assert(W <= KB_POLY_WMAX, "no polynomial form for this width");
#pragma unroll
  for (int l = 0; l < W; ++l) {
    double a = c[l][KB_POLYD_DP - 1];
#pragma unroll
    for (int k = KB_POLYD_DP - 2; k >= 0; --k) a = fma(a, s, c[l][k]);
    v[l] = a;
  }
}

// the same from t0 = n x - u in [m, m+1)
template <int W>
__device__ __forceinline__ void kb_poly_taps(float t0, int m, const float (&c)[KB_POLY_WMAX][KB_POLY_DP],
                                             float (&v)[W])
{
  static_assert(W <= KB_POLY_WMAX, "no polynomial form for this width");
  const float s = fmaf(2.f, t0, -(float)(2 * m + 1));  // exact: 2 (t0 - m) - 1
#pragma unroll
  for (int l = 0; l < W; ++l) {
    float a = c[l][KB_POLY_DP - 1];
#pragma unroll
    for (int k = KB_POLY_DP - 2; k >= 0; --k) a = fmaf(a, s, c[l][k]);
    v[l] = a;
  }
}
__device__ __forceinline__ double kb_window_t(double t, double mm, double b) { return kb_phi_t<double>(t, mm, b); }

// Unwrapped window start u = floor(x n) - m (reference nfft.c:324-332).  The
// same expression is used by the binning and by every transform kernel so a
// node lands in the same tile everywhere.
template <typename R>
__device__ __forceinline__ int node_u(R x, R nR, int m)
{
  return (int)gb_floor(x * nR) - m;
}

__device__ __forceinline__ int wrap(int i, int n)
{
  int r = i % n;
  return r < 0 ? r + n : r;
}

// window values of one node in one dimension: out[l] = phi(x - (u+l)/n)
template <typename R, int W>
__device__ __forceinline__ void node_psi(R x, int u, R nR, R mm, R b, R *out)
{
#pragma unroll
  for (int l = 0; l < W; ++l)
    out[l] = kb_phi<R>(x - R(u + l) / nR, nR, mm, b);
}

template <typename R>
__device__ __forceinline__ void node_psi_rt(R x, int u, int w, R nR, R mm, R b, R *out)
{
  for (int l = 0; l < w; ++l)
    out[l] = kb_phi<R>(x - R(u + l) / nR, nR, mm, b);
}

// complex helpers
__device__ __forceinline__ float2 cmake(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 cmake(double a, double b) { return make_double2(a, b); }

__device__ __forceinline__ void atomic_add_c(float2 *p, float2 v)
{
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void atomic_add_c(double2 *p, double2 v)
{
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
// global complex accumulate: one vector reduction for float2 on sm_90+
__device__ __forceinline__ void global_add_c(float2 *p, float2 v)
{
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  atomicAdd(p, v);
#else
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
#endif
}
__device__ __forceinline__ void global_add_c(double2 *p, double2 v)
{
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
#endif  // __CUDACC__

}  // namespace gb
