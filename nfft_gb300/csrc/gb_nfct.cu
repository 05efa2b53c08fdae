// gb_nfct.cu -- NFCT, the nonequispaced fast cosine transform, reference
// kernel/nfct/nfct.c, both precisions:
//
//   f_j = sum_{0 <= k < N} f_hat_k prod_t cos(2 pi k_t x_jt),   x in [0, 1/2)^d
//   f_hat_k = sum_j f_j prod_t cos(2 pi k_t x_jt)                 (adjoint)
//
// The reference's factorisation (nfct.c:702-778) on the GPU:
//  * D: g_hat_k = f_hat_k prod_t c_t(k_t) / phi_hat(k_t), c = 1 at k_t = 0 and
//    1/2 elsewhere, zero-padded to the DCT-I lengths n_t;
//  * DCT-I (FFTW's REDFT00) of lengths n_t: the even extension of period
//    L_t = 2 (n_t - 1) through one real-to-complex cuFFT, real parts kept;
//  * B: f_j = sum over the 2m+2 taps l = u..o, u = rint(L x) - m, of
//    phi(x - l / L) g[l folded into [0, n - 1] by reflection at 0 and n - 1]
//    (nfct.c:261-268, 420-481), the Kaiser-Bessel window of grid length L;
//  * the adjoint: B^T with weight 1/2 per dimension at interior grid points
//    (nfct.c:445), the same DCT-I, then D without the 1/2.
// Kernels are generic over d (odometer over the taps as in the reference);
// the NFCT is not on the headline path and favours simplicity over speed.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>

#include "gb_common.cuh"

namespace gb {

template <typename R>
struct CtGeom {
  int d, m;
  int N[GB_MAXD], n[GB_MAXD], L[GB_MAXD];  // bandwidths, DCT-I lengths, window grid lengths 2 (n - 1)
  R b[GB_MAXD];
  long long M, N_total, n_total, ext_total;
};

template <typename R>
__device__ __forceinline__ R ct_phi(R x, int L, int m, R b)
{
  const R xn = x * (R)L;
  const R a = (R)m * (R)m - xn * xn;
  if (a > R(0)) {
    const R s = gb_sqrt(a);
    return gb_sinh(b * s) / (gb_pi<R>() * s);
  }
  if (a < R(0)) {
    const R s = gb_sqrt(-a);
    return gb_sin(b * s) / (gb_pi<R>() * s);
  }
  return b / gb_pi<R>();
}

// reflection of an unwrapped grid index into [0, n - 1] (period 2 (n - 1))
__device__ __forceinline__ int ct_fold(int l, int n)
{
  const int P = 2 * (n - 1);
  int r = l % P;
  if (r < 0) r += P;
  return r <= n - 1 ? r : P - r;
}

// D (trafo): g[i] over the n-grid; cphi[off_t + k] = 1 / phi_hat_t(k) in double
template <typename R>
__global__ void k_ct_dpad(CtGeom<R> g, const R *__restrict__ fhat, const double *__restrict__ cphi,
                          R *__restrict__ grid)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_total) return;
  long long rem = i, kl = 0, stride = 1;
  double c = 1.0;
  bool in = true;
  int off = 0;
  int kg[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    kg[t] = (int)(rem % g.n[t]);
    rem /= g.n[t];
  }
  for (int t = 0; t < g.d; ++t) {
    if (kg[t] >= g.N[t]) in = false;
  }
  if (!in) {
    grid[i] = R(0);
    return;
  }
  for (int t = g.d - 1; t >= 0; --t) {
    kl += stride * kg[t];
    stride *= g.N[t];
  }
  for (int t = 0; t < g.d; ++t) {
    c *= (kg[t] == 0 ? 1.0 : 0.5) * cphi[off + kg[t]];
    off += g.N[t];
  }
  grid[i] = (R)((double)fhat[kl] * c);
}

// D^T (adjoint): f_hat[k] = g[k] prod_t 1 / phi_hat_t(k_t)
template <typename R>
__global__ void k_ct_dcrop(CtGeom<R> g, const R *__restrict__ grid, const double *__restrict__ cphi,
                           R *__restrict__ fhat)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.N_total) return;
  long long rem = k, gi = 0, stride = 1;
  int kg[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    kg[t] = (int)(rem % g.N[t]);
    rem /= g.N[t];
  }
  double c = 1.0;
  int off = 0;
  for (int t = 0; t < g.d; ++t) {
    c *= cphi[off + kg[t]];
    off += g.N[t];
  }
  for (int t = g.d - 1; t >= 0; --t) {
    gi += stride * kg[t];
    stride *= g.n[t];
  }
  fhat[k] = (R)((double)grid[gi] * c);
}

// even extension of the n-grid to the L-grid (DCT-I as a real FFT)
template <typename R>
__global__ void k_ct_extend(CtGeom<R> g, const R *__restrict__ grid, R *__restrict__ ext)
{
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.ext_total) return;
  long long rem = e, src = 0, stride = 1;
  int idx[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    idx[t] = (int)(rem % g.L[t]);
    rem /= g.L[t];
  }
  for (int t = g.d - 1; t >= 0; --t) {
    const int s = idx[t] < g.n[t] ? idx[t] : g.L[t] - idx[t];
    src += stride * s;
    stride *= g.n[t];
  }
  ext[e] = grid[src];
}

// real parts of the half spectrum (last dimension L/2 + 1 long) back on the n-grid
template <typename R>
__global__ void k_ct_extract(CtGeom<R> g, const typename Cx<R>::T *__restrict__ spec, R *__restrict__ grid)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_total) return;
  long long rem = i, si = 0, stride = 1;
  int k[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    k[t] = (int)(rem % g.n[t]);
    rem /= g.n[t];
  }
  for (int t = g.d - 1; t >= 0; --t) {
    si += stride * k[t];
    stride *= (t == g.d - 1) ? (g.L[t] / 2 + 1) : g.L[t];
  }
  grid[i] = spec[si].x;
}

// B (trafo, ADJ = false: gather) and B^T (ADJ = true: scatter), one thread per
// node, taps in odometer order with per-dimension prefix products
template <typename R, bool ADJ>
__global__ void k_ct_b(CtGeom<R> g, const R *__restrict__ x, R *__restrict__ f, R *__restrict__ grid)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.M) return;
  const int w = 2 * g.m + 2;
  int u[GB_MAXD], lj[GB_MAXD];
  R xj[GB_MAXD];
  for (int t = 0; t < g.d; ++t) {
    xj[t] = x[j * g.d + t];
    u[t] = (int)lrint((double)(xj[t] * (R)g.L[t])) - g.m;  // nfct.c:261-268, LRINT in plan precision
    lj[t] = 0;
  }
  R pp[GB_MAXD + 1];
  long long lp[GB_MAXD + 1];
  pp[0] = R(1);
  lp[0] = 0;
  long long taps = 1;
  for (int t = 0; t < g.d; ++t) taps *= w;
  const R fj = ADJ ? f[j] : R(0);
  R acc = R(0);
  int t2 = 0;
  for (long long q = 0; q < taps; ++q) {
    for (int t = t2; t < g.d; ++t) {
      const int l = u[t] + lj[t];
      const int lf = ct_fold(l, g.n[t]);
      R ph = ct_phi<R>(xj[t] - (R)l / (R)g.L[t], g.L[t], g.m, g.b[t]);
      if (ADJ && lf != 0 && lf != g.n[t] - 1) ph *= R(0.5);
      pp[t + 1] = pp[t] * ph;
      lp[t + 1] = lp[t] * g.n[t] + lf;
    }
    if (ADJ) atomicAdd(&grid[lp[g.d]], pp[g.d] * fj);
    else acc += pp[g.d] * grid[lp[g.d]];
    // odometer: advance the last dimension, carry into earlier ones
    t2 = g.d - 1;
    while (++lj[t2] == w && t2 > 0) {
      lj[t2] = 0;
      --t2;
    }
  }
  if (!ADJ) f[j] = acc;
}

// direct transforms (nfct.c:88-255) in double arithmetic, one thread per output
template <typename R, bool ADJ>
__global__ void k_ct_direct(CtGeom<R> g, const R *__restrict__ x, const R *__restrict__ in, R *__restrict__ out)
{
  const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nout = ADJ ? g.N_total : g.M, nin = ADJ ? g.M : g.N_total;
  if (o >= nout) return;
  double s = 0.0;
  for (long long q = 0; q < nin; ++q) {
    const long long j = ADJ ? q : o;
    long long kl = ADJ ? o : q;
    double p = 1.0;
    for (int t = g.d - 1; t >= 0; --t) {
      const int k = (int)(kl % g.N[t]);
      kl /= g.N[t];
      p *= cospi(2.0 * (double)k * (double)x[j * g.d + t]);
    }
    s += (double)in[q] * p;
  }
  out[o] = (R)s;
}

}  // namespace gb

// ---------------------------------------------------------------- host side
#include <cstring>
#include <vector>

#include "../../include/nfft3.h"

namespace {

template <typename R> struct CtApi;
template <> struct CtApi<double> {
  typedef nfct_plan plan;
  static void *mal(size_t n) { return nfft_malloc(n); }
  static void fre(void *p) { nfft_free(p); }
  static NFFT_INT npow2(NFFT_INT v) { return nfft_next_power_of_2(v); }
  static const cufftType R2C = CUFFT_D2Z;
  static cufftResult exec(cufftHandle h, double *in, double2 *out) { return cufftExecD2Z(h, in, out); }
  static const int default_m = 8;
};
template <> struct CtApi<float> {
  typedef nfctf_plan plan;
  static void *mal(size_t n) { return nfftf_malloc(n); }
  static void fre(void *p) { nfftf_free(p); }
  static NFFT_INT npow2(NFFT_INT v) { return nfftf_next_power_of_2(v); }
  static const cufftType R2C = CUFFT_R2C;
  static cufftResult exec(cufftHandle h, float *in, float2 *out) { return cufftExecR2C(h, in, out); }
  static const int default_m = 4;
};

template <typename R>
struct CtCtx {
  gb::CtGeom<R> g;
  cudaStream_t s = nullptr;
  cufftHandle fft = 0;
  R *x = nullptr, *f = nullptr, *fhat = nullptr, *grid = nullptr, *ext = nullptr;
  typename gb::Cx<R>::T *spec = nullptr;
  double *cphi = nullptr;
  cudaEvent_t ev[4] = {};
};

unsigned ctb(long long n) { return (unsigned)((n + 255) / 256); }

template <typename R>
CtCtx<R> *ct_ctx(const typename CtApi<R>::plan *p)
{
  CtCtx<R> *c = reinterpret_cast<CtCtx<R> *>(p->my_fftw_r2r_plan);
  if (!c) gb::fatal("nfct: plan has no device context (not initialised by this library)");
  return c;
}

template <typename R>
void ct_init_help(typename CtApi<R>::plan *ths)
{
  typedef CtApi<R> A;
  const int d = (int)ths->d;
  if (d < 1 || d > 3) gb::fatal("nfct: dimension %d not supported on the GPU (1..3)", d);
  ths->N_total = 1;
  ths->n_total = 1;
  for (int t = 0; t < d; ++t) {  // nfct.c:927-940
    ths->N_total *= ths->N[t];
    ths->n_total *= ths->n[t];
  }
  ths->sigma = (R *)A::mal((size_t)d * sizeof(R));
  ths->b = (R *)A::mal((size_t)d * sizeof(R));
  ths->r2r_kind = (int *)A::mal((size_t)d * sizeof(int));
  for (int t = 0; t < d; ++t) {
    ths->sigma[t] = (R)(ths->n[t] - 1) / (R)ths->N[t];
    ths->b[t] = (R)3.1415926535897932384626433832795028841971693993751 * ((R)2.0 - (R)1.0 / ths->sigma[t]);
    ths->r2r_kind[t] = 0;  // FFTW_REDFT00
  }
  if (ths->flags & MALLOC_X) ths->x = (R *)A::mal((size_t)(d * ths->M_total) * sizeof(R));
  if (ths->flags & MALLOC_F_HAT) ths->f_hat = (R *)A::mal((size_t)ths->N_total * sizeof(R));
  if (ths->flags & MALLOC_F) ths->f = (R *)A::mal((size_t)ths->M_total * sizeof(R));
  // the window is evaluated on the fly: no psi tables; grids live on the device
  ths->psi = nullptr;
  ths->psi_index_g = ths->psi_index_f = nullptr;
  ths->g = ths->g_hat = ths->g1 = ths->g2 = nullptr;
  ths->spline_coeffs = nullptr;
  ths->K = (ths->flags & PRE_LIN_PSI) ? (NFFT_INT)((1U << 10) * (ths->m + 2)) : 0;
  ths->MEASURE_TIME_t[0] = ths->MEASURE_TIME_t[1] = ths->MEASURE_TIME_t[2] = 0;

  CtCtx<R> *c = new CtCtx<R>();
  gb::CtGeom<R> &g = c->g;
  g.d = d;
  g.m = (int)ths->m;
  g.M = ths->M_total;
  g.N_total = ths->N_total;
  g.n_total = ths->n_total;
  g.ext_total = 1;
  int L[3];
  for (int t = 0; t < d; ++t) {
    g.N[t] = (int)ths->N[t];
    g.n[t] = (int)ths->n[t];
    g.L[t] = 2 * (g.n[t] - 1);
    g.b[t] = ths->b[t];
    g.ext_total *= g.L[t];
    L[t] = g.L[t];
    if (g.n[t] < 2) gb::fatal("nfct: DCT-I length n[%d] = %d below 2", t, g.n[t]);
  }
  // 1 / phi_hat(k) of the window with grid length L (nfct.c:780-800), double
  std::vector<double> ch;
  for (int t = 0; t < d; ++t)
    for (int k = 0; k < g.N[t]; ++k) {
      const double a = 2.0 * M_PI * k / (double)g.L[t];
      ch.push_back(1.0 / std::cyl_bessel_i(0.0, (double)g.m * std::sqrt((double)g.b[t] * g.b[t] - a * a)));
    }
  if (ths->flags & PRE_PHI_HUT) {
    ths->c_phi_inv = (R **)A::mal((size_t)d * sizeof(R *));
    size_t off = 0;
    for (int t = 0; t < d; ++t) {
      ths->c_phi_inv[t] = (R *)A::mal((size_t)g.N[t] * sizeof(R));
      for (int k = 0; k < g.N[t]; ++k) ths->c_phi_inv[t][k] = (R)ch[off + k];
      off += g.N[t];
    }
  } else {
    ths->c_phi_inv = nullptr;
  }
  GB_CUDA(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
  for (int i = 0; i < 4; ++i) GB_CUDA(cudaEventCreate(&c->ev[i]));
  const size_t Mz = (size_t)(g.M > 0 ? g.M : 1);
  long long spec_total = 1;
  for (int t = 0; t < d; ++t) spec_total *= (t == d - 1) ? (L[t] / 2 + 1) : L[t];
  GB_CUDA(cudaMalloc((void **)&c->x, Mz * d * sizeof(R)));
  GB_CUDA(cudaMalloc((void **)&c->f, Mz * sizeof(R)));
  GB_CUDA(cudaMalloc((void **)&c->fhat, (size_t)g.N_total * sizeof(R)));
  GB_CUDA(cudaMalloc((void **)&c->grid, (size_t)g.n_total * sizeof(R)));
  GB_CUDA(cudaMalloc((void **)&c->ext, (size_t)g.ext_total * sizeof(R)));
  GB_CUDA(cudaMalloc((void **)&c->spec, (size_t)spec_total * sizeof(typename gb::Cx<R>::T)));
  GB_CUDA(cudaMalloc((void **)&c->cphi, ch.size() * sizeof(double)));
  GB_CUDA(cudaMemcpy(c->cphi, ch.data(), ch.size() * sizeof(double), cudaMemcpyHostToDevice));
  if (cufftPlanMany(&c->fft, d, L, nullptr, 1, 0, nullptr, 1, 0, A::R2C, 1) != CUFFT_SUCCESS)
    gb::fatal("nfct: cuFFT plan failed");
  cufftSetStream(c->fft, c->s);
  ths->my_fftw_r2r_plan = reinterpret_cast<decltype(ths->my_fftw_r2r_plan)>(c);
}

// DCT-I of the device grid in place (even extension, real FFT, real parts)
template <typename R>
void ct_dct(CtCtx<R> *c)
{
  gb::k_ct_extend<R><<<ctb(c->g.ext_total), 256, 0, c->s>>>(c->g, c->grid, c->ext);
  if (CtApi<R>::exec(c->fft, c->ext, c->spec) != CUFFT_SUCCESS) gb::fatal("nfct: cuFFT exec failed");
  gb::k_ct_extract<R><<<ctb(c->g.n_total), 256, 0, c->s>>>(c->g, c->spec, c->grid);
}

template <typename R>
void ct_times(typename CtApi<R>::plan *ths, CtCtx<R> *c)
{
  GB_CUDA(cudaEventSynchronize(c->ev[3]));
  float a, b, e;
  cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&e, c->ev[2], c->ev[3]);
  ths->MEASURE_TIME_t[0] = a * 1e-3;
  ths->MEASURE_TIME_t[1] = b * 1e-3;
  ths->MEASURE_TIME_t[2] = e * 1e-3;
}

template <typename R>
void ct_trafo(typename CtApi<R>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R>(ths);
  const gb::CtGeom<R> &g = c->g;
  if (!ths->x || !ths->f_hat || !ths->f) gb::fatal("nfct: x, f_hat or f not set");
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemcpyAsync(c->fhat, ths->f_hat, (size_t)g.N_total * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaEventRecord(c->ev[0], c->s));
  gb::k_ct_dpad<R><<<ctb(g.n_total), 256, 0, c->s>>>(g, c->fhat, c->cphi, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[1], c->s));
  ct_dct<R>(c);
  GB_CUDA(cudaEventRecord(c->ev[2], c->s));
  if (g.M > 0) gb::k_ct_b<R, false><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->f, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[3], c->s));
  GB_LAUNCHED("nfct_trafo");
  GB_CUDA(cudaMemcpyAsync(ths->f, c->f, (size_t)g.M * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
  ct_times<R>(ths, c);
}

template <typename R>
void ct_adjoint(typename CtApi<R>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R>(ths);
  const gb::CtGeom<R> &g = c->g;
  if (!ths->x || !ths->f_hat || !ths->f) gb::fatal("nfct: x, f_hat or f not set");
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemcpyAsync(c->f, ths->f, (size_t)g.M * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemsetAsync(c->grid, 0, (size_t)g.n_total * sizeof(R), c->s));
  GB_CUDA(cudaEventRecord(c->ev[0], c->s));
  if (g.M > 0) gb::k_ct_b<R, true><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->f, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[1], c->s));
  ct_dct<R>(c);
  GB_CUDA(cudaEventRecord(c->ev[2], c->s));
  gb::k_ct_dcrop<R><<<ctb(g.N_total), 256, 0, c->s>>>(g, c->grid, c->cphi, c->fhat);
  GB_CUDA(cudaEventRecord(c->ev[3], c->s));
  GB_LAUNCHED("nfct_adjoint");
  GB_CUDA(cudaMemcpyAsync(ths->f_hat, c->fhat, (size_t)g.N_total * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
  // timings: D^T, DCT, B^T in the reference's order of MEASURE_TIME_t
  float a, b, e;
  cudaEventElapsedTime(&e, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&a, c->ev[2], c->ev[3]);
  ths->MEASURE_TIME_t[0] = a * 1e-3;
  ths->MEASURE_TIME_t[1] = b * 1e-3;
  ths->MEASURE_TIME_t[2] = e * 1e-3;
}

template <typename R, bool ADJ>
void ct_direct(const typename CtApi<R>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R>(ths);
  const gb::CtGeom<R> &g = c->g;
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  if (ADJ) {
    GB_CUDA(cudaMemcpyAsync(c->f, ths->f, (size_t)g.M * sizeof(R), cudaMemcpyHostToDevice, c->s));
    if (g.N_total > 0) gb::k_ct_direct<R, true><<<ctb(g.N_total), 256, 0, c->s>>>(g, c->x, c->f, c->fhat);
    GB_CUDA(cudaMemcpyAsync(ths->f_hat, c->fhat, (size_t)g.N_total * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  } else {
    GB_CUDA(cudaMemcpyAsync(c->fhat, ths->f_hat, (size_t)g.N_total * sizeof(R), cudaMemcpyHostToDevice, c->s));
    if (g.M > 0) gb::k_ct_direct<R, false><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->fhat, c->f);
    GB_CUDA(cudaMemcpyAsync(ths->f, c->f, (size_t)g.M * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  }
  GB_LAUNCHED("nfct_direct");
  GB_CUDA(cudaStreamSynchronize(c->s));
}

template <typename R>
const char *ct_check(typename CtApi<R>::plan *ths)
{
  // nfct.c:1108-1138
  if (!ths->f) return "Member f not initialized.";
  if (!ths->x) return "Member x not initialized.";
  if (!ths->f_hat) return "Member f_hat not initialized.";
  for (NFFT_INT j = 0; j < ths->M_total * ths->d; ++j)
    if (ths->x[j] < (R)0.0 || ths->x[j] >= (R)0.5) return "ths->x out of range [0.0,0.5)";
  for (NFFT_INT t = 0; t < ths->d; ++t) {
    if (ths->sigma[t] <= 1) return "Oversampling factor too small";
    if (ths->N[t] - 1 <= ths->m) return "Polynomial degree N is smaller than cut-off m";
  }
  return nullptr;
}

template <typename R>
void ct_finalize(typename CtApi<R>::plan *ths)
{
  typedef CtApi<R> A;
  CtCtx<R> *c = reinterpret_cast<CtCtx<R> *>(ths->my_fftw_r2r_plan);
  if (c) {
    cudaStreamSynchronize(c->s);
    cufftDestroy(c->fft);
    cudaFree(c->x);
    cudaFree(c->f);
    cudaFree(c->fhat);
    cudaFree(c->grid);
    cudaFree(c->ext);
    cudaFree(c->spec);
    cudaFree(c->cphi);
    for (int i = 0; i < 4; ++i) cudaEventDestroy(c->ev[i]);
    cudaStreamDestroy(c->s);
    delete c;
    ths->my_fftw_r2r_plan = nullptr;
  }
  if (ths->c_phi_inv) {
    for (NFFT_INT t = 0; t < ths->d; ++t) A::fre(ths->c_phi_inv[t]);
    A::fre(ths->c_phi_inv);
  }
  if (ths->flags & MALLOC_F) A::fre(ths->f);
  if (ths->flags & MALLOC_F_HAT) A::fre(ths->f_hat);
  if (ths->flags & MALLOC_X) A::fre(ths->x);
  A::fre(ths->b);
  A::fre(ths->N);
  A::fre(ths->n);
  A::fre(ths->sigma);
  A::fre(ths->r2r_kind);
}

template <typename R>
void ct_init_guru(typename CtApi<R>::plan *ths, int d, int *N, int M_total, int *n, int m, unsigned flags,
                  unsigned fftw_flags)
{
  typedef CtApi<R> A;
  ths->d = d;
  ths->M_total = M_total;
  ths->N = (NFFT_INT *)A::mal((size_t)d * sizeof(NFFT_INT));
  ths->n = (NFFT_INT *)A::mal((size_t)d * sizeof(NFFT_INT));
  for (int t = 0; t < d; ++t) {
    ths->N[t] = N[t];
    ths->n[t] = n[t];
  }
  ths->m = m;
  ths->flags = flags;
  ths->fftw_flags = fftw_flags;
  ct_init_help<R>(ths);
}

template <typename R>
void ct_init(typename CtApi<R>::plan *ths, int d, int *N, int M_total)
{
  // nfct.c:1014-1051: n = 2 (next_power_of_2(N) - 1), default m, default flags
  std::vector<int> n(d);
  for (int t = 0; t < d; ++t) n[t] = (int)(2 * (CtApi<R>::npow2(N[t]) - 1));
  const unsigned flags = PRE_PHI_HUT | PRE_PSI | MALLOC_X | MALLOC_F_HAT | MALLOC_F | FFTW_INIT |
                         (d > 1 ? NFFT_SORT_NODES : FFT_OUT_OF_PLACE);
  ct_init_guru<R>(ths, d, N, M_total, n.data(), CtApi<R>::default_m, flags, FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
}

}  // namespace

#define GB_NFCT_API(P, R)                                                                                  \
  extern "C" {                                                                                             \
  void P##init_guru(P##plan *ths, int d, int *N, int M_total, int *n, int m, unsigned flags,              \
                    unsigned fftw_flags)                                                                   \
  {                                                                                                        \
    ct_init_guru<R>(ths, d, N, M_total, n, m, flags, fftw_flags);                                          \
    ths->mv_trafo = (void (*)(void *))P##trafo;                                                            \
    ths->mv_adjoint = (void (*)(void *))P##adjoint;                                                        \
  }                                                                                                        \
  void P##init(P##plan *ths, int d, int *N, int M_total)                                                   \
  {                                                                                                        \
    ct_init<R>(ths, d, N, M_total);                                                                        \
    ths->mv_trafo = (void (*)(void *))P##trafo;                                                            \
    ths->mv_adjoint = (void (*)(void *))P##adjoint;                                                        \
  }                                                                                                        \
  void P##init_1d(P##plan *ths, int N0, int M_total) { P##init(ths, 1, &N0, M_total); }                   \
  void P##init_2d(P##plan *ths, int N0, int N1, int M_total)                                               \
  {                                                                                                        \
    int N[2] = {N0, N1};                                                                                   \
    P##init(ths, 2, N, M_total);                                                                           \
  }                                                                                                        \
  void P##init_3d(P##plan *ths, int N0, int N1, int N2, int M_total)                                       \
  {                                                                                                        \
    int N[3] = {N0, N1, N2};                                                                               \
    P##init(ths, 3, N, M_total);                                                                           \
  }                                                                                                        \
  /* the window is evaluated on the fly: the precompute calls have nothing to do */                       \
  void P##precompute_one_psi(P##plan *ths) { (void)ct_ctx<R>(ths); }                                       \
  void P##precompute_psi(P##plan *ths) { (void)ct_ctx<R>(ths); }                                           \
  void P##precompute_full_psi(P##plan *ths) { (void)ct_ctx<R>(ths); }                                      \
  void P##precompute_fg_psi(P##plan *ths) { (void)ct_ctx<R>(ths); }                                        \
  void P##precompute_lin_psi(P##plan *ths) { (void)ct_ctx<R>(ths); }                                       \
  void P##trafo(P##plan *ths) { ct_trafo<R>(ths); }                                                        \
  void P##adjoint(P##plan *ths) { ct_adjoint<R>(ths); }                                                    \
  void P##trafo_direct(const P##plan *ths) { ct_direct<R, false>(ths); }                                   \
  void P##adjoint_direct(const P##plan *ths) { ct_direct<R, true>(ths); }                                  \
  const char *P##check(P##plan *ths) { return ct_check<R>(ths); }                                          \
  void P##finalize(P##plan *ths) { ct_finalize<R>(ths); }                                                  \
  }

GB_NFCT_API(nfct_, double)
GB_NFCT_API(nfctf_, float)
