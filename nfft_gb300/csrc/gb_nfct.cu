// gb_nfct.cu -- NFCT and NFST, the nonequispaced fast cosine and sine
// transforms, reference kernel/nfct/nfct.c and kernel/nfst/nfst.c, both
// precisions:
//
//   NFCT: f_j = sum_{0 <= k < N} f_hat_k prod_t cos(2 pi k_t x_jt)
//   NFST: f_j = sum_{1 <= k < N} f_hat_{k-1} prod_t sin(2 pi k_t x_jt)
//   (x in [0, 1/2)^d; the adjoints are the transposed sums)
//
// The reference's factorisation (nfct.c / nfst.c:702-778) on the GPU, with
// S = 0 for the cosine and S = 1 for the sine transform:
//  * D: g_hat_k = f_hat_k prod_t c_t(k_t) / phi_hat(k_t + S) on the grid of
//    DCT-I / DST-I lengths n_t; c = 1 at k_t = 0 and 1/2 elsewhere for the
//    cosine, 1/2 throughout for the sine (and in the sine's D^T);
//  * DCT-I (FFTW's REDFT00) or DST-I (RODFT00): the even (odd) extension of
//    period L_t = 2 (n_t - 1) (2 (n_t + 1)) through one real-to-complex
//    cuFFT;
//  * B: f_j = sum over the 2m+2 taps l = u..o, u = rint(L x) - m, of
//    phi(x - l / L) times the extended grid at l (nfct.c:261-268, 420-481):
//    for the cosine the index reflected into [0, n - 1]; for the sine the
//    odd extension's value (zero at 0 and L/2, sign -1 beyond L/2);
//  * the adjoints: B^T with the cosine's weight 1/2 per dimension at interior
//    grid points (the sine's signs), the same DCT-I / DST-I, then D^T.
// Kernels are generic over d <= 3 (the tap odometer of the reference); these
// transforms are not on the headline path and favour simplicity over speed.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>

#include "gb_common.cuh"

namespace gb {

template <typename R>
struct CtGeom {
  int d, m;
  int N[GB_MAXD], Nf[GB_MAXD], n[GB_MAXD], L[GB_MAXD];  // bandwidth, frequencies N - S, grid, extension period
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

// grid index and sign of the extended grid at the unwrapped index l
// (period L); sign 0 where the sine's odd extension vanishes
template <bool S>
__device__ __forceinline__ int ct_tap(int l, int n, int L, int &sign)
{
  int p = l % L;
  if (p < 0) p += L;
  if (!S) {
    sign = 1;
    return p <= n - 1 ? p : L - p;
  }
  const int h = L / 2;  // n + 1
  if (p == 0 || p == h) {
    sign = 0;
    return 0;
  }
  sign = p < h ? 1 : -1;
  return p < h ? p - 1 : L - p - 1;
}

// D (trafo) over the n-grid; cphi[off_t + k] = 1 / phi_hat_t(k + S) in double
template <typename R, bool S>
__global__ void k_ct_dpad(CtGeom<R> g, const R *__restrict__ fhat, const double *__restrict__ cphi,
                          R *__restrict__ grid)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_total) return;
  long long rem = i, kl = 0, stride = 1;
  int kg[GB_MAXD];
  bool in = true;
  for (int t = g.d - 1; t >= 0; --t) {
    kg[t] = (int)(rem % g.n[t]);
    rem /= g.n[t];
    if (kg[t] >= g.Nf[t]) in = false;
  }
  if (!in) {
    grid[i] = R(0);
    return;
  }
  for (int t = g.d - 1; t >= 0; --t) {
    kl += stride * kg[t];
    stride *= g.Nf[t];
  }
  double c = 1.0;
  int off = 0;
  for (int t = 0; t < g.d; ++t) {
    c *= ((S || kg[t] != 0) ? 0.5 : 1.0) * cphi[off + kg[t]];
    off += g.Nf[t];
  }
  grid[i] = (R)((double)fhat[kl] * c);
}

// D^T (adjoint)
template <typename R, bool S>
__global__ void k_ct_dcrop(CtGeom<R> g, const R *__restrict__ grid, const double *__restrict__ cphi,
                           R *__restrict__ fhat)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.N_total) return;
  long long rem = k, gi = 0, stride = 1;
  int kg[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    kg[t] = (int)(rem % g.Nf[t]);
    rem /= g.Nf[t];
  }
  double c = 1.0;
  int off = 0;
  for (int t = 0; t < g.d; ++t) {
    c *= (S ? 0.5 : 1.0) * cphi[off + kg[t]];
    off += g.Nf[t];
  }
  for (int t = g.d - 1; t >= 0; --t) {
    gi += stride * kg[t];
    stride *= g.n[t];
  }
  fhat[k] = (R)((double)grid[gi] * c);
}

// even (odd) extension of the n-grid to the L-grid
template <typename R, bool S>
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
  int sign = 1;
  for (int t = g.d - 1; t >= 0; --t) {
    int s;
    const int q = ct_tap<S>(idx[t], g.n[t], g.L[t], s);
    sign *= s;
    src += stride * q;
    stride *= g.n[t];
  }
  ext[e] = sign == 0 ? R(0) : (sign > 0 ? grid[src] : -grid[src]);
}

// the transform from the half spectrum (last dimension L/2 + 1 long): real
// parts at k for the DCT-I; for the DST-I the spectrum at k + 1 times i^d
template <typename R, bool S>
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
    si += stride * (k[t] + (S ? 1 : 0));
    stride *= (t == g.d - 1) ? (g.L[t] / 2 + 1) : g.L[t];
  }
  const typename Cx<R>::T v = spec[si];
  if (!S) {
    grid[i] = v.x;
  } else {
    switch (g.d & 3) {  // real part of i^d v
      case 1: grid[i] = -v.y; break;
      case 2: grid[i] = -v.x; break;
      case 3: grid[i] = v.y; break;
      default: grid[i] = v.x; break;
    }
  }
}

// B (ADJ = false: gather) and B^T (ADJ = true: scatter), one thread per node
template <typename R, bool S, bool ADJ>
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
      int sign;
      const int li = ct_tap<S>(l, g.n[t], g.L[t], sign);
      R ph = ct_phi<R>(xj[t] - (R)l / (R)g.L[t], g.L[t], g.m, g.b[t]) * (R)sign;
      if (!S && ADJ && li != 0 && li != g.n[t] - 1) ph *= R(0.5);
      pp[t + 1] = pp[t] * ph;
      lp[t + 1] = lp[t] * g.n[t] + li;
    }
    if (ADJ) atomicAdd(&grid[lp[g.d]], pp[g.d] * fj);
    else acc += pp[g.d] * grid[lp[g.d]];
    t2 = g.d - 1;  // odometer: advance the last dimension, carry into earlier ones
    while (++lj[t2] == w && t2 > 0) {
      lj[t2] = 0;
      --t2;
    }
  }
  if (!ADJ) f[j] = acc;
}

// direct transforms (nfct.c / nfst.c:88-255) in double arithmetic
template <typename R, bool S, bool ADJ>
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
      const int k = (int)(kl % g.Nf[t]) + (S ? 1 : 0);
      kl /= g.Nf[t];
      const double a = 2.0 * (double)k * (double)x[j * g.d + t];
      p *= S ? sinpi(a) : cospi(a);
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

template <typename R> struct CtBase;
template <> struct CtBase<double> {
  static void *mal(size_t n) { return nfft_malloc(n); }
  static void fre(void *p) { nfft_free(p); }
  static NFFT_INT npow2(NFFT_INT v) { return nfft_next_power_of_2(v); }
  static const cufftType R2C = CUFFT_D2Z;
  static cufftResult exec(cufftHandle h, double *in, double2 *out) { return cufftExecD2Z(h, in, out); }
  static const int default_m = 8;
};
template <> struct CtBase<float> {
  static void *mal(size_t n) { return nfftf_malloc(n); }
  static void fre(void *p) { nfftf_free(p); }
  static NFFT_INT npow2(NFFT_INT v) { return nfftf_next_power_of_2(v); }
  static const cufftType R2C = CUFFT_R2C;
  static cufftResult exec(cufftHandle h, float *in, float2 *out) { return cufftExecR2C(h, in, out); }
  static const int default_m = 4;
};
// S = false: NFCT, S = true: NFST (nfst.c: NN(n) = n + 1, OFFSET = 1)
template <typename R, bool S> struct CtApi;
template <> struct CtApi<double, false> : CtBase<double> { typedef nfct_plan plan; };
template <> struct CtApi<float, false> : CtBase<float> { typedef nfctf_plan plan; };
template <> struct CtApi<double, true> : CtBase<double> { typedef nfst_plan plan; };
template <> struct CtApi<float, true> : CtBase<float> { typedef nfstf_plan plan; };

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

template <typename R, bool S>
CtCtx<R> *ct_ctx(const typename CtApi<R, S>::plan *p)
{
  CtCtx<R> *c = reinterpret_cast<CtCtx<R> *>(p->my_fftw_r2r_plan);
  if (!c) gb::fatal("nfct/nfst: plan has no device context (not initialised by this library)");
  return c;
}

template <typename R, bool S>
void ct_init_help(typename CtApi<R, S>::plan *ths)
{
  typedef CtApi<R, S> A;
  const int d = (int)ths->d;
  if (d < 1 || d > 3) gb::fatal("nfct/nfst: dimension %d not supported on the GPU (1..3)", d);
  ths->N_total = 1;
  ths->n_total = 1;
  for (int t = 0; t < d; ++t) {  // nfct.c:927-940
    ths->N_total *= ths->N[t] - (S ? 1 : 0);  // OFFSET
    ths->n_total *= ths->n[t];
  }
  ths->sigma = (R *)A::mal((size_t)d * sizeof(R));
  ths->b = (R *)A::mal((size_t)d * sizeof(R));
  ths->r2r_kind = (int *)A::mal((size_t)d * sizeof(int));
  for (int t = 0; t < d; ++t) {
    ths->sigma[t] = (R)(ths->n[t] + (S ? 1 : -1)) / (R)ths->N[t];  // NN(n) / N
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
    g.Nf[t] = g.N[t] - (S ? 1 : 0);
    g.n[t] = (int)ths->n[t];
    g.L[t] = 2 * (g.n[t] + (S ? 1 : -1));  // 2 NN(n)
    g.b[t] = ths->b[t];
    g.ext_total *= g.L[t];
    L[t] = g.L[t];
    if (g.n[t] < (S ? 1 : 2)) gb::fatal("nfct/nfst: transform length n[%d] = %d too small", t, g.n[t]);
  }
  // 1 / phi_hat(k) of the window with grid length L (nfct.c:780-800), double
  std::vector<double> ch;
  for (int t = 0; t < d; ++t)
    for (int k = 0; k < g.Nf[t]; ++k) {
      const double a = 2.0 * M_PI * (k + (S ? 1 : 0)) / (double)g.L[t];
      ch.push_back(1.0 / std::cyl_bessel_i(0.0, (double)g.m * std::sqrt((double)g.b[t] * g.b[t] - a * a)));
    }
  if (ths->flags & PRE_PHI_HUT) {
    ths->c_phi_inv = (R **)A::mal((size_t)d * sizeof(R *));
    size_t off = 0;
    for (int t = 0; t < d; ++t) {
      ths->c_phi_inv[t] = (R *)A::mal((size_t)g.Nf[t] * sizeof(R));
      for (int k = 0; k < g.Nf[t]; ++k) ths->c_phi_inv[t][k] = (R)ch[off + k];
      off += g.Nf[t];
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
    gb::fatal("nfct/nfst: cuFFT plan failed");
  cufftSetStream(c->fft, c->s);
  ths->my_fftw_r2r_plan = reinterpret_cast<decltype(ths->my_fftw_r2r_plan)>(c);
}

// DCT-I of the device grid in place (even extension, real FFT, real parts)
template <typename R, bool S>
void ct_dct(CtCtx<R> *c)
{
  gb::k_ct_extend<R, S><<<ctb(c->g.ext_total), 256, 0, c->s>>>(c->g, c->grid, c->ext);
  if (CtApi<R, S>::exec(c->fft, c->ext, c->spec) != CUFFT_SUCCESS) gb::fatal("nfct/nfst: cuFFT exec failed");
  gb::k_ct_extract<R, S><<<ctb(c->g.n_total), 256, 0, c->s>>>(c->g, c->spec, c->grid);
}

template <typename R, bool S>
void ct_times(typename CtApi<R, S>::plan *ths, CtCtx<R> *c)
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

template <typename R, bool S>
void ct_trafo(typename CtApi<R, S>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R, S>(ths);
  const gb::CtGeom<R> &g = c->g;
  if (!ths->x || !ths->f_hat || !ths->f) gb::fatal("nfct/nfst: x, f_hat or f not set");
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemcpyAsync(c->fhat, ths->f_hat, (size_t)g.N_total * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaEventRecord(c->ev[0], c->s));
  gb::k_ct_dpad<R, S><<<ctb(g.n_total), 256, 0, c->s>>>(g, c->fhat, c->cphi, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[1], c->s));
  ct_dct<R, S>(c);
  GB_CUDA(cudaEventRecord(c->ev[2], c->s));
  if (g.M > 0) gb::k_ct_b<R, S, false><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->f, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[3], c->s));
  GB_LAUNCHED("nfct_trafo");
  GB_CUDA(cudaMemcpyAsync(ths->f, c->f, (size_t)g.M * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
  ct_times<R, S>(ths, c);
}

template <typename R, bool S>
void ct_adjoint(typename CtApi<R, S>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R, S>(ths);
  const gb::CtGeom<R> &g = c->g;
  if (!ths->x || !ths->f_hat || !ths->f) gb::fatal("nfct/nfst: x, f_hat or f not set");
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemcpyAsync(c->f, ths->f, (size_t)g.M * sizeof(R), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaMemsetAsync(c->grid, 0, (size_t)g.n_total * sizeof(R), c->s));
  GB_CUDA(cudaEventRecord(c->ev[0], c->s));
  if (g.M > 0) gb::k_ct_b<R, S, true><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->f, c->grid);
  GB_CUDA(cudaEventRecord(c->ev[1], c->s));
  ct_dct<R, S>(c);
  GB_CUDA(cudaEventRecord(c->ev[2], c->s));
  gb::k_ct_dcrop<R, S><<<ctb(g.N_total), 256, 0, c->s>>>(g, c->grid, c->cphi, c->fhat);
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

template <typename R, bool S, bool ADJ>
void ct_direct(const typename CtApi<R, S>::plan *ths)
{
  CtCtx<R> *c = ct_ctx<R, S>(ths);
  const gb::CtGeom<R> &g = c->g;
  GB_CUDA(cudaMemcpyAsync(c->x, ths->x, (size_t)g.M * g.d * sizeof(R), cudaMemcpyHostToDevice, c->s));
  if (ADJ) {
    GB_CUDA(cudaMemcpyAsync(c->f, ths->f, (size_t)g.M * sizeof(R), cudaMemcpyHostToDevice, c->s));
    if (g.N_total > 0) gb::k_ct_direct<R, S, true><<<ctb(g.N_total), 256, 0, c->s>>>(g, c->x, c->f, c->fhat);
    GB_CUDA(cudaMemcpyAsync(ths->f_hat, c->fhat, (size_t)g.N_total * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  } else {
    GB_CUDA(cudaMemcpyAsync(c->fhat, ths->f_hat, (size_t)g.N_total * sizeof(R), cudaMemcpyHostToDevice, c->s));
    if (g.M > 0) gb::k_ct_direct<R, S, false><<<ctb(g.M), 256, 0, c->s>>>(g, c->x, c->fhat, c->f);
    GB_CUDA(cudaMemcpyAsync(ths->f, c->f, (size_t)g.M * sizeof(R), cudaMemcpyDeviceToHost, c->s));
  }
  GB_LAUNCHED("nfct_direct");
  GB_CUDA(cudaStreamSynchronize(c->s));
}

template <typename R, bool S>
const char *ct_check(typename CtApi<R, S>::plan *ths)
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

template <typename R, bool S>
void ct_finalize(typename CtApi<R, S>::plan *ths)
{
  typedef CtApi<R, S> A;
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

template <typename R, bool S>
void ct_init_guru(typename CtApi<R, S>::plan *ths, int d, int *N, int M_total, int *n, int m, unsigned flags,
                  unsigned fftw_flags)
{
  typedef CtApi<R, S> A;
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
  ct_init_help<R, S>(ths);
}

template <typename R, bool S>
void ct_init(typename CtApi<R, S>::plan *ths, int d, int *N, int M_total)
{
  // nfct.c:1014-1051: n = 2 (next_power_of_2(N) - 1), default m, default flags
  std::vector<int> n(d);
  for (int t = 0; t < d; ++t) n[t] = (int)(2 * (CtApi<R, S>::npow2(N[t]) - 1)) + (S ? 1 : 0);
  const unsigned flags = PRE_PHI_HUT | PRE_PSI | MALLOC_X | MALLOC_F_HAT | MALLOC_F | FFTW_INIT |
                         (d > 1 ? NFFT_SORT_NODES : FFT_OUT_OF_PLACE);
  ct_init_guru<R, S>(ths, d, N, M_total, n.data(), CtApi<R, S>::default_m, flags, FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
}

}  // namespace

#define GB_NFCT_API(P, R, S)                                                                                  \
  extern "C" {                                                                                             \
  void P##init_guru(P##plan *ths, int d, int *N, int M_total, int *n, int m, unsigned flags,              \
                    unsigned fftw_flags)                                                                   \
  {                                                                                                        \
    ct_init_guru<R, S>(ths, d, N, M_total, n, m, flags, fftw_flags);                                          \
    ths->mv_trafo = (void (*)(void *))P##trafo;                                                            \
    ths->mv_adjoint = (void (*)(void *))P##adjoint;                                                        \
  }                                                                                                        \
  void P##init(P##plan *ths, int d, int *N, int M_total)                                                   \
  {                                                                                                        \
    ct_init<R, S>(ths, d, N, M_total);                                                                        \
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
  void P##precompute_one_psi(P##plan *ths) { (void)ct_ctx<R, S>(ths); }                                       \
  void P##precompute_psi(P##plan *ths) { (void)ct_ctx<R, S>(ths); }                                           \
  void P##precompute_full_psi(P##plan *ths) { (void)ct_ctx<R, S>(ths); }                                      \
  void P##precompute_fg_psi(P##plan *ths) { (void)ct_ctx<R, S>(ths); }                                        \
  void P##precompute_lin_psi(P##plan *ths) { (void)ct_ctx<R, S>(ths); }                                       \
  void P##trafo(P##plan *ths) { ct_trafo<R, S>(ths); }                                                        \
  void P##adjoint(P##plan *ths) { ct_adjoint<R, S>(ths); }                                                    \
  void P##trafo_direct(const P##plan *ths) { ct_direct<R, S, false>(ths); }                                   \
  void P##adjoint_direct(const P##plan *ths) { ct_direct<R, S, true>(ths); }                                  \
  const char *P##check(P##plan *ths) { return ct_check<R, S>(ths); }                                          \
  void P##finalize(P##plan *ths) { ct_finalize<R, S>(ths); }                                                  \
  }

GB_NFCT_API(nfct_, double, false)
GB_NFCT_API(nfctf_, float, false)
GB_NFCT_API(nfst_, double, true)
GB_NFCT_API(nfstf_, float, true)
