// gb_dstage.cu -- the roll-off correction D fused into the zero-pad (trafo)
// and D^T fused into the crop (adjoint), with FP64 Kaiser-Bessel Fourier
// coefficients.
//
// Reference: trafo_2d D part (nfft.c:3833-3897), trafo_3d (nfft.c:5415-5513),
// generic D_openmp_A / D_openmp_T (nfft.c:440-613), precompute_phi_hut
// (nfft.c:5754-5770), PHI_HUT (include/infft.h:208).
//
// Frequency k_t in [-N_t/2, N_t/2) sits at FFT-order grid position
// k_t mod n_t; every other grid point of the trafo input is zero.  The pad
// zeroes the grid with a memset and scatters the N_total scaled
// coefficients, one thread per frequency (reads and writes coalesced along
// the last dimension); the crop gathers them back.
#include "gb_internal.h"

namespace gb {

// c_phi_inv[t][k + N_t/2] = 1 / I0(m sqrt(b_t^2 - (2 pi k / n_t)^2)), in FP64
// whatever the plan precision.  cyl_bessel_i0 is CUDA's double-precision I0.
template <typename R>
__global__ void k_cphi(Geom<R> g, double *__restrict__ cphi)
{
  int off = 0;
  for (int t = 0; t < g.d; ++t) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.N[t]; k += gridDim.x * blockDim.x) {
      // the window's own shape parameter (in plan precision) keeps D and B consistent
      const double b = (double)g.b[t];
      const double a = 2.0 * 3.14159265358979323846 * (double)(k - g.N[t] / 2) / (double)g.n[t];
      const double arg = (double)g.m * sqrt(b * b - a * a);
      cphi[off + k] = 1.0 / cyl_bessel_i0(arg);
    }
    off += g.N[t];
  }
}

template <typename R>
void launch_cphi(const Geom<R> &g, double *cphi, cudaStream_t s)
{
  k_cphi<R><<<16, 256, 0, s>>>(g, cphi);
  GB_LAUNCHED("cphi");
}

// In single precision the FP64 coefficient product is rounded once to float
// and applied in float.
template <typename R>
__device__ __forceinline__ typename Cx<R>::T d_scale(typename Cx<R>::T v, double c);
template <>
__device__ __forceinline__ float2 d_scale<float>(float2 v, double c)
{
  const float cf = (float)c;
  return make_float2(v.x * cf, v.y * cf);
}
template <>
__device__ __forceinline__ double2 d_scale<double>(double2 v, double c)
{
  return make_double2(v.x * c, v.y * c);
}

// FFT-order grid index of natural frequency index k (row-major over N) and
// the FP64 coefficient product, formed in the order the row-wise form used:
// dims d-2 .. 0 from 1.0, then the last dimension.
template <typename R>
__device__ __forceinline__ long long d_point(long long k, const Geom<R> &g, const double *__restrict__ cphi,
                                             double &c)
{
  int kk[GB_MAXD];
  if (g.N_total <= 0xffffffffLL) {  // 32-bit division where the index fits
    unsigned r = (unsigned)k;
    for (int t = g.d - 1; t >= 0; --t) {
      const unsigned q = r / (unsigned)g.N[t];
      kk[t] = (int)(r - q * (unsigned)g.N[t]);
      r = q;
    }
  } else {
    for (int t = g.d - 1; t >= 0; --t) {
      const long long q = k / g.N[t];
      kk[t] = (int)(k - q * g.N[t]);
      k = q;
    }
  }
  int off = 0;
  for (int t = 0; t < g.d - 1; ++t) off += g.N[t];
  const int offl = off;
  c = 1.0;
  for (int t = g.d - 2; t >= 0; --t) {
    off -= g.N[t];
    c *= cphi[off + kk[t]];
  }
  c = c * cphi[offl + kk[g.d - 1]];
  long long gi = 0;
  for (int t = 0; t < g.d; ++t) {
    const int f = kk[t] - g.N[t] / 2;
    gi = gi * g.n[t] + (f < 0 ? f + g.n[t] : f);
  }
  return gi;
}

// Trafo: g = f_hat(k) prod_t c_t inside the frequency box (the grid is
// zeroed before by a memset); one thread per frequency.
template <typename R>
__global__ void __launch_bounds__(256) k_d_pad(const typename Cx<R>::T *__restrict__ fhat,
                                               const double *__restrict__ cphi,
                                               typename Cx<R>::T *__restrict__ grid, Geom<R> g)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < g.N_total;
       k += (long long)gridDim.x * blockDim.x) {
    double c;
    const long long gi = d_point<R>(k, g, cphi, c);
    grid[gi] = d_scale<R>(fhat[k], c);
  }
}

// Adjoint: f_hat(k) = g(k mod n) prod_t c_t; one thread per frequency.
template <typename R>
__global__ void __launch_bounds__(256) k_d_crop(const typename Cx<R>::T *__restrict__ grid,
                                                const double *__restrict__ cphi,
                                                typename Cx<R>::T *__restrict__ fhat, Geom<R> g)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < g.N_total;
       k += (long long)gridDim.x * blockDim.x) {
    double c;
    const long long gi = d_point<R>(k, g, cphi, c);
    fhat[k] = d_scale<R>(grid[gi], c);
  }
}

static unsigned d_blocks(long long n)
{
  const long long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

template <typename R>
void launch_d_pad(const typename Cx<R>::T *fhat, const double *cphi, typename Cx<R>::T *grid,
                  const Geom<R> &g, cudaStream_t s)
{
  GB_CUDA(cudaMemsetAsync(grid, 0, (size_t)g.n_total * sizeof(typename Cx<R>::T), s));
  k_d_pad<R><<<d_blocks(g.N_total), 256, 0, s>>>(fhat, cphi, grid, g);
  GB_LAUNCHED("d_pad");
}

template <typename R>
void launch_d_crop(const typename Cx<R>::T *grid, const double *cphi, typename Cx<R>::T *fhat,
                   const Geom<R> &g, cudaStream_t s)
{
  k_d_crop<R><<<d_blocks(g.N_total), 256, 0, s>>>(grid, cphi, fhat, g);
  GB_LAUNCHED("d_crop");
}

template void launch_cphi<float>(const Geom<float> &, double *, cudaStream_t);
template void launch_cphi<double>(const Geom<double> &, double *, cudaStream_t);
template void launch_d_pad<float>(const float2 *, const double *, float2 *, const Geom<float> &,
                                  cudaStream_t);
template void launch_d_pad<double>(const double2 *, const double *, double2 *,
                                   const Geom<double> &, cudaStream_t);
template void launch_d_crop<float>(const float2 *, const double *, float2 *, const Geom<float> &,
                                   cudaStream_t);
template void launch_d_crop<double>(const double2 *, const double *, double2 *,
                                    const Geom<double> &, cudaStream_t);

}  // namespace gb
