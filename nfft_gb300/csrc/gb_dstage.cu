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
// kernel writes the whole n_total grid in one coalesced pass, so no separate
// memset of the grid is needed.
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

// One thread per grid cell, last dimension fastest: g = f_hat(k) prod_t c_t
// inside the frequency box, zero elsewhere.
template <typename R>
__global__ void k_d_pad(const typename Cx<R>::T *__restrict__ fhat, const double *__restrict__ cphi,
                        typename Cx<R>::T *__restrict__ grid, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= g.n_total) return;
  long long rem = cell;
  long long fidx = 0;
  double c = 1.0;
  bool inside = true;
  int off = 0;
  int pos[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    pos[t] = (int)(rem % g.n[t]);
    rem /= g.n[t];
  }
  for (int t = 0; t < g.d; ++t) {
    const int i = pos[t];
    const int k = (i < g.n[t] / 2) ? i : i - g.n[t];  // frequency at this grid point
    const int kk = k + g.N[t] / 2;                     // natural-order index
    if (kk < 0 || kk >= g.N[t]) inside = false;
    else c *= cphi[off + kk];
    fidx = fidx * g.N[t] + kk;
    off += g.N[t];
  }
  C out = cmake(R(0), R(0));
  if (inside) {
    const C v = fhat[fidx];
    out = cmake((R)((double)v.x * c), (R)((double)v.y * c));
  }
  grid[cell] = out;
}

template <typename R>
__global__ void k_d_crop(const typename Cx<R>::T *__restrict__ grid, const double *__restrict__ cphi,
                         typename Cx<R>::T *__restrict__ fhat, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const long long kl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kl >= g.N_total) return;
  long long rem = kl, gidx = 0;
  double c = 1.0;
  int kk[GB_MAXD];
  for (int t = g.d - 1; t >= 0; --t) {
    kk[t] = (int)(rem % g.N[t]);
    rem /= g.N[t];
  }
  int off = 0;
  for (int t = 0; t < g.d; ++t) {
    const int k = kk[t] - g.N[t] / 2;
    const int i = k < 0 ? k + g.n[t] : k;
    gidx = gidx * g.n[t] + i;
    c *= cphi[off + kk[t]];
    off += g.N[t];
  }
  const C v = grid[gidx];
  fhat[kl] = cmake((R)((double)v.x * c), (R)((double)v.y * c));
}

template <typename R>
void launch_d_pad(const typename Cx<R>::T *fhat, const double *cphi, typename Cx<R>::T *grid,
                  const Geom<R> &g, cudaStream_t s)
{
  const int th = 256;
  k_d_pad<R><<<(unsigned)((g.n_total + th - 1) / th), th, 0, s>>>(fhat, cphi, grid, g);
  GB_LAUNCHED("d_pad");
}

template <typename R>
void launch_d_crop(const typename Cx<R>::T *grid, const double *cphi, typename Cx<R>::T *fhat,
                   const Geom<R> &g, cudaStream_t s)
{
  const int th = 256;
  k_d_crop<R><<<(unsigned)((g.N_total + th - 1) / th), th, 0, s>>>(grid, cphi, fhat, g);
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
