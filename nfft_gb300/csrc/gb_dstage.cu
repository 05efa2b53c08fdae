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

// Row-wise D and D^T.  A block owns (part of) one grid row along the last
// dimension: the row's position in the other dimensions, whether it meets
// the frequency box and the product of their FP64 coefficients are computed
// once per block with 32-bit index arithmetic; threads then stride along the
// row with coalesced loads and stores.  In single precision the FP64
// coefficient product is rounded once to float and applied in float.
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

// Natural-order index kk of grid position i (FFT order) along a dimension of
// length n with bandwidth N, or -1 outside the frequency box.
__device__ __forceinline__ int d_natural(int i, int n, int N)
{
  const int k = (i < n / 2) ? i : i - n;
  const int kk = k + N / 2;
  return (kk >= 0 && kk < N) ? kk : -1;
}

// Grid row r (over dims 0..d-2 of n) -> whether it meets the frequency box,
// the natural-order row of f_hat it holds and the FP64 coefficient product.
template <typename R>
__device__ __forceinline__ bool d_pad_row(unsigned r, const Geom<R> &g, const double *cphi, long long &frow,
                                          double &c)
{
  bool inside = true;
  long long fmul = 1;
  int off = 0;
  for (int t = 0; t < g.d - 1; ++t) off += g.N[t];
  frow = 0;
  c = 1.0;
  for (int t = g.d - 2; t >= 0; --t) {
    const unsigned nt = (unsigned)g.n[t];
    const unsigned q = r / nt;
    const int i = (int)(r - q * nt);
    r = q;
    off -= g.N[t];
    const int kk = d_natural(i, g.n[t], g.N[t]);
    if (kk < 0) inside = false;
    else c *= cphi[off + kk];
    frow += fmul * kk;
    fmul *= g.N[t];
  }
  return inside;
}

// Row r of f_hat (over dims 0..d-2 of N) -> the grid row holding it and the
// FP64 coefficient product.
template <typename R>
__device__ __forceinline__ long long d_crop_row(unsigned r, const Geom<R> &g, const double *cphi, double &c)
{
  long long grow = 0, gmul = 1;
  int off = 0;
  for (int t = 0; t < g.d - 1; ++t) off += g.N[t];
  c = 1.0;
  for (int t = g.d - 2; t >= 0; --t) {
    const unsigned Nt = (unsigned)g.N[t];
    const unsigned q = r / Nt;
    const int kk = (int)(r - q * Nt);
    r = q;
    off -= g.N[t];
    const int k = kk - g.N[t] / 2;
    c *= cphi[off + kk];
    grow += gmul * (k < 0 ? k + g.n[t] : k);
    gmul *= g.n[t];
  }
  return grow;
}

// Trafo: g = f_hat(k) prod_t c_t inside the frequency box, zero elsewhere;
// writes the whole n_total grid (no separate memset).  Blocks stride over
// the grid rows.
template <typename R>
__global__ void __launch_bounds__(256) k_d_pad(const typename Cx<R>::T *__restrict__ fhat,
                                               const double *__restrict__ cphi,
                                               typename Cx<R>::T *__restrict__ grid, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const int nl = g.n[g.d - 1], Nl = g.N[g.d - 1];
  const double *cl = cphi;
  for (int t = 0; t < g.d - 1; ++t) cl += g.N[t];
  const unsigned rows = (unsigned)(g.n_total / nl);
  for (unsigned r = blockIdx.x; r < rows; r += gridDim.x) {
    long long frow;
    double c;
    const bool inside = d_pad_row<R>(r, g, cphi, frow, c);
    C *row = grid + (long long)r * nl;
    const C *src = fhat + frow * Nl;
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < nl; i += gridDim.y * blockDim.x) {
      C out = cmake(R(0), R(0));
      const int kk = d_natural(i, nl, Nl);
      if (inside && kk >= 0) out = d_scale<R>(src[kk], c * cl[kk]);
      row[i] = out;
    }
  }
}

// Adjoint: f_hat(k) = g(k mod n) prod_t c_t.  Blocks stride over the rows
// of f_hat.
template <typename R>
__global__ void __launch_bounds__(256) k_d_crop(const typename Cx<R>::T *__restrict__ grid,
                                                const double *__restrict__ cphi,
                                                typename Cx<R>::T *__restrict__ fhat, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const int nl = g.n[g.d - 1], Nl = g.N[g.d - 1];
  const double *cl = cphi;
  for (int t = 0; t < g.d - 1; ++t) cl += g.N[t];
  const unsigned rows = (unsigned)(g.N_total / Nl);
  for (unsigned r = blockIdx.x; r < rows; r += gridDim.x) {
    double c;
    const C *src = grid + d_crop_row<R>(r, g, cphi, c) * nl;
    C *out = fhat + (long long)r * Nl;
    for (int kk = blockIdx.y * blockDim.x + threadIdx.x; kk < Nl; kk += gridDim.y * blockDim.x) {
      const int k = kk - Nl / 2;
      out[kk] = d_scale<R>(src[k < 0 ? k + nl : k], c * cl[kk]);
    }
  }
}

// blocks stride over rows (at most 16 resident blocks' worth per SM)
static dim3 d_rows_grid(long long rows, int len, int th)
{
  const long long chunks = (len + th - 1) / th;
  const long long bx = rows < 152 * 16 ? rows : 152 * 16;
  return dim3((unsigned)bx, (unsigned)(chunks < 65535 ? chunks : 65535), 1);
}

template <typename R>
void launch_d_pad(const typename Cx<R>::T *fhat, const double *cphi, typename Cx<R>::T *grid,
                  const Geom<R> &g, cudaStream_t s)
{
  const int th = 256;
  const int nl = g.n[g.d - 1];
  k_d_pad<R><<<d_rows_grid(g.n_total / nl, nl, th), th, 0, s>>>(fhat, cphi, grid, g);
  GB_LAUNCHED("d_pad");
}

template <typename R>
void launch_d_crop(const typename Cx<R>::T *grid, const double *cphi, typename Cx<R>::T *fhat,
                   const Geom<R> &g, cudaStream_t s)
{
  const int th = 256;
  const int Nl = g.N[g.d - 1];
  k_d_crop<R><<<d_rows_grid(g.N_total / Nl, Nl, th), th, 0, s>>>(grid, cphi, fhat, g);
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
