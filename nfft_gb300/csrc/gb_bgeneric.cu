// gb_bgeneric.cu -- global-memory B / B^T for any dimension and cut-off, and
// the NDFT (direct transforms).
//
// Reference: generic B_openmp_A (nfft.c:1172-1278) and B_openmp_T
// (nfft.c:1974-2098) for d >= 4; nfft_trafo_direct (nfft.c:145-205) and
// nfft_adjoint_direct (nfft.c:207-297).
//
// The generic kernels run one thread per node in tile order, gather the
// (2m+2)^d taps straight from the grid (L1/L2-cached) and scatter with
// global atomics.  They cover the (d, m) pairs without a tiled kernel.
#include "gb_internal.h"

namespace gb {

template <typename R>
__global__ void __launch_bounds__(128) k_b_generic(const typename Cx<R>::T *__restrict__ grid,
                                                   const R *__restrict__ xs,
                                                   const uint32_t *__restrict__ perm,
                                                   typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.M) return;
  R psi[GB_MAXD * GB_MAXW];
  int u[GB_MAXD], l[GB_MAXD];
  const int d = g.d, w = g.w;
  for (int t = 0; t < d; ++t) {
    const R x = xs[i * d + t];
    u[t] = node_u<R>(x, g.nR[t], g.m);
    node_psi_rt<R>(x, u[t], w, g.nR[t], g.mm, g.b[t], psi + t * w);
    l[t] = 0;
  }
  R ar = 0, ai = 0;
  for (;;) {
    long long pos = 0;
    R wgt = 1;
    for (int t = 0; t < d; ++t) {
      pos = pos * g.n[t] + wrap(u[t] + l[t], g.n[t]);
      wgt *= psi[t * w + l[t]];
    }
    const C v = grid[pos];
    ar += wgt * v.x;
    ai += wgt * v.y;
    int t = d - 1;
    for (; t >= 0; --t) {
      if (++l[t] < w) break;
      l[t] = 0;
    }
    if (t < 0) break;
  }
  f[perm[i]] = cmake(ar, ai);
}

template <typename R>
__global__ void __launch_bounds__(128) k_bt_generic(typename Cx<R>::T *__restrict__ grid,
                                                    const R *__restrict__ xs,
                                                    const uint32_t *__restrict__ perm,
                                                    const typename Cx<R>::T *__restrict__ f,
                                                    Geom<R> g)
{
  typedef typename Cx<R>::T C;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.M) return;
  R psi[GB_MAXD * GB_MAXW];
  int u[GB_MAXD], l[GB_MAXD];
  const int d = g.d, w = g.w;
  for (int t = 0; t < d; ++t) {
    const R x = xs[i * d + t];
    u[t] = node_u<R>(x, g.nR[t], g.m);
    node_psi_rt<R>(x, u[t], w, g.nR[t], g.mm, g.b[t], psi + t * w);
    l[t] = 0;
  }
  const C fj = f[perm[i]];
  for (;;) {
    long long pos = 0;
    R wgt = 1;
    for (int t = 0; t < d; ++t) {
      pos = pos * g.n[t] + wrap(u[t] + l[t], g.n[t]);
      wgt *= psi[t * w + l[t]];
    }
    global_add_c(grid + pos, cmake(wgt * fj.x, wgt * fj.y));
    int t = d - 1;
    for (; t >= 0; --t) {
      if (++l[t] < w) break;
      l[t] = 0;
    }
    if (t < 0) break;
  }
}

template <typename R>
void launch_b_generic(const typename Cx<R>::T *grid, const R *xs, const uint32_t *perm,
                      typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)
{
  if (g.M == 0) return;
  const int th = 128;
  k_b_generic<R><<<(unsigned)((g.M + th - 1) / th), th, 0, s>>>(grid, xs, perm, f, g);
  GB_LAUNCHED("b_generic");
}

template <typename R>
void launch_bt_generic(typename Cx<R>::T *grid, const R *xs, const uint32_t *perm,
                       const typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)
{
  if (g.M == 0) return;
  const int th = 128;
  k_bt_generic<R><<<(unsigned)((g.M + th - 1) / th), th, 0, s>>>(grid, xs, perm, f, g);
  GB_LAUNCHED("bt_generic");
}

// ---------------------------------------------------------------- NDFT
// f_j = sum_k f^_k exp(-2 pi i k.x_j) over k_t in [-N_t/2, N_t/2), k in
// natural row-major order (reference nfft.c:145-205).  The phase k.x is
// formed in FP64 and evaluated with sincospi for both precisions.
static constexpr int NDFT_TILE = 256;

template <typename R>
__global__ void __launch_bounds__(NDFT_TILE) k_ndft_trafo(const R *__restrict__ x,
                                                         const typename Cx<R>::T *__restrict__ fhat,
                                                         typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  __shared__ double2 sf[NDFT_TILE];
  __shared__ int sk[NDFT_TILE][GB_MAXD];
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = j < g.M;
  double xj[GB_MAXD];
  for (int t = 0; t < g.d; ++t) xj[t] = valid ? (double)x[j * g.d + t] : 0.0;
  double sr = 0.0, si = 0.0;
  for (long long k0 = 0; k0 < g.N_total; k0 += NDFT_TILE) {
    __syncthreads();
    const long long kl = k0 + threadIdx.x;
    if (kl < g.N_total) {
      const C v = fhat[kl];
      sf[threadIdx.x] = make_double2((double)v.x, (double)v.y);
      long long rem = kl;
      for (int t = g.d - 1; t >= 0; --t) {
        sk[threadIdx.x][t] = (int)(rem % g.N[t]) - g.N[t] / 2;
        rem /= g.N[t];
      }
    }
    __syncthreads();
    const int cnt = (int)min((long long)NDFT_TILE, g.N_total - k0);
    for (int q = 0; q < cnt; ++q) {
      double ph = 0.0;
      for (int t = 0; t < g.d; ++t) ph += (double)sk[q][t] * xj[t];
      ph -= rint(ph);
      double sn, cs;
      sincospi(-2.0 * ph, &sn, &cs);
      const double2 v = sf[q];
      sr += v.x * cs - v.y * sn;
      si += v.x * sn + v.y * cs;
    }
  }
  if (valid) f[j] = cmake((R)sr, (R)si);
}

// f^_k = sum_j f_j exp(+2 pi i k.x_j) (reference nfft.c:207-297)
template <typename R>
__global__ void __launch_bounds__(NDFT_TILE) k_ndft_adjoint(const R *__restrict__ x,
                                                           const typename Cx<R>::T *__restrict__ f,
                                                           typename Cx<R>::T *__restrict__ fhat,
                                                           Geom<R> g)
{
  typedef typename Cx<R>::T C;
  __shared__ double2 sf[NDFT_TILE];
  __shared__ double sx[NDFT_TILE][GB_MAXD];
  const long long kl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = kl < g.N_total;
  int k[GB_MAXD];
  {
    long long rem = valid ? kl : 0;
    for (int t = g.d - 1; t >= 0; --t) {
      k[t] = (int)(rem % g.N[t]) - g.N[t] / 2;
      rem /= g.N[t];
    }
  }
  double sr = 0.0, si = 0.0;
  for (long long j0 = 0; j0 < g.M; j0 += NDFT_TILE) {
    __syncthreads();
    const long long j = j0 + threadIdx.x;
    if (j < g.M) {
      const C v = f[j];
      sf[threadIdx.x] = make_double2((double)v.x, (double)v.y);
      for (int t = 0; t < g.d; ++t) sx[threadIdx.x][t] = (double)x[j * g.d + t];
    }
    __syncthreads();
    const int cnt = (int)min((long long)NDFT_TILE, g.M - j0);
    for (int q = 0; q < cnt; ++q) {
      double ph = 0.0;
      for (int t = 0; t < g.d; ++t) ph += (double)k[t] * sx[q][t];
      ph -= rint(ph);
      double sn, cs;
      sincospi(2.0 * ph, &sn, &cs);
      const double2 v = sf[q];
      sr += v.x * cs - v.y * sn;
      si += v.x * sn + v.y * cs;
    }
  }
  if (valid) fhat[kl] = cmake((R)sr, (R)si);
}

template <typename R>
void launch_ndft_trafo(const R *x, const typename Cx<R>::T *fhat, typename Cx<R>::T *f,
                       const Geom<R> &g, cudaStream_t s)
{
  if (g.M == 0) return;
  k_ndft_trafo<R><<<(unsigned)((g.M + NDFT_TILE - 1) / NDFT_TILE), NDFT_TILE, 0, s>>>(x, fhat, f, g);
  GB_LAUNCHED("ndft_trafo");
}

template <typename R>
void launch_ndft_adjoint(const R *x, const typename Cx<R>::T *f, typename Cx<R>::T *fhat,
                         const Geom<R> &g, cudaStream_t s)
{
  if (g.N_total == 0) return;
  k_ndft_adjoint<R><<<(unsigned)((g.N_total + NDFT_TILE - 1) / NDFT_TILE), NDFT_TILE, 0, s>>>(
      x, f, fhat, g);
  GB_LAUNCHED("ndft_adjoint");
}

#define GB_INST(R)                                                                                \
  template void launch_b_generic<R>(const Cx<R>::T *, const R *, const uint32_t *, Cx<R>::T *,     \
                                    const Geom<R> &, cudaStream_t);                                \
  template void launch_bt_generic<R>(Cx<R>::T *, const R *, const uint32_t *, const Cx<R>::T *,    \
                                     const Geom<R> &, cudaStream_t);                               \
  template void launch_ndft_trafo<R>(const R *, const Cx<R>::T *, Cx<R>::T *, const Geom<R> &,     \
                                     cudaStream_t);                                                \
  template void launch_ndft_adjoint<R>(const R *, const Cx<R>::T *, Cx<R>::T *, const Geom<R> &,   \
                                       cudaStream_t);
GB_INST(float)
GB_INST(double)

}  // namespace gb
