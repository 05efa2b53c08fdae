// gb_btiled.cuh -- shared-memory tiled B (interpolation) and B^T (spreading).
//
// Reference: nfft_trafo_{1,2,3}d_B (nfft.c:2283-2445, 3221-3410, 4687-4914)
// with their per-node tensor-product gathers (nfft_trafo_2d_compute
// nfft.c:2927-3004, 3-D nfft.c:4020-4265), and nfft_adjoint_{1,2,3}d_B
// (nfft.c:2585-2773, 3583-3805, 5126-5384) with the blockwise scatter
// (nfft.c:1345-1420, 3064-3139).
//
// GB300 design: nodes are binned by the tile of the oversampled grid that
// holds their wrapped window start.  A CTA takes one work item (a tile and
// a range of its sorted nodes), stages the tile's padded subgrid
// (T_t + 2m + 1 cells per dimension, wrapped periodically) in shared memory,
// and evaluates the Kaiser-Bessel window on the fly (d * (2m+2) values per
// node instead of the reference's PRE_PSI table).
//  * B:   subgrid loaded once per item, each thread gathers its nodes'
//         (2m+2)^d taps from shared memory; results scattered to f[perm].
//  * B^T: each thread accumulates its nodes' taps into the shared subgrid
//         with shared-memory atomics; the subgrid is then added to the
//         global grid once per item (one vector reduction per cell), never
//         per node.
#pragma once

#include "gb_internal.h"

namespace gb {

template <typename R, int D>
__device__ __forceinline__ void tile_origin(const WorkItem &it, const Geom<R> &g, int *org)
{
  int rem = it.tile;
#pragma unroll
  for (int t = D - 1; t >= 0; --t) {
    const int tc = rem % g.ntile[t];
    rem /= g.ntile[t];
    org[t] = tc * g.T[t];
  }
}

template <int D>
__device__ __forceinline__ int sub_cells(const int *ext)
{
  int c = 1;
#pragma unroll
  for (int t = 0; t < D; ++t) c *= ext[t];
  return c;
}

// global index of subgrid cell `idx` (row-major over ext, wrapped mod n)
template <typename R, int D>
__device__ __forceinline__ long long sub_to_global(int idx, const int *org, const Geom<R> &g)
{
  int c[D];
#pragma unroll
  for (int t = D - 1; t >= 0; --t) {
    c[t] = idx % g.ext[t];
    idx /= g.ext[t];
  }
  long long gi = 0;
#pragma unroll
  for (int t = 0; t < D; ++t) {
    int p = org[t] + c[t];
    while (p >= g.n[t]) p -= g.n[t];  // a padded tile can wrap more than once on small grids
    gi = gi * g.n[t] + p;
  }
  return gi;
}

template <typename R, int D, int W>
__global__ void __launch_bounds__(256) k_b_tiled(const WorkItem *__restrict__ items,
                                                 const typename Cx<R>::T *__restrict__ grid,
                                                 const R *__restrict__ xs,
                                                 const uint32_t *__restrict__ perm,
                                                 typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *sg = reinterpret_cast<C *>(smem_raw);
  const WorkItem it = items[blockIdx.x];
  int org[D];
  tile_origin<R, D>(it, g, org);
  const int cells = sub_cells<D>(g.ext);
  for (int idx = threadIdx.x; idx < cells; idx += blockDim.x)
    sg[idx] = grid[sub_to_global<R, D>(idx, org, g)];
  __syncthreads();

  for (int i = it.start + threadIdx.x; i < it.end; i += blockDim.x) {
    R psi[D][W];
    int loc[D];
#pragma unroll
    for (int t = 0; t < D; ++t) {
      const R x = xs[(long long)i * D + t];
      const int u = node_u<R>(x, g.nR[t], g.m);
      loc[t] = wrap(u, g.n[t]) - org[t];
      node_psi<R, W>(x, u, g.nR[t], g.mm, g.b[t], psi[t]);
    }
    R ar = 0, ai = 0;
    if (D == 1) {
#pragma unroll
      for (int l = 0; l < W; ++l) {
        const C v = sg[loc[0] + l];
        ar += psi[0][l] * v.x;
        ai += psi[0][l] * v.y;
      }
    } else if (D == 2) {
#pragma unroll 2
      for (int l0 = 0; l0 < W; ++l0) {
        const C *row = sg + (loc[0] + l0) * g.ext[1] + loc[1];
        R rr = 0, ri = 0;
#pragma unroll
        for (int l1 = 0; l1 < W; ++l1) {
          const C v = row[l1];
          rr += psi[1][l1] * v.x;
          ri += psi[1][l1] * v.y;
        }
        ar += psi[0][l0] * rr;
        ai += psi[0][l0] * ri;
      }
    } else {
      const int e1 = g.ext[1], e2 = g.ext[2];
      for (int l0 = 0; l0 < W; ++l0) {
        R pr = 0, pi_ = 0;
#pragma unroll 2
        for (int l1 = 0; l1 < W; ++l1) {
          const C *row = sg + ((loc[0] + l0) * e1 + (loc[1] + l1)) * e2 + loc[2];
          R rr = 0, ri = 0;
#pragma unroll
          for (int l2 = 0; l2 < W; ++l2) {
            const C v = row[l2];
            rr += psi[2][l2] * v.x;
            ri += psi[2][l2] * v.y;
          }
          pr += psi[1][l1] * rr;
          pi_ += psi[1][l1] * ri;
        }
        ar += psi[0][l0] * pr;
        ai += psi[0][l0] * pi_;
      }
    }
    f[perm[i]] = cmake(ar, ai);
  }
}

template <typename R, int D, int W>
__global__ void __launch_bounds__(256) k_bt_tiled(const WorkItem *__restrict__ items,
                                                  typename Cx<R>::T *__restrict__ grid,
                                                  const R *__restrict__ xs,
                                                  const uint32_t *__restrict__ perm,
                                                  const typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *sg = reinterpret_cast<C *>(smem_raw);
  const WorkItem it = items[blockIdx.x];
  int org[D];
  tile_origin<R, D>(it, g, org);
  const int cells = sub_cells<D>(g.ext);
  for (int idx = threadIdx.x; idx < cells; idx += blockDim.x) sg[idx] = cmake(R(0), R(0));
  __syncthreads();

  for (int i = it.start + threadIdx.x; i < it.end; i += blockDim.x) {
    R psi[D][W];
    int loc[D];
#pragma unroll
    for (int t = 0; t < D; ++t) {
      const R x = xs[(long long)i * D + t];
      const int u = node_u<R>(x, g.nR[t], g.m);
      loc[t] = wrap(u, g.n[t]) - org[t];
      node_psi<R, W>(x, u, g.nR[t], g.mm, g.b[t], psi[t]);
    }
    const C fj = f[perm[i]];
    if (D == 1) {
#pragma unroll
      for (int l = 0; l < W; ++l) {
        C *c = sg + loc[0] + l;
        atomicAdd(&c->x, psi[0][l] * fj.x);
        atomicAdd(&c->y, psi[0][l] * fj.y);
      }
    } else if (D == 2) {
      for (int l0 = 0; l0 < W; ++l0) {
        C *row = sg + (loc[0] + l0) * g.ext[1] + loc[1];
        const R wr = psi[0][l0] * fj.x, wi = psi[0][l0] * fj.y;
#pragma unroll
        for (int l1 = 0; l1 < W; ++l1) {
          atomicAdd(&row[l1].x, psi[1][l1] * wr);
          atomicAdd(&row[l1].y, psi[1][l1] * wi);
        }
      }
    } else {
      const int e1 = g.ext[1], e2 = g.ext[2];
      for (int l0 = 0; l0 < W; ++l0) {
        for (int l1 = 0; l1 < W; ++l1) {
          C *row = sg + ((loc[0] + l0) * e1 + (loc[1] + l1)) * e2 + loc[2];
          const R p01 = psi[0][l0] * psi[1][l1];
          const R wr = p01 * fj.x, wi = p01 * fj.y;
#pragma unroll
          for (int l2 = 0; l2 < W; ++l2) {
            atomicAdd(&row[l2].x, psi[2][l2] * wr);
            atomicAdd(&row[l2].y, psi[2][l2] * wi);
          }
        }
      }
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < cells; idx += blockDim.x) {
    const C v = sg[idx];
    if (v.x != R(0) || v.y != R(0)) global_add_c(grid + sub_to_global<R, D>(idx, org, g), v);
  }
}

}  // namespace gb

namespace gb {

// Window widths w = 2m+2 with a tiled kernel (m = 2..8); other m use the
// generic global-memory kernels.
#define GB_TILED_WIDTHS(X, D) X(D, 6) X(D, 8) X(D, 10) X(D, 12) X(D, 14) X(D, 16) X(D, 18)

template <typename R>
size_t tiled_smem_bytes_impl(const Geom<R> &g)
{
  size_t c = 1;
  for (int t = 0; t < g.d; ++t) c *= (size_t)g.ext[t];
  return c * sizeof(typename Cx<R>::T);
}

template <typename R, int D, int W>
static void run_b(const WorkItem *items, int nitems, const typename Cx<R>::T *grid, const R *xs,
                  const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)
{
  const size_t smem = tiled_smem_bytes_impl(g);
  set_smem_limit((const void *)k_b_tiled<R, D, W>, smem);
  k_b_tiled<R, D, W><<<nitems, 256, smem, s>>>(items, grid, xs, perm, f, g);
  GB_LAUNCHED("b_tiled");
}

template <typename R, int D, int W>
static void run_bt(const WorkItem *items, int nitems, typename Cx<R>::T *grid, const R *xs,
                   const uint32_t *perm, const typename Cx<R>::T *f, const Geom<R> &g,
                   cudaStream_t s)
{
  const size_t smem = tiled_smem_bytes_impl(g);
  set_smem_limit((const void *)k_bt_tiled<R, D, W>, smem);
  k_bt_tiled<R, D, W><<<nitems, 256, smem, s>>>(items, grid, xs, perm, f, g);
  GB_LAUNCHED("bt_tiled");
}

#define GB_TILED_W(X) X(6) X(8) X(10) X(12) X(14) X(16) X(18)
#define GB_CASE_OK(D, W) case D * 1000 + W:

template <typename R>
bool tiled_supported_impl(int d, int w)
{
  switch (d * 1000 + w) {
    GB_TILED_WIDTHS(GB_CASE_OK, 1)
    GB_TILED_WIDTHS(GB_CASE_OK, 2)
    GB_TILED_WIDTHS(GB_CASE_OK, 3)
    return true;
    default:
      return false;
  }
}

// One dimension's kernels, by window width (instantiated per precision and
// dimension in gb_btiled_<precision><d>.cu, which compile in parallel).
template <typename R, int D>
void launch_b_tiled_dim(const WorkItem *items, int nitems, const typename Cx<R>::T *grid, const R *xs,
                        const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)
{
  switch (g.w) {
#define GB_CASE_BW(W) \
  case W: run_b<R, D, W>(items, nitems, grid, xs, perm, f, g, s); return;
    GB_TILED_W(GB_CASE_BW)
#undef GB_CASE_BW
    default:
      fatal("no tiled interpolation kernel for d=%d w=%d", g.d, g.w);
  }
}

template <typename R, int D>
void launch_bt_tiled_dim(const WorkItem *items, int nitems, typename Cx<R>::T *grid, const R *xs,
                         const uint32_t *perm, const typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)
{
  switch (g.w) {
#define GB_CASE_BTW(W) \
  case W: run_bt<R, D, W>(items, nitems, grid, xs, perm, f, g, s); return;
    GB_TILED_W(GB_CASE_BTW)
#undef GB_CASE_BTW
    default:
      fatal("no tiled spreading kernel for d=%d w=%d", g.d, g.w);
  }
}

#define GB_TILED_DIM_DECL(EXT, R, D)                                                                        \
  EXT template void launch_b_tiled_dim<R, D>(const WorkItem *, int, const Cx<R>::T *, const R *,         \
                                             const uint32_t *, Cx<R>::T *, const Geom<R> &, cudaStream_t); \
  EXT template void launch_bt_tiled_dim<R, D>(const WorkItem *, int, Cx<R>::T *, const R *,              \
                                              const uint32_t *, const Cx<R>::T *, const Geom<R> &, cudaStream_t);
GB_TILED_DIM_DECL(extern, float, 1)
GB_TILED_DIM_DECL(extern, float, 2)
GB_TILED_DIM_DECL(extern, float, 3)
GB_TILED_DIM_DECL(extern, double, 1)
GB_TILED_DIM_DECL(extern, double, 2)
GB_TILED_DIM_DECL(extern, double, 3)

template <typename R>
void launch_b_tiled_impl(const WorkItem *items, int nitems, const typename Cx<R>::T *grid,
                         const R *xs, const uint32_t *perm, typename Cx<R>::T *f,
                         const Geom<R> &g, cudaStream_t s)
{
  if (nitems <= 0) return;
  switch (g.d) {
    case 1: launch_b_tiled_dim<R, 1>(items, nitems, grid, xs, perm, f, g, s); return;
    case 2: launch_b_tiled_dim<R, 2>(items, nitems, grid, xs, perm, f, g, s); return;
    case 3: launch_b_tiled_dim<R, 3>(items, nitems, grid, xs, perm, f, g, s); return;
    default:
      fatal("no tiled interpolation kernel for d=%d w=%d", g.d, g.w);
  }
}

template <typename R>
void launch_bt_tiled_impl(const WorkItem *items, int nitems, typename Cx<R>::T *grid,
                          const R *xs, const uint32_t *perm, const typename Cx<R>::T *f,
                          const Geom<R> &g, cudaStream_t s)
{
  if (nitems <= 0) return;
  switch (g.d) {
    case 1: launch_bt_tiled_dim<R, 1>(items, nitems, grid, xs, perm, f, g, s); return;
    case 2: launch_bt_tiled_dim<R, 2>(items, nitems, grid, xs, perm, f, g, s); return;
    case 3: launch_bt_tiled_dim<R, 3>(items, nitems, grid, xs, perm, f, g, s); return;
    default:
      fatal("no tiled spreading kernel for d=%d w=%d", g.d, g.w);
  }
}

}  // namespace gb

#define GB_INSTANTIATE_TILED(R)                                                                   \
  namespace gb {                                                                                  \
  template <> bool tiled_supported<R>(int d, int w) { return tiled_supported_impl<R>(d, w); }     \
  template <> size_t tiled_smem_bytes<R>(const Geom<R> &g) { return tiled_smem_bytes_impl<R>(g); } \
  template <>                                                                                     \
  void launch_b_tiled<R>(const WorkItem *items, int nitems, const Cx<R>::T *grid, const R *xs,    \
                         const uint32_t *perm, Cx<R>::T *f, const Geom<R> &g, cudaStream_t s)     \
  {                                                                                               \
    launch_b_tiled_impl<R>(items, nitems, grid, xs, perm, f, g, s);                               \
  }                                                                                               \
  template <>                                                                                     \
  void launch_bt_tiled<R>(const WorkItem *items, int nitems, Cx<R>::T *grid, const R *xs,         \
                          const uint32_t *perm, const Cx<R>::T *f, const Geom<R> &g,              \
                          cudaStream_t s)                                                         \
  {                                                                                               \
    launch_bt_tiled_impl<R>(items, nitems, grid, xs, perm, f, g, s);                              \
  }                                                                                               \
  }
