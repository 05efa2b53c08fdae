// gb_b3group.cuh -- 3-D B (interpolation) and B^T (spreading) by separable
// sub-cell groups: the hot kernels of the 3-D transform.
//
// Reference: nfft_trafo_3d_B (nfft.c:4687-4914) with nfft_trafo_3d_compute
// (nfft.c:4020-4265), and nfft_adjoint_3d_B (nfft.c:5126-5384) with its
// blockwise scatter (nfft.c:4289-4388).
//
// Node set-up sorts the nodes by (tile, sub-cell): a tile is T^3 cells of the
// oversampled grid, a sub-cell CS^3 cells of a tile.  All nodes whose window
// start lies in one sub-cell share one box of (w + CS - 1)^3 grid cells.  A
// warp treats such a group of nodes together:
//  * the lanes own the (x, y) rows of the box and hold a row's w + CS - 1
//    values along z in registers;
//  * each node's window is evaluated once, on the fly, into three
//    zero-padded vectors in shared memory, read back as broadcasts;
//  * B   contracts z by FMAs in registers, then x and y, and reduces the
//        per-lane partial sums of up to PMAX nodes with one butterfly
//        transpose-reduction over the warp;
//  * B^T builds the rank-1 tensor products of up to PMAX nodes in registers
//        and adds each row to the shared subgrid once per pass (instead of
//        once per tap and node).
// The tile's padded subgrid ((T + w - 1)^3 cells, wrapped periodically) sits
// in shared memory as separate real and imaginary planes; rows are ext_z
// apart (odd), so the row accesses of a warp hit distinct banks.
#pragma once

#include "gb_internal.h"

namespace gb {

static constexpr int G3_THREADS = 256;
static constexpr int G3_WARPS = G3_THREADS / 32;
static constexpr int G3_MAXITEM = 1024;  // nodes per work item (node set-up chunk)

template <typename R, int W, int CS>
struct G3 {
  static constexpr int BOX = W + CS - 1;                        // box edge
  static constexpr int BOXP = (BOX + 3) / 4 * 4;                // padded for vector loads
  static constexpr int ROWS = BOX * BOX;                        // (x, y) rows of a box
  static constexpr int RITER = (ROWS + 31) / 32;                // row iterations per lane
  static constexpr int PMAX = sizeof(R) == 4 ? 16 : 8;          // nodes per pass
  static constexpr int NV = 2 * PMAX;                           // reduced values per pass
  static constexpr int WARP_FLOATS = 3 * PMAX * BOXP + 2 * PMAX;  // per-warp scratch (R)
};

template <typename R, int W, int CS>
inline size_t g3_smem_bytes(const Geom<R> &g)
{
  typedef G3<R, W, CS> P;
  const size_t cells = (size_t)g.ext[0] * g.ext[1] * g.ext[2];
  return (2 * cells + (size_t)G3_WARPS * P::WARP_FLOATS) * sizeof(R) +
         (2 * G3_MAXITEM + 1 + G3_WARPS) * sizeof(int);
}

// Butterfly transpose-reduction over the warp: NV values per lane in; lane l
// holds the warp-wide sum of value (l mod NV) in v[0] on return.
template <typename R, int NV>
__device__ __forceinline__ void warp_transpose_reduce(R (&v)[NV])
{
  const int lane = threadIdx.x & 31;
  if (NV == 16) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], 16);
  }
#pragma unroll
  for (int h = NV / 2; h >= 1; h >>= 1) {
    const bool upper = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const R send = upper ? v[i] : v[i + h];
      const R keep = upper ? v[i + h] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
}

// sub-cell of a node inside its tile (row-major over the tile's sub-cells);
// loc = window start relative to the tile origin, box0 = its sub-cell origin
template <typename R, int CS>
__device__ __forceinline__ int node_subcell(const R *x3, const Geom<R> &g, const int *org, int *box0)
{
  int s = 0;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const int u = node_u<R>(x3[t], g.nR[t], g.m);
    const int loc = wrap(u, g.n[t]) - org[t];
    const int sc = loc / CS;
    box0[t] = sc * CS;
    s = s * (g.T[t] / CS) + sc;
  }
  return s;
}

// Group discovery inside one work item: gstart[k] = first node of the k-th
// run of equal sub-cell ids (in sorted order), gstart[ng] = item end.
template <typename R, int CS>
__device__ int g3_groups(const WorkItem &it, const R *__restrict__ xs, const Geom<R> &g,
                         const int *org, int *sub, int *gstart, int *wsum)
{
  const int n = it.end - it.start;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < n; k += G3_THREADS) {
    int b[3];
    sub[k] = node_subcell<R, CS>(xs + (long long)(it.start + k) * 3, g, org, b);
  }
  __syncthreads();
  int base = 0;
  for (int c0 = 0; c0 < n; c0 += G3_THREADS) {
    const int k = c0 + threadIdx.x;
    const bool head = k < n && (k == 0 || sub[k] != sub[k - 1]);
    const unsigned bal = __ballot_sync(0xffffffffu, head);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int before = base, total = 0;
#pragma unroll
    for (int w = 0; w < G3_WARPS; ++w) {
      if (w < warp) before += wsum[w];
      total += wsum[w];
    }
    if (head) gstart[before + __popc(bal & ((1u << lane) - 1u))] = it.start + k;
    base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) gstart[base] = it.end;
  __syncthreads();
  return base;
}

// Window values of node i, zero-padded into the warp's box vectors.
template <typename R, int W, int CS>
__device__ __forceinline__ void g3_node_weights(long long i, const R *__restrict__ xs, const Geom<R> &g,
                                                const int *org, const int *box0, R *wx, R *wy, R *wz)
{
  typedef G3<R, W, CS> P;
  R *dst[3] = {wx, wy, wz};
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const R x = xs[i * 3 + t];
    const int u = node_u<R>(x, g.nR[t], g.m);
    const int o = wrap(u, g.n[t]) - org[t] - box0[t];  // in [0, CS)
    R psi[W];
    node_psi<R, W>(x, u, g.nR[t], g.mm, g.b[t], psi);
#pragma unroll
    for (int b = 0; b < P::BOXP; ++b) dst[t][b] = R(0);
#pragma unroll
    for (int q = 0; q < W; ++q) dst[t][o + q] = psi[q];
  }
}

template <typename R, int W, int CS>
__device__ __forceinline__ void g3_tile_origin(const WorkItem &it, const Geom<R> &g, int *org)
{
  int rem = it.tile;
#pragma unroll
  for (int t = 2; t >= 0; --t) {
    org[t] = (rem % g.ntile[t]) * g.T[t];
    rem /= g.ntile[t];
  }
}

template <typename R>
__device__ __forceinline__ long long g3_global_cell(int idx, const int *org, const Geom<R> &g)
{
  const int c2 = idx % g.ext[2], r = idx / g.ext[2];
  const int c1 = r % g.ext[1], c0 = r / g.ext[1];
  int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
  p0 = p0 >= g.n[0] ? p0 - g.n[0] : p0;
  p1 = p1 >= g.n[1] ? p1 - g.n[1] : p1;
  p2 = p2 >= g.n[2] ? p2 - g.n[2] : p2;
  return ((long long)p0 * g.n[1] + p1) * g.n[2] + p2;
}

template <typename R, int W, int CS>
__global__ void __launch_bounds__(G3_THREADS, 2) k_b3_group(const WorkItem *__restrict__ items,
                                                             const typename Cx<R>::T *__restrict__ grid,
                                                             const R *__restrict__ xs,
                                                             const uint32_t *__restrict__ perm,
                                                             typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef G3<R, W, CS> P;
  typedef typename Cx<R>::T C;
  typedef typename std::conditional<sizeof(R) == 4, float4, double2>::type V4;
  constexpr int VPER = sizeof(V4) / sizeof(R);  // reals per vector load
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cells = g.ext[0] * g.ext[1] * g.ext[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  R *wbase = reinterpret_cast<R *>(smem_raw);  // per-warp scratch first: 16-byte aligned
  R *wx = wbase + warp * P::WARP_FLOATS;
  R *wy = wx + P::PMAX * P::BOXP;
  R *wz = wy + P::PMAX * P::BOXP;
  R *sre = wbase + G3_WARPS * P::WARP_FLOATS;
  R *sim = sre + cells;
  int *sub = reinterpret_cast<int *>(sim + cells);
  int *gstart = sub + G3_MAXITEM;
  int *wsum = gstart + G3_MAXITEM + 1;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R, W, CS>(it, g, org);
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    const C v = grid[g3_global_cell<R>(idx, org, g)];
    sre[idx] = v.x;
    sim[idx] = v.y;
  }
  const int ng = g3_groups<R, CS>(it, xs, g, org, sub, gstart, wsum);  // has barriers
  const int e1 = g.ext[1], e2 = g.ext[2];

  for (int gi = warp; gi < ng; gi += G3_WARPS) {
    const int g0 = gstart[gi], g1 = gstart[gi + 1];
    int box0[3];
    node_subcell<R, CS>(xs + (long long)g0 * 3, g, org, box0);
    for (int p0 = g0; p0 < g1; p0 += P::PMAX) {
      const int np = min(P::PMAX, g1 - p0);
      if (lane < np)
        g3_node_weights<R, W, CS>(p0 + lane, xs, g, org, box0, wx + lane * P::BOXP,
                                  wy + lane * P::BOXP, wz + lane * P::BOXP);
      __syncwarp();
      R acc[P::NV];
#pragma unroll
      for (int j = 0; j < P::NV; ++j) acc[j] = R(0);
#pragma unroll 1
      for (int ri = 0; ri < P::RITER; ++ri) {
        const int row = lane + 32 * ri;
        if (row < P::ROWS) {
          const int bx = row / P::BOX, by = row - bx * P::BOX;
          const int base = ((box0[0] + bx) * e1 + (box0[1] + by)) * e2 + box0[2];
          R gr[P::BOX], gim[P::BOX];
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) {
            gr[z] = sre[base + z];
            gim[z] = sim[base + z];
          }
#pragma unroll
          for (int j = 0; j < P::PMAX; ++j) {
            if (j < np) {
              R wzj[P::BOXP];
              const V4 *wv = reinterpret_cast<const V4 *>(wz + j * P::BOXP);
#pragma unroll
              for (int q = 0; q < P::BOXP / VPER; ++q) {
                const V4 t = wv[q];
                const R *tt = reinterpret_cast<const R *>(&t);
#pragma unroll
                for (int e = 0; e < VPER; ++e) wzj[q * VPER + e] = tt[e];
              }
              R tr = R(0), ti = R(0);
#pragma unroll
              for (int z = 0; z < P::BOX; ++z) {
                tr += wzj[z] * gr[z];
                ti += wzj[z] * gim[z];
              }
              const R wxy = wx[j * P::BOXP + bx] * wy[j * P::BOXP + by];
              acc[2 * j] += wxy * tr;
              acc[2 * j + 1] += wxy * ti;
            }
          }
        }
      }
      warp_transpose_reduce<R, P::NV>(acc);
      const R re = __shfl_sync(0xffffffffu, acc[0], (2 * lane) & 31);
      const R im = __shfl_sync(0xffffffffu, acc[0], (2 * lane + 1) & 31);
      if (lane < np) f[perm[p0 + lane]] = cmake(re, im);
      __syncwarp();
    }
  }
}

template <typename R, int W, int CS>
__global__ void __launch_bounds__(G3_THREADS, 2) k_bt3_group(const WorkItem *__restrict__ items,
                                                              typename Cx<R>::T *__restrict__ grid,
                                                              const R *__restrict__ xs,
                                                              const uint32_t *__restrict__ perm,
                                                              const typename Cx<R>::T *__restrict__ f,
                                                              Geom<R> g)
{
  typedef G3<R, W, CS> P;
  typedef typename Cx<R>::T C;
  typedef typename std::conditional<sizeof(R) == 4, float4, double2>::type V4;
  constexpr int VPER = sizeof(V4) / sizeof(R);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cells = g.ext[0] * g.ext[1] * g.ext[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  R *wbase = reinterpret_cast<R *>(smem_raw);
  R *wx = wbase + warp * P::WARP_FLOATS;
  R *wy = wx + P::PMAX * P::BOXP;
  R *wz = wy + P::PMAX * P::BOXP;
  R *fv = wz + P::PMAX * P::BOXP;
  R *sre = wbase + G3_WARPS * P::WARP_FLOATS;
  R *sim = sre + cells;
  int *sub = reinterpret_cast<int *>(sim + cells);
  int *gstart = sub + G3_MAXITEM;
  int *wsum = gstart + G3_MAXITEM + 1;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R, W, CS>(it, g, org);
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    sre[idx] = R(0);
    sim[idx] = R(0);
  }
  const int ng = g3_groups<R, CS>(it, xs, g, org, sub, gstart, wsum);
  const int e1 = g.ext[1], e2 = g.ext[2];

  for (int gi = warp; gi < ng; gi += G3_WARPS) {
    const int g0 = gstart[gi], g1 = gstart[gi + 1];
    int box0[3];
    node_subcell<R, CS>(xs + (long long)g0 * 3, g, org, box0);
    for (int p0 = g0; p0 < g1; p0 += P::PMAX) {
      const int np = min(P::PMAX, g1 - p0);
      if (lane < np) {
        g3_node_weights<R, W, CS>(p0 + lane, xs, g, org, box0, wx + lane * P::BOXP,
                                  wy + lane * P::BOXP, wz + lane * P::BOXP);
        const C v = f[perm[p0 + lane]];
        fv[2 * lane] = v.x;
        fv[2 * lane + 1] = v.y;
      }
      __syncwarp();
#pragma unroll 1
      for (int ri = 0; ri < P::RITER; ++ri) {
        const int row = lane + 32 * ri;
        if (row < P::ROWS) {
          const int bx = row / P::BOX, by = row - bx * P::BOX;
          R ar[P::BOX], ai[P::BOX];
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) ar[z] = ai[z] = R(0);
#pragma unroll
          for (int j = 0; j < P::PMAX; ++j) {
            if (j < np) {
              const R wxy = wx[j * P::BOXP + bx] * wy[j * P::BOXP + by];
              const R hr = wxy * fv[2 * j], hi = wxy * fv[2 * j + 1];
              R wzj[P::BOXP];
              const V4 *wv = reinterpret_cast<const V4 *>(wz + j * P::BOXP);
#pragma unroll
              for (int q = 0; q < P::BOXP / VPER; ++q) {
                const V4 t = wv[q];
                const R *tt = reinterpret_cast<const R *>(&t);
#pragma unroll
                for (int e = 0; e < VPER; ++e) wzj[q * VPER + e] = tt[e];
              }
#pragma unroll
              for (int z = 0; z < P::BOX; ++z) {
                ar[z] += wzj[z] * hr;
                ai[z] += wzj[z] * hi;
              }
            }
          }
          const int base = ((box0[0] + bx) * e1 + (box0[1] + by)) * e2 + box0[2];
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) {
            atomicAdd(sre + base + z, ar[z]);
            atomicAdd(sim + base + z, ai[z]);
          }
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  // one vector reduction per non-zero cell of the padded subgrid
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    const R vr = sre[idx], vi = sim[idx];
    if (vr == R(0) && vi == R(0)) continue;
    global_add_c(grid + g3_global_cell<R>(idx, org, g), cmake(vr, vi));
  }
}

}  // namespace gb
