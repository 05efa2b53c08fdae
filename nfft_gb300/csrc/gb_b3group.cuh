// gb_b3group.cuh -- 3-D B (interpolation) and B^T (spreading) by separable
// sub-cell groups: the hot kernels of the 3-D transform.
//
// Reference: nfft_trafo_3d_B (nfft.c:4687-4914) with nfft_trafo_3d_compute
// (nfft.c:4020-4265), and nfft_adjoint_3d_B (nfft.c:5126-5384) with its
// blockwise scatter (nfft.c:4289-4388).
//
// Node set-up sorts the nodes by (tile, sub-cell): a tile is T^3 cells of the
// oversampled grid, a sub-cell CS^3 cells of a tile.  All nodes whose window
// start lies in one sub-cell share one box of (w + CS - 1)^3 grid cells.
//
// A CTA takes one work item (a tile and a range of its nodes) and stages the
// tile's padded subgrid ((T + w - 1)^3 cells, wrapped periodically) in shared
// memory as separate real and imaginary planes; rows are ext_z apart (odd),
// so the row accesses of a warp hit distinct banks.  The item's nodes are cut
// into units of at most PMAX nodes of one sub-cell; the warps take units in
// turn:
//  * all 32 lanes evaluate the unit's Kaiser-Bessel window values on the fly
//    (3 (2m+2) per node) into zero-padded box vectors in shared memory;
//  * the lanes own the (x, y) rows of the box and hold a row's w + CS - 1
//    values along z in registers;
//  * B   contracts z by FMAs, then x and y, and reduces the per-lane partial
//        sums of the unit's nodes with one butterfly transpose-reduction;
//  * B^T builds the rank-1 tensor products of the unit's nodes in registers
//        and adds each row to the shared subgrid once per unit (not once per
//        tap and node); the subgrid goes to the global grid once per item.
#pragma once

#include <type_traits>

#include "gb_internal.h"

namespace gb {

static constexpr int G3_THREADS = 256;
static constexpr int G3_WARPS = G3_THREADS / 32;
static constexpr int G3_WINDOW = 1024;     // nodes per unit-building window
static constexpr int G3_MAXITEM = 16384;   // nodes per work item

template <typename R, int W, int CS>
struct G3 {
  static constexpr int BOX = W + CS - 1;                          // box edge
  static constexpr int BOXP = (BOX + 3) / 4 * 4;                  // padded for vector loads
  static constexpr int ROWS = BOX * BOX;                          // (x, y) rows of a box
  static constexpr int RITER = (ROWS + 31) / 32;                  // row iterations per lane
  static constexpr int PMAX = sizeof(R) == 4 ? 16 : 8;            // nodes per unit
  static constexpr int NV = 2 * PMAX;                             // reduced values per unit
  static constexpr int WARP_FLOATS = 3 * PMAX * BOXP + 2 * PMAX;  // per-warp scratch (R)
  static constexpr int INTS = 4 * G3_WINDOW + 2 + G3_WARPS;       // sub, gstart, ucount, ustart, wsum
};

template <typename R, int W, int CS>
inline size_t g3_smem_bytes(const Geom<R> &g)
{
  typedef G3<R, W, CS> P;
  const size_t cells = (size_t)g.ext[0] * g.ext[1] * g.ext[2];
  return (2 * cells + (size_t)G3_WARPS * P::WARP_FLOATS) * sizeof(R) + P::INTS * sizeof(int);
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
// box0 = origin of that sub-cell relative to the tile origin
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

// Exclusive scan of n <= 4 * G3_THREADS ints in place; returns the total.
__device__ __forceinline__ int g3_block_scan(int *a, int n, int *wsum)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = threadIdx.x * 4;
  int v[4], s = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[i] = (b + i < n) ? a[b + i] : 0;
    s += v[i];
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < G3_WARPS; ++w) {
    if (w < warp) before += wsum[w];
    total += wsum[w];
  }
  int run = before + incl - s;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (b + i < n) a[b + i] = run;
    run += v[i];
  }
  __syncthreads();
  return total;
}

// Units of one window [c0, c1) of sorted nodes: runs of equal sub-cell cut
// into pieces of at most PMAX nodes.  ustart[0..nu] (ustart[nu] = c1).
template <typename R, int CS, int PMAX>
__device__ int g3_units(int c0, int c1, const R *__restrict__ xs, const Geom<R> &g, const int *org,
                        int *sub, int *gstart, int *ucnt, int *ustart, int *wsum)
{
  const int n = c1 - c0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < n; k += G3_THREADS) {
    int b[3];
    sub[k] = node_subcell<R, CS>(xs + (long long)(c0 + k) * 3, g, org, b);
  }
  __syncthreads();
  // ordered compaction of the run heads
  int ng = 0;
  for (int k0 = 0; k0 < n; k0 += G3_THREADS) {
    const int k = k0 + threadIdx.x;
    const bool head = k < n && (k == 0 || sub[k] != sub[k - 1]);
    const unsigned bal = __ballot_sync(0xffffffffu, head);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int before = ng, total = 0;
#pragma unroll
    for (int w = 0; w < G3_WARPS; ++w) {
      if (w < warp) before += wsum[w];
      total += wsum[w];
    }
    if (head) gstart[before + __popc(bal & ((1u << lane) - 1u))] = k;
    ng += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) gstart[ng] = n;
  __syncthreads();
  for (int k = threadIdx.x; k < ng; k += G3_THREADS)
    ucnt[k] = (gstart[k + 1] - gstart[k] + PMAX - 1) / PMAX;
  __syncthreads();
  const int nu = g3_block_scan(ucnt, ng, wsum);
  for (int k = threadIdx.x; k < ng; k += G3_THREADS) {
    const int s0 = gstart[k], s1 = gstart[k + 1];
    int u = ucnt[k];
    for (int p = s0; p < s1; p += PMAX) ustart[u++] = c0 + p;
  }
  if (threadIdx.x == 0) ustart[nu] = c1;
  __syncthreads();
  return nu;
}

// All 32 lanes evaluate the window values of the unit's np nodes into the
// warp's zero-padded box vectors wx, wy, wz ([PMAX][BOXP] each).
template <typename R, int W, int CS>
__device__ __forceinline__ void g3_unit_weights(int u0, int np, const R *__restrict__ xs, const Geom<R> &g,
                                                const int *org, const int *box0, R *wx)
{
  typedef G3<R, W, CS> P;
  const int lane = threadIdx.x & 31;
  const int nz = 3 * P::PMAX * P::BOXP;
  for (int k = lane; k < nz; k += 32) wx[k] = R(0);
  __syncwarp();
  for (int k = lane; k < np * 3 * W; k += 32) {
    const int j = k / (3 * W), rem = k - j * (3 * W);
    const int t = rem / W, l = rem - t * W;
    const R x = xs[(long long)(u0 + j) * 3 + t];
    const int u = node_u<R>(x, g.nR[t], g.m);
    const int o = wrap(u, g.n[t]) - org[t] - box0[t];  // in [0, CS)
    wx[(t * P::PMAX + j) * P::BOXP + o + l] = kb_phi<R>(x - R(u + l) / g.nR[t], g.nR[t], g.mm, g.b[t]);
  }
  __syncwarp();
}

template <typename R>
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

// load the padded z-vector of a node's box (BOXP reals) from shared memory
template <typename R, int BOXP>
__device__ __forceinline__ void g3_load_vec(const R *src, R (&dst)[BOXP])
{
  typedef typename std::conditional<sizeof(R) == 4, float4, double2>::type V;
  constexpr int VPER = sizeof(V) / sizeof(R);
  const V *v = reinterpret_cast<const V *>(src);
#pragma unroll
  for (int q = 0; q < BOXP / VPER; ++q) {
    const V t = v[q];
    const R *tt = reinterpret_cast<const R *>(&t);
#pragma unroll
    for (int e = 0; e < VPER; ++e) dst[q * VPER + e] = tt[e];
  }
}

struct G3Smem {
  template <typename R, int W, int CS>
  __device__ static void carve(unsigned char *raw, int cells, R *&wscratch, R *&sre, R *&sim, int *&sub,
                               int *&gstart, int *&ucnt, int *&ustart, int *&wsum)
  {
    typedef G3<R, W, CS> P;
    R *base = reinterpret_cast<R *>(raw);  // per-warp scratch first: 16-byte aligned
    wscratch = base + (threadIdx.x >> 5) * P::WARP_FLOATS;
    sre = base + G3_WARPS * P::WARP_FLOATS;
    sim = sre + cells;
    sub = reinterpret_cast<int *>(sim + cells);
    gstart = sub + G3_WINDOW;
    ucnt = gstart + G3_WINDOW + 1;
    ustart = ucnt + G3_WINDOW;
    wsum = ustart + G3_WINDOW + 1;
  }
};

template <typename R, int W, int CS>
__global__ void __launch_bounds__(G3_THREADS, 2) k_b3_group(const WorkItem *__restrict__ items,
                                                             const typename Cx<R>::T *__restrict__ grid,
                                                             const R *__restrict__ xs,
                                                             const uint32_t *__restrict__ perm,
                                                             typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  typedef G3<R, W, CS> P;
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cells = g.ext[0] * g.ext[1] * g.ext[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  R *wx, *sre, *sim;
  int *sub, *gstart, *ucnt, *ustart, *wsum;
  G3Smem::carve<R, W, CS>(smem_raw, cells, wx, sre, sim, sub, gstart, ucnt, ustart, wsum);
  R *wy = wx + P::PMAX * P::BOXP;
  R *wz = wy + P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    const C v = grid[g3_global_cell<R>(idx, org, g)];
    sre[idx] = v.x;
    sim[idx] = v.y;
  }
  const int e1 = g.ext[1], e2 = g.ext[2];
  for (int c0 = it.start; c0 < it.end; c0 += G3_WINDOW) {
    const int c1 = min(c0 + G3_WINDOW, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, sub, gstart, ucnt, ustart, wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = ustart[ui], np = ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      g3_unit_weights<R, W, CS>(u0, np, xs, g, org, box0, wx);
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
              g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
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
      if (lane < np) f[perm[u0 + lane]] = cmake(re, im);
      __syncwarp();
    }
    __syncthreads();
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
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cells = g.ext[0] * g.ext[1] * g.ext[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  R *wx, *sre, *sim;
  int *sub, *gstart, *ucnt, *ustart, *wsum;
  G3Smem::carve<R, W, CS>(smem_raw, cells, wx, sre, sim, sub, gstart, ucnt, ustart, wsum);
  R *wy = wx + P::PMAX * P::BOXP;
  R *wz = wy + P::PMAX * P::BOXP;
  R *fv = wz + P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    sre[idx] = R(0);
    sim[idx] = R(0);
  }
  const int e1 = g.ext[1], e2 = g.ext[2];
  for (int c0 = it.start; c0 < it.end; c0 += G3_WINDOW) {
    const int c1 = min(c0 + G3_WINDOW, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, sub, gstart, ucnt, ustart, wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = ustart[ui], np = ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      if (lane < np) {
        const C v = f[perm[u0 + lane]];
        fv[2 * lane] = v.x;
        fv[2 * lane + 1] = v.y;
      }
      g3_unit_weights<R, W, CS>(u0, np, xs, g, org, box0, wx);  // ends with __syncwarp
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
              g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
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
    __syncthreads();
  }
  // one vector reduction per non-zero cell of the padded subgrid
  for (int idx = threadIdx.x; idx < cells; idx += G3_THREADS) {
    const R vr = sre[idx], vi = sim[idx];
    if (vr == R(0) && vi == R(0)) continue;
    global_add_c(grid + g3_global_cell<R>(idx, org, g), cmake(vr, vi));
  }
}

}  // namespace gb
