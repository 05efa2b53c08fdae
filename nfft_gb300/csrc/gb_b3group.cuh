// gb_b3group.cuh -- 3-D B (interpolation) and B^T (spreading) by separable
// sub-cell groups: the hot kernels of the 3-D transform.
//
// Reference: nfft_trafo_3d_B (nfft.c:4687-4914) with nfft_trafo_3d_compute
// (nfft.c:4020-4265), and nfft_adjoint_3d_B (nfft.c:5126-5384) with its
// blockwise scatter (nfft.c:4289-4388).
//
// Node set-up sorts the nodes by (tile, sub-cell): a tile is 8^3 cells of the
// oversampled grid, a sub-cell CS^3 cells of a tile.  All nodes whose window
// start lies in one sub-cell share one box of (w + CS - 1)^3 grid cells.
//
// A CTA takes one work item (a tile and a range of its nodes) and stages the
// tile's padded subgrid ((8 + w - 1)^3 cells, wrapped periodically) in shared
// memory as separate real and imaginary planes whose x / y strides are padded
// so that the 32 box rows a warp reads at once fall in distinct banks.  The
// item's nodes are cut into units of at most PMAX nodes of one sub-cell; the
// warps take units in turn:
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
static constexpr int G3_TILE = 8;          // tile edge (cells)
static constexpr int G3_WINDOW = 1024;     // nodes per unit-building window
static constexpr int G3_MAXITEM = 16384;   // nodes per work item

// nodes per unit: B keeps 2 PMAX partial sums per lane, B^T 2 (w + CS - 1)
// accumulators, so B^T prefers smaller units
template <typename R> __host__ __device__ constexpr int g3_pm_b() { return sizeof(R) == 4 ? 16 : 8; }
template <typename R> __host__ __device__ constexpr int g3_pm_bt() { return 8; }

template <typename R, int W, int CS, int PM>
struct G3 {
  static constexpr int EXT = G3_TILE + W - 1;                     // padded subgrid edge
  static constexpr int BOX = W + CS - 1;                          // box edge
  static constexpr int BOXP = (BOX + 3) / 4 * 4;                  // padded for vector loads
  static constexpr int ROWS = BOX * BOX;                          // (x, y) rows of a box
  static constexpr int RITER = (ROWS + 31) / 32;                  // row iterations per lane
  static constexpr int PMAX = PM;                                 // nodes per unit
  static constexpr int NV = 2 * PMAX;                             // reduced values per unit
  // per-warp scratch (R): wx, wy, wz [PMAX][BOXP] each, f values [PMAX][2],
  // window offsets t0 [3 PMAX], box offsets o [3 PMAX] (as int)
  static constexpr int WARP_FLOATS = 3 * PMAX * BOXP + 2 * PMAX + 6 * PMAX;
  static constexpr int INTS = 4 * G3_WINDOW + 2 + G3_WARPS;       // sub, gstart, ucount, ustart, wsum
};

template <typename R, int W, int CS, int PM = (g3_pm_b<R>() > g3_pm_bt<R>() ? g3_pm_b<R>() : g3_pm_bt<R>())>
inline size_t g3_smem_bytes(const Geom<R> &g)
{
  typedef G3<R, W, CS, PM> P;
  const size_t plane = (size_t)P::EXT * g.sx;
  return (2 * plane + (size_t)G3_WARPS * P::WARP_FLOATS) * sizeof(R) + P::INTS * sizeof(int);
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
    s = s * (G3_TILE / CS) + sc;
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
// warp's zero-padded box vectors w[t][j][b] ([3][PMAX][BOXP]).  t0 / so are
// per (node, dim) scratch: t0 = n x - u (the argument of tap 0), so = box
// offset of the window.
template <typename R, int W, int CS, int PM>
__device__ __forceinline__ void g3_unit_weights(int u0, int np, const R *__restrict__ xs, const Geom<R> &g,
                                                const int *org, const int *box0, R *w, R *t0, int *so)
{
  typedef G3<R, W, CS, PM> P;
  const int lane = threadIdx.x & 31;
  for (int k = lane; k < 3 * np; k += 32) {
    const int j = k / 3, t = k - 3 * j;
    const R xn = xs[(long long)(u0 + j) * 3 + t] * g.nR[t];
    const int u = (int)gb_floor(xn) - g.m;  // node_u
    so[k] = wrap(u, g.n[t]) - org[t] - box0[t];
    t0[k] = xn - R(u);
  }
  __syncwarp();
  for (int k = lane; k < 3 * np * P::BOXP; k += 32) {
    const int jt = k / P::BOXP, b = k - jt * P::BOXP;
    const int j = jt / 3, t = jt - 3 * j;
    const int l = b - so[jt];
    R v = R(0);
    if (l >= 0 && l < W) v = kb_window_t(t0[jt] - R(l), g.mm, g.b[t]);
    w[(t * P::PMAX + j) * P::BOXP + b] = v;
  }
  __syncwarp();
}

template <typename R>
__device__ __forceinline__ void g3_tile_origin(const WorkItem &it, const Geom<R> &g, int *org)
{
  int rem = it.tile;
#pragma unroll
  for (int t = 2; t >= 0; --t) {
    org[t] = (rem % g.ntile[t]) * G3_TILE;
    rem /= g.ntile[t];
  }
}

// subgrid cell idx (row-major over EXT^3) -> shared index and global index
template <typename R, int EXT>
__device__ __forceinline__ void g3_cell(int idx, const int *org, const Geom<R> &g, int &si, long long &gi)
{
  const int c2 = idx % EXT, r = idx / EXT;
  const int c1 = r % EXT, c0 = r / EXT;
  si = c0 * g.sx + c1 * g.sy + c2;
  int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
  while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
  while (p1 >= g.n[1]) p1 -= g.n[1];
  while (p2 >= g.n[2]) p2 -= g.n[2];
  gi = ((long long)p0 * g.n[1] + p1) * g.n[2] + p2;
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

template <typename R, int W, int CS, int PM>
struct G3Smem {
  R *w, *fv, *t0;
  int *so;
  R *sre, *sim;
  int *sub, *gstart, *ucnt, *ustart, *wsum;
  __device__ G3Smem(unsigned char *raw, const Geom<R> &g)
  {
    typedef G3<R, W, CS, PM> P;
    R *base = reinterpret_cast<R *>(raw);  // per-warp scratch first: 16-byte aligned
    w = base + (threadIdx.x >> 5) * P::WARP_FLOATS;
    fv = w + 3 * P::PMAX * P::BOXP;
    t0 = fv + 2 * P::PMAX;
    so = reinterpret_cast<int *>(t0 + 3 * P::PMAX);
    sre = base + G3_WARPS * P::WARP_FLOATS;
    sim = sre + P::EXT * g.sx;
    sub = reinterpret_cast<int *>(sim + P::EXT * g.sx);
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
  constexpr int PM = g3_pm_b<R>();
  typedef G3<R, W, CS, PM> P;
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  G3Smem<R, W, CS, PM> S(smem_raw, g);
  const R *wx = S.w, *wy = S.w + P::PMAX * P::BOXP, *wz = S.w + 2 * P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  for (int idx = threadIdx.x; idx < P::EXT * P::EXT * P::EXT; idx += G3_THREADS) {
    int si;
    long long gi;
    g3_cell<R, P::EXT>(idx, org, g, si, gi);
    const C v = grid[gi];
    S.sre[si] = v.x;
    S.sim[si] = v.y;
  }
  for (int c0 = it.start; c0 < it.end; c0 += G3_WINDOW) {
    const int c1 = min(c0 + G3_WINDOW, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, S.sub, S.gstart, S.ucnt, S.ustart, S.wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = S.ustart[ui], np = S.ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      g3_unit_weights<R, W, CS, PM>(u0, np, xs, g, org, box0, S.w, S.t0, S.so);
      const int sbase = box0[0] * g.sx + box0[1] * g.sy + box0[2];
      R acc[P::NV];
#pragma unroll
      for (int j = 0; j < P::NV; ++j) acc[j] = R(0);
#pragma unroll 1
      for (int ri = 0; ri < P::RITER; ++ri) {
        const int row = lane + 32 * ri;
        if (row < P::ROWS) {
          const int bx = row / P::BOX, by = row - bx * P::BOX;
          const int base = sbase + bx * g.sx + by * g.sy;
          R gr[P::BOX], gim[P::BOX];
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) {
            gr[z] = S.sre[base + z];
            gim[z] = S.sim[base + z];
          }
#pragma unroll
          for (int j = 0; j < P::PMAX; ++j) {
            if (j < np) {
              R wzj[P::BOXP];
              g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
              R tr0 = R(0), ti0 = R(0), tr1 = R(0), ti1 = R(0);
#pragma unroll
              for (int z = 0; z + 1 < P::BOX; z += 2) {
                tr0 += wzj[z] * gr[z];
                ti0 += wzj[z] * gim[z];
                tr1 += wzj[z + 1] * gr[z + 1];
                ti1 += wzj[z + 1] * gim[z + 1];
              }
              if (P::BOX & 1) {
                tr0 += wzj[P::BOX - 1] * gr[P::BOX - 1];
                ti0 += wzj[P::BOX - 1] * gim[P::BOX - 1];
              }
              const R wxy = wx[j * P::BOXP + bx] * wy[j * P::BOXP + by];
              acc[2 * j] += wxy * (tr0 + tr1);
              acc[2 * j + 1] += wxy * (ti0 + ti1);
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
  constexpr int PM = g3_pm_bt<R>();
  typedef G3<R, W, CS, PM> P;
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  G3Smem<R, W, CS, PM> S(smem_raw, g);
  const R *wx = S.w, *wy = S.w + P::PMAX * P::BOXP, *wz = S.w + 2 * P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  for (int i = threadIdx.x; i < P::EXT * g.sx; i += G3_THREADS) {
    S.sre[i] = R(0);
    S.sim[i] = R(0);
  }
  for (int c0 = it.start; c0 < it.end; c0 += G3_WINDOW) {
    const int c1 = min(c0 + G3_WINDOW, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, S.sub, S.gstart, S.ucnt, S.ustart, S.wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = S.ustart[ui], np = S.ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      if (lane < np) {
        const C v = f[perm[u0 + lane]];
        S.fv[2 * lane] = v.x;
        S.fv[2 * lane + 1] = v.y;
      }
      g3_unit_weights<R, W, CS, PM>(u0, np, xs, g, org, box0, S.w, S.t0, S.so);  // ends with __syncwarp
      const int sbase = box0[0] * g.sx + box0[1] * g.sy + box0[2];
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
              const R hr = wxy * S.fv[2 * j], hi = wxy * S.fv[2 * j + 1];
              R wzj[P::BOXP];
              g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
#pragma unroll
              for (int z = 0; z < P::BOX; ++z) {
                ar[z] += wzj[z] * hr;
                ai[z] += wzj[z] * hi;
              }
            }
          }
          const int base = sbase + bx * g.sx + by * g.sy;
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) {
            atomicAdd(S.sre + base + z, ar[z]);
            atomicAdd(S.sim + base + z, ai[z]);
          }
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
  // one vector reduction per non-zero cell of the padded subgrid
  for (int idx = threadIdx.x; idx < P::EXT * P::EXT * P::EXT; idx += G3_THREADS) {
    int si;
    long long gi;
    g3_cell<R, P::EXT>(idx, org, g, si, gi);
    const R vr = S.sre[si], vi = S.sim[si];
    if (vr == R(0) && vi == R(0)) continue;
    global_add_c(grid + gi, cmake(vr, vi));
  }
}

}  // namespace gb
