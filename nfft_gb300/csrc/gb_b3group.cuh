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
// Nodes per unit-building window (B, B^T): a smaller window shrinks the
// index scratch, which lets three B^T CTAs share an SM.
#ifndef GB_G3_WINDOW
#define GB_G3_WINDOW 1024
#endif
#ifndef GB_G3_WINDOW_BT
#define GB_G3_WINDOW_BT 512
#endif
static constexpr int G3_MAXITEM = 16384;   // nodes per work item

// Nodes per unit: B keeps 2 PMAX partial sums per lane, B^T 2 (w + CS - 1)
// accumulators per row, so B^T prefers smaller units.
#ifndef GB_G3_PM_B_FLOAT
#define GB_G3_PM_B_FLOAT 16
#endif
#ifndef GB_G3_PM_BT_FLOAT
#define GB_G3_PM_BT_FLOAT 16
#endif
// Box rows a lane holds at once (they share the unit's z weight vectors);
// B^T keeps 2 (w + CS - 1) accumulators per row, so it holds fewer.
#ifndef GB_G3_ROWS_PER_LANE
#define GB_G3_ROWS_PER_LANE 2
#endif
#ifndef GB_G3_ROWS_PER_LANE_BT
#define GB_G3_ROWS_PER_LANE_BT 1
#endif
template <typename R> __host__ __device__ constexpr int g3_pm_b() { return sizeof(R) == 4 ? GB_G3_PM_B_FLOAT : 8; }
template <typename R> __host__ __device__ constexpr int g3_pm_bt() { return sizeof(R) == 4 ? GB_G3_PM_BT_FLOAT : 8; }
template <typename R, int W, bool ADJ> __host__ __device__ constexpr int g3_rpl()
{
  return (sizeof(R) == 4 && W >= 10 && W <= 12) ? (ADJ ? GB_G3_ROWS_PER_LANE_BT : GB_G3_ROWS_PER_LANE) : 1;
}

template <typename R, int W, int CS, int PM, bool ADJ = false>
struct G3 {
  static constexpr int EXT = G3_TILE + W - 1;                     // padded subgrid edge
  static constexpr int BOX = W + CS - 1;                          // box edge
  static constexpr int BOXP = (BOX + 3) / 4 * 4;                  // padded for vector loads
  static constexpr int ROWS = BOX * BOX;                          // (x, y) rows of a box
  static constexpr int RPL = g3_rpl<R, W, ADJ>();                 // rows a lane holds at once
  static constexpr int RITER = (ROWS + 32 * RPL - 1) / (32 * RPL);  // row iterations per lane
  static constexpr int PMAX = PM;                                 // nodes per unit
  static constexpr int NV = 2 * PMAX;                             // reduced values per unit
  // per-warp scratch (R): window vectors [4][PMAX][BOXP] (x, y, z, and for
  // B^T x scaled by Im f while slot 0 holds x scaled by Re f)
  static constexpr int WARP_FLOATS = 4 * PMAX * BOXP;
  static constexpr int WIN = ADJ ? GB_G3_WINDOW_BT : GB_G3_WINDOW;  // nodes per unit-building window
  static constexpr int INTS = 4 * WIN + 2 + G3_WARPS;             // sub, gstart, ucount, ustart, wsum
};

template <typename R, int W, int CS, bool ADJ>
inline size_t g3_smem_bytes(const Geom<R> &g)
{
  typedef G3<R, W, CS, ADJ ? g3_pm_bt<R>() : g3_pm_b<R>(), ADJ> P;
  const size_t plane = (size_t)P::EXT * g.sx;
  return (2 * plane + (size_t)G3_WARPS * P::WARP_FLOATS) * sizeof(R) + P::INTS * sizeof(int);
}

// the larger of the B and B^T kernels' dynamic shared memory
template <typename R, int W, int CS>
inline size_t g3_smem_max(const Geom<R> &g)
{
  const size_t b = g3_smem_bytes<R, W, CS, false>(g), bt = g3_smem_bytes<R, W, CS, true>(g);
  return b > bt ? b : bt;
}

// Butterfly transpose-reduction over the warp of the first K (16 or 32)
// values of each lane; lane l holds the warp-wide sum of value (l mod K) in
// v[0] on return.
template <typename R, int K, int NV>
__device__ __forceinline__ void warp_transpose_reduce(R (&v)[NV])
{
  static_assert(K <= NV && (K == 16 || K == 32), "K");
  const int lane = threadIdx.x & 31;
  if (K == 16) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], 16);
  }
#pragma unroll
  for (int h = K / 2; h >= 1; h >>= 1) {
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

// store BOXP reals (a padded window vector) to shared memory with vector stores
template <typename R, int BOXP>
__device__ __forceinline__ void g3_store_vec(R *dst, const R (&src)[BOXP])
{
  typedef typename std::conditional<sizeof(R) == 4, float4, double2>::type V;
  constexpr int VPER = sizeof(V) / sizeof(R);
  V *v = reinterpret_cast<V *>(dst);
#pragma unroll
  for (int q = 0; q < BOXP / VPER; ++q) {
    V t;
    R *tt = reinterpret_cast<R *>(&t);
#pragma unroll
    for (int e = 0; e < VPER; ++e) tt[e] = src[q * VPER + e];
    v[q] = t;
  }
}

// Window vectors of a unit: lane k < 3 np takes node j = k / 3, dimension
// t = k mod 3, evaluates its W taps phi(t0 - l), t0 = n x - u, and stores
// them zero-padded at the window's offset so in [0, CS) of the box:
// w[t][j][b] ([3][PMAX][BOXP]).  With fv != nullptr (B^T), the x vector is
// stored twice, scaled by Re f_j in slot 0 and by Im f_j in slot 3.
template <typename R, int W, int CS, int PM>
__device__ __forceinline__ void g3_unit_weights(int u0, int np, const R *__restrict__ xs, const Geom<R> &g,
                                                const int *org, const int *box0, R *w,
                                                const typename Cx<R>::T *__restrict__ fv = nullptr,
                                                const uint32_t *__restrict__ perm = nullptr)
{
  typedef G3<R, W, CS, PM> P;
  const int lane = threadIdx.x & 31;
  for (int k = lane; k < 3 * np; k += 32) {
    const int j = k / 3, t = k - 3 * j;
    const R xn = xs[(long long)(u0 + j) * 3 + t] * g.nR[t];
    const int u = (int)gb_floor(xn) - g.m;  // node_u
    const int so = wrap(u, g.n[t]) - org[t] - box0[t];
    const R t0 = xn - R(u);
    R v[W];
#pragma unroll
    for (int l = 0; l < W; ++l) v[l] = kb_window_t(t0 - R(l), g.mm, g.b[t]);
    R out[P::BOXP];
#pragma unroll
    for (int b = 0; b < P::BOXP; ++b) {
      R val = R(0);
#pragma unroll
      for (int c = 0; c < CS; ++c)
        if (b - c >= 0 && b - c < W && so == c) val = v[b - c];
      out[b] = val;
    }
    if (fv != nullptr && t == 0) {
      const typename Cx<R>::T fj = fv[perm[u0 + j]];
      R o2[P::BOXP];
#pragma unroll
      for (int b = 0; b < P::BOXP; ++b) {
        o2[b] = out[b] * fj.y;
        out[b] *= fj.x;
      }
      g3_store_vec<R, P::BOXP>(w + (3 * P::PMAX + j) * P::BOXP, o2);
    }
    g3_store_vec<R, P::BOXP>(w + (t * P::PMAX + j) * P::BOXP, out);
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

// z contraction of one box row (B): (tr, ti) = sum_z wz[z] (gr[z], gi[z]).
template <typename R, int BOX, int BOXP>
__device__ __forceinline__ void g3_zdot(const R (&wz)[BOXP], const R (&gr)[BOX], const R (&gi)[BOX], R &tr, R &ti)
{
  R r0 = R(0), i0 = R(0), r1 = R(0), i1 = R(0);
#pragma unroll
  for (int z = 0; z + 1 < BOX; z += 2) {
    r0 += wz[z] * gr[z];
    i0 += wz[z] * gi[z];
    r1 += wz[z + 1] * gr[z + 1];
    i1 += wz[z + 1] * gi[z + 1];
  }
  if (BOX & 1) {
    r0 += wz[BOX - 1] * gr[BOX - 1];
    i0 += wz[BOX - 1] * gi[BOX - 1];
  }
  tr = r0 + r1;
  ti = i0 + i1;
}

// FP32: two adjacent z taps per paired FMA (fma.rn.f32x2 of the sm_100
// family), halving the issued instructions of the dominant loop.
template <int BOX, int BOXP>
__device__ __forceinline__ void g3_zdot(const float (&wz)[BOXP], const float (&gr)[BOX], const float (&gi)[BOX],
                                        float &tr, float &ti)
{
  float2 r2 = make_float2(0.f, 0.f), i2 = make_float2(0.f, 0.f);
#pragma unroll
  for (int z = 0; z + 1 < BOX; z += 2) {
    const float2 w2 = make_float2(wz[z], wz[z + 1]);
    r2 = __ffma2_rn(w2, make_float2(gr[z], gr[z + 1]), r2);
    i2 = __ffma2_rn(w2, make_float2(gi[z], gi[z + 1]), i2);
  }
  tr = r2.x + r2.y;
  ti = i2.x + i2.y;
  if (BOX & 1) {
    tr += wz[BOX - 1] * gr[BOX - 1];
    ti += wz[BOX - 1] * gi[BOX - 1];
  }
}

// rank-1 update of one box row (B^T): (ar[z], ai[z]) += wz[z] (hr, hi).
template <typename R, int BOX, int BOXP>
__device__ __forceinline__ void g3_zaxpy(const R (&wz)[BOXP], R hr, R hi, R (&ar)[BOX], R (&ai)[BOX])
{
#pragma unroll
  for (int z = 0; z < BOX; ++z) {
    ar[z] += wz[z] * hr;
    ai[z] += wz[z] * hi;
  }
}

template <int BOX, int BOXP>
__device__ __forceinline__ void g3_zaxpy(const float (&wz)[BOXP], float hr, float hi, float (&ar)[BOX],
                                         float (&ai)[BOX])
{
  const float2 h2r = make_float2(hr, hr), h2i = make_float2(hi, hi);
#pragma unroll
  for (int z = 0; z + 1 < BOX; z += 2) {
    const float2 w2 = make_float2(wz[z], wz[z + 1]);
    const float2 a = __ffma2_rn(w2, h2r, make_float2(ar[z], ar[z + 1]));
    const float2 b = __ffma2_rn(w2, h2i, make_float2(ai[z], ai[z + 1]));
    ar[z] = a.x;
    ar[z + 1] = a.y;
    ai[z] = b.x;
    ai[z + 1] = b.y;
  }
  if (BOX & 1) {
    ar[BOX - 1] += wz[BOX - 1] * hr;
    ai[BOX - 1] += wz[BOX - 1] * hi;
  }
}

template <typename R, int W, int CS, int PM, bool ADJ>
struct G3Smem {
  R *w;
  R *sre, *sim;
  int *sub, *gstart, *ucnt, *ustart, *wsum;
  __device__ G3Smem(unsigned char *raw, const Geom<R> &g)
  {
    typedef G3<R, W, CS, PM, ADJ> P;
    R *base = reinterpret_cast<R *>(raw);  // per-warp scratch first: 16-byte aligned
    w = base + (threadIdx.x >> 5) * P::WARP_FLOATS;
    sre = base + G3_WARPS * P::WARP_FLOATS;
    sim = sre + P::EXT * g.sx;
    sub = reinterpret_cast<int *>(sim + P::EXT * g.sx);
    gstart = sub + P::WIN;
    ucnt = gstart + P::WIN + 1;
    ustart = ucnt + P::WIN;
    wsum = ustart + P::WIN + 1;
  }
};

// The box rows a lane holds in row iteration ri: row = lane + 32 (ri RPL + q);
// rows past the box are clamped to row 0 and flagged.
template <typename P>
__device__ __forceinline__ void g3_rows(int ri, int lane, int (&bx)[P::RPL], int (&by)[P::RPL],
                                        bool (&ok)[P::RPL])
{
#pragma unroll
  for (int q = 0; q < P::RPL; ++q) {
    const int row = lane + 32 * (ri * P::RPL + q);
    ok[q] = row < P::ROWS;
    const int rr = ok[q] ? row : 0;
    bx[q] = rr / P::BOX;
    by[q] = rr - bx[q] * P::BOX;
  }
}

template <typename R, int W, int CS>
__global__ void __launch_bounds__(G3_THREADS, 2) k_b3_group(const WorkItem *__restrict__ items,
                                                             const typename Cx<R>::T *__restrict__ grid,
                                                             const R *__restrict__ xs,
                                                             const uint32_t *__restrict__ perm,
                                                             typename Cx<R>::T *__restrict__ f, Geom<R> g)
{
  constexpr int PM = g3_pm_b<R>();
  typedef G3<R, W, CS, PM> P;
  constexpr int RPL = P::RPL;
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  G3Smem<R, W, CS, PM, false> S(smem_raw, g);
  const R *wx = S.w, *wy = S.w + P::PMAX * P::BOXP, *wz = S.w + 2 * P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  // several grid loads in flight per thread
#pragma unroll 4
  for (int idx = threadIdx.x; idx < P::EXT * P::EXT * P::EXT; idx += G3_THREADS) {
    int si;
    long long gi;
    g3_cell<R, P::EXT>(idx, org, g, si, gi);
    const C v = grid[gi];
    S.sre[si] = v.x;
    S.sim[si] = v.y;
  }
  for (int c0 = it.start; c0 < it.end; c0 += P::WIN) {
    const int c1 = min(c0 + P::WIN, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, S.sub, S.gstart, S.ucnt, S.ustart, S.wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = S.ustart[ui], np = S.ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      g3_unit_weights<R, W, CS, PM>(u0, np, xs, g, org, box0, S.w);
      const int sbase = box0[0] * g.sx + box0[1] * g.sy + box0[2];
      R acc[P::NV];
#pragma unroll
      for (int j = 0; j < P::NV; ++j) acc[j] = R(0);
#pragma unroll 1
      for (int ri = 0; ri < P::RITER; ++ri) {
        int bx[RPL], by[RPL];
        bool ok[RPL];
        g3_rows<P>(ri, lane, bx, by, ok);
        R gr[RPL][P::BOX], gim[RPL][P::BOX];
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int base = sbase + bx[q] * g.sx + by[q] * g.sy;
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) {
            gr[q][z] = S.sre[base + z];
            gim[q][z] = S.sim[base + z];
          }
        }
#pragma unroll
        for (int j = 0; j < P::PMAX; ++j) {
          if (j < np) {
            R wzj[P::BOXP];
            g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
            R tr[RPL], ti[RPL];
#pragma unroll
            for (int q = 0; q < RPL; ++q) g3_zdot(wzj, gr[q], gim[q], tr[q], ti[q]);
#pragma unroll
            for (int q = 0; q < RPL; ++q) {
              const R wxy = ok[q] ? wx[j * P::BOXP + bx[q]] * wy[j * P::BOXP + by[q]] : R(0);
              acc[2 * j] += wxy * tr[q];
              acc[2 * j + 1] += wxy * ti[q];
            }
          }
        }
      }
      if constexpr (P::NV >= 32) {
        if (np > 8) warp_transpose_reduce<R, 32>(acc);
        else warp_transpose_reduce<R, 16>(acc);
      } else {
        warp_transpose_reduce<R, 16>(acc);
      }
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
  typedef G3<R, W, CS, PM, true> P;
  constexpr int RPL = P::RPL;
  typedef typename Cx<R>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  G3Smem<R, W, CS, PM, true> S(smem_raw, g);
  // x vectors scaled by Re f (slot 0) and Im f (slot 3), y, z
  const R *wxr = S.w, *wy = S.w + P::PMAX * P::BOXP, *wz = S.w + 2 * P::PMAX * P::BOXP;
  const R *wxi = S.w + 3 * P::PMAX * P::BOXP;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  g3_tile_origin<R>(it, g, org);
  for (int i = threadIdx.x; i < P::EXT * g.sx; i += G3_THREADS) {
    S.sre[i] = R(0);
    S.sim[i] = R(0);
  }
  for (int c0 = it.start; c0 < it.end; c0 += P::WIN) {
    const int c1 = min(c0 + P::WIN, it.end);
    const int nu = g3_units<R, CS, P::PMAX>(c0, c1, xs, g, org, S.sub, S.gstart, S.ucnt, S.ustart, S.wsum);
    for (int ui = warp; ui < nu; ui += G3_WARPS) {
      const int u0 = S.ustart[ui], np = S.ustart[ui + 1] - u0;
      int box0[3];
      node_subcell<R, CS>(xs + (long long)u0 * 3, g, org, box0);
      g3_unit_weights<R, W, CS, PM>(u0, np, xs, g, org, box0, S.w, f, perm);  // ends with __syncwarp
      const int sbase = box0[0] * g.sx + box0[1] * g.sy + box0[2];
#pragma unroll 1
      for (int ri = 0; ri < P::RITER; ++ri) {
        int bx[RPL], by[RPL];
        bool ok[RPL];
        g3_rows<P>(ri, lane, bx, by, ok);
        R ar[RPL][P::BOX], ai[RPL][P::BOX];
#pragma unroll
        for (int q = 0; q < RPL; ++q)
#pragma unroll
          for (int z = 0; z < P::BOX; ++z) ar[q][z] = ai[q][z] = R(0);
#pragma unroll
        for (int j = 0; j < P::PMAX; ++j) {
          if (j < np) {
            R hr[RPL], hi[RPL];
#pragma unroll
            for (int q = 0; q < RPL; ++q) {
              const R wyq = wy[j * P::BOXP + by[q]];
              hr[q] = wxr[j * P::BOXP + bx[q]] * wyq;
              hi[q] = wxi[j * P::BOXP + bx[q]] * wyq;
            }
            R wzj[P::BOXP];
            g3_load_vec<R, P::BOXP>(wz + j * P::BOXP, wzj);
#pragma unroll
            for (int q = 0; q < RPL; ++q) g3_zaxpy(wzj, hr[q], hi[q], ar[q], ai[q]);
          }
        }
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          if (ok[q]) {
            const int base = sbase + bx[q] * g.sx + by[q] * g.sy;
#pragma unroll
            for (int z = 0; z < P::BOX; ++z) {
              atomicAdd(S.sre + base + z, ar[q][z]);
              atomicAdd(S.sim + base + z, ai[q][z]);
            }
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
