// gb_col2.cuh -- the single-precision 2-D column B^T and B of one work item
// (device functions), shared by the per-plan kernels of gb_col2.cu and the
// batched persistent kernels of gb_batch.cu.
//
// B^T: reference nfft_adjoint_2d_B (nfft.c:3583-3805) with its blockwise
// scatter (nfft.c:3064-3139): g[l mod n] += phi_0 phi_1 f_j over the
// (2m+2)^2 window of every node.  B: reference nfft_trafo_2d_B
// (nfft.c:3221-3410, per node nfft.c:2927-3004): f_j = sum of
// phi_0 phi_1 g[l mod n] over the same window.
//
// The per-node kernels (gb_btiled.cuh) serialise where nodes crowd: radial
// and spiral k-space trajectories pass every spoke or arm through the centre,
// a node's 2 (2m+2)^2 shared-memory atomic adds are compare-and-swap loops in
// single precision, and its gathers hit the same banks as its neighbours'.
// Here no node touches a cell by itself:
//  * node set-up sorts the nodes by (32^2 tile, column of the tile), a column
//    being CX x-cells by 8 y-cells of window starts; a column's nodes touch
//    ROWS = CX + W - 1 rows of the tile's padded subgrid over NPOS = 8 + W - 1
//    y positions;
//  * a warp takes 32 consecutive nodes of a work item (one or more columns);
//    lane j evaluates node j's window (the polynomial form, gb_window.cpp)
//    into per-warp vectors: its x taps at the node's row offset in its column
//    (scaled by f_j for B^T), its y taps at its y offset in a zero vector;
//  * lane (h, r) owns row r of the current column and half h of its y
//    positions.  B^T keeps the row's complex cells as accumulators in
//    registers and takes every node of the column with paired FMAs
//    (fma.rn.f32x2: two y positions per instruction), then adds them to the
//    shared subgrid once per column (64-bit compare-and-swap of the complex
//    cell, an atomic add where another warp got there in between); the
//    subgrid goes to the global grid once per work item with vector
//    reductions.  B keeps the row's cells of the subgrid in registers, forms
//    each node's partial sum over them with the same paired FMAs, and adds the
//    32 lanes' partials of eight nodes at a time with a transposing butterfly
//    (18 shuffles for eight complex sums).
#pragma once

#include "gb_internal.h"

namespace gb {

static constexpr int C2_THREADS = 256;
static constexpr int C2_WARPS = C2_THREADS / 32;
static constexpr int C2_TILE = 32;   // tile edge in both dimensions
static constexpr int C2_CY = 8;      // column depth along y
static constexpr int C2_SLABS = C2_TILE / C2_CY;
static constexpr int C2_CHUNK = 32;  // nodes per warp task (one per lane at set-up)

template <int W>
struct C2 {
  // column width along x: the widest power of two with ROWS <= 16
  static constexpr int CX = (17 - W) >= 8 ? 8 : (17 - W) >= 4 ? 4 : (17 - W) >= 2 ? 2 : 1;
  static constexpr int ROWS = CX + W - 1;
  static constexpr int NPOS = C2_CY + W - 1;  // y positions of a column
  static constexpr int NPAIR = (NPOS + 1) / 2;
  static constexpr int HP = (NPAIR + 1) / 2;  // y pairs per half-warp
  static constexpr int YV = 4 * HP;           // y vector length (floats)
  static constexpr int XS = 17;               // x vector stride (odd: set-up stores spread over banks)
  static constexpr int YS = YV + 2;           // y vector stride (floats; even: pairs stay aligned)
  static constexpr int EXT = C2_TILE + W - 1;  // padded subgrid edge
  static constexpr int SY = EXT | 1;           // subgrid row stride (complex)
  // per-warp scratch (floats): x vectors (complex for B^T, real for B), y vectors
  static constexpr int WARP_FLOATS_T = XS * C2_CHUNK + YS * C2_CHUNK;  // B^T keeps f_j at y slot YV
  static constexpr int WARP_FLOATS_B = XS * C2_CHUNK + YS * C2_CHUNK;
  static_assert(ROWS <= 16, "a column's rows fill at most a half-warp");
  static_assert(4 * HP >= NPOS, "two halves cover the column's y positions");
  static_assert(W % 2 == 0 && W <= KB_POLY_WMAX, "even window with a polynomial form");
};

// comp: B^T with a compensated subgrid (a second plane of rounding errors)
template <int W>
inline size_t c2_smem_bytes(bool adjoint, bool comp = false)
{
  typedef C2<W> P;
  return (size_t)C2_WARPS * (adjoint ? P::WARP_FLOATS_T : P::WARP_FLOATS_B) * sizeof(float)
         + (size_t)(comp ? 2 : 1) * P::EXT * P::SY * sizeof(float2);
}

// s = a + b rounded, and its rounding error e (a + b = s + e exactly): the
// error-free sum (TwoSum, Knuth), componentwise, in separately rounded steps
__device__ __forceinline__ float2 c2_two_sum(float2 a, float2 b, float2 &s)
{
  s = make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
  const float bx = __fsub_rn(s.x, a.x), by = __fsub_rn(s.y, a.y);
  return make_float2(__fadd_rn(__fsub_rn(a.x, __fsub_rn(s.x, bx)), __fsub_rn(b.x, bx)),
                     __fadd_rn(__fsub_rn(a.y, __fsub_rn(s.y, by)), __fsub_rn(b.y, by)));
}

// *p += v by 64-bit compare-and-swap on the complex cell; returns the
// rounding error of the add that went in
__device__ __forceinline__ float2 c2_cas_add_err(float2 *p, float2 v)
{
  unsigned long long *u = reinterpret_cast<unsigned long long *>(p);
  unsigned long long old = *reinterpret_cast<volatile unsigned long long *>(u);
  for (;;) {
    union {
      unsigned long long u;
      float2 f;
    } cur, nxt;
    cur.u = old;
    const float2 e = c2_two_sum(cur.f, v, nxt.f);
    const unsigned long long seen = atomicCAS(u, cur.u, nxt.u);
    if (seen == old) return e;
    old = seen;
  }
}

__device__ __forceinline__ unsigned long long c2_bits(float2 v)
{
  union {
    float2 f;
    unsigned long long u;
  } c;
  c.f = v;
  return c.u;
}

// Adds the lane's cells e < nv (pairs vr / vi: cell 2k + b holds component b
// of pair k) to the interleaved complex cells p[e]: each cell of a block of
// four is read, summed and offered by one 64-bit compare-and-swap before any
// result is checked; a cell another warp changed in between is added again
// with the atomic add of each component.  Zero cells are skipped.
// COMP: the compensated form for wide windows -- every add into p is
// error-free transformed and its rounding error is added into plo, the
// subgrid's error plane, so p + plo carries the column sums to about twice
// single precision.
template <int HP, bool COMP = false>
__device__ __forceinline__ void c2_flush(float2 *p, const float2 (&vr)[HP], const float2 (&vi)[HP], int nv,
                                         float2 *plo = nullptr)
{
  constexpr int N = 2 * HP, ZB = 4;
  volatile float2 *vp = p;
#pragma unroll
  for (int e0 = 0; e0 < N; e0 += ZB) {
    float2 cur[ZB], v[ZB];
    bool on[ZB];
#pragma unroll
    for (int q = 0; q < ZB; ++q) {
      const int e = e0 + q;
      on[q] = false;
      if (e < N) {
        v[q] = make_float2((e & 1) ? vr[e >> 1].y : vr[e >> 1].x, (e & 1) ? vi[e >> 1].y : vi[e >> 1].x);
        on[q] = e < nv && (v[q].x != 0.f || v[q].y != 0.f);
        if (on[q]) {
          const volatile float2 &c = vp[e];
          cur[q] = make_float2(c.x, c.y);
        }
      }
    }
    unsigned miss = 0;
    float2 err[ZB];
#pragma unroll
    for (int q = 0; q < ZB; ++q)
      if (on[q]) {
        float2 sum;
        if (COMP) err[q] = c2_two_sum(cur[q], v[q], sum);
        else sum = __fadd2_rn(cur[q], v[q]);
        const unsigned long long old = c2_bits(cur[q]);
        if (atomicCAS(reinterpret_cast<unsigned long long *>(p + e0 + q), old, c2_bits(sum)) != old) miss |= 1u << q;
      }
    if (COMP) {
#pragma unroll
      for (int q = 0; q < ZB; ++q)
        if (on[q]) {
          // a cell another warp changed in between: add again, with its error
          if ((miss >> q) & 1u) err[q] = c2_cas_add_err(p + e0 + q, v[q]);
          if (err[q].x != 0.f || err[q].y != 0.f) c2_cas_add_err(plo + e0 + q, err[q]);
        }
    } else if (miss) {
#pragma unroll
      for (int q = 0; q < ZB; ++q)
        if ((miss >> q) & 1u) {
          atomicAdd(&p[e0 + q].x, v[q].x);
          atomicAdd(&p[e0 + q].y, v[q].y);
        }
    }
  }
}

// The compensated write-back of one subgrid cell (hi, lo): hi goes into the
// grid by compare-and-swap with its rounding error, which joins lo in the
// grid's error plane (plain atomic adds: the error plane's own rounding is
// below single precision of the errors)
__device__ __forceinline__ void c2_global_add_comp(float2 *g, float2 *glo, float2 hi, float2 lo)
{
  const float2 e = c2_cas_add_err(g, hi);
  const float2 t = make_float2(__fadd_rn(e.x, lo.x), __fadd_rn(e.y, lo.y));
  if (t.x != 0.f || t.y != 0.f) global_add_c(glo, t);
}

// Set-up of one node (lane j of a task): its column in the tile at
// (org0, org1), from the same window starts as the sort key (node_u,
// wrapped), and its x / y windows written at its offsets in the column into
// the lane's vectors (x scaled by fj when ADJ).  Returns the column.
template <int W, bool ADJ>
__device__ __forceinline__ int c2_setup(const float *x, const Geom<float> &g, int org0, int org1,
                                        const WinPoly &poly, float2 fj, float *xv, float *yv)
{
  typedef C2<W> P;
  const float xn0 = x[0] * g.nR[0], xn1 = x[1] * g.nR[1];
  const int u0 = (int)floorf(xn0) - g.m, u1 = (int)floorf(xn1) - g.m;  // node_u
  const float s0 = fmaf(2.f, xn0 - (float)u0, -(float)(2 * g.m + 1));
  const float s1 = fmaf(2.f, xn1 - (float)u1, -(float)(2 * g.m + 1));
  const int ux = min(max(wrap(u0, g.n[0]) - org0, 0), C2_TILE - 1);
  const int uy = min(max(wrap(u1, g.n[1]) - org1, 0), C2_TILE - 1);
  const int ox = ux % P::CX, oy = uy % C2_CY;
  float v[W];
  kb_poly_taps_s<W>(s0, poly.c[0], v);
#pragma unroll
  for (int q = 0; q < 16; ++q) xv[q] = 0.f;
#pragma unroll
  for (int l = 0; l < W; ++l) xv[ox + l] = v[l];
  if (ADJ) reinterpret_cast<float2 *>(yv)[P::YV / 2] = fj;  // the node's f_j beside its y taps
#pragma unroll
  for (int q = 0; q < P::YV / 2; ++q) reinterpret_cast<float2 *>(yv)[q] = make_float2(0.f, 0.f);
  kb_poly_taps_s<W>(s1, poly.c[1], v);
#pragma unroll
  for (int l = 0; l < W; ++l) yv[oy + l] = v[l];
  return (ux / P::CX) * C2_SLABS + uy / C2_CY;
}

// B^T of one work item by a CTA of C2_THREADS threads with
// c2_smem_bytes<W>(true, COMP) bytes of shared memory at smem_raw; adds the
// item's subgrid to grid.  COMP: the compensated form (subgrid error plane,
// error-free adds into grid with the errors into grid_lo, which the caller
// folds into grid afterwards).
// The nodes of one work item accumulated into the zeroed subgrid sg (rows of
// SYV complex cells; sgl its error plane when COMP), each warp with its
// vectors at wx / wy.
template <int W, bool COMP, int SYV>
__device__ __forceinline__ void c2_bt_nodes(const WorkItem &it, float2 *sg, float2 *sgl,
                                            const float *__restrict__ xs, const uint32_t *__restrict__ perm,
                                            const float2 *__restrict__ f, const Geom<float> &g, const WinPoly &poly,
                                            float *wx, float *wy, int org0, int org1)
{
  typedef C2<W> P;
  constexpr int CX = P::CX, HP = P::HP, SY = SYV;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int h = lane >> 4, r = lane & 15;

  for (int a = it.start + warp * C2_CHUNK; a < it.end; a += C2_WARPS * C2_CHUNK) {
    const int np = min(C2_CHUNK, it.end - a);
    // ---- set-up: lane j evaluates node j's window
    int col = -1;
    if (lane < np)
      col = c2_setup<W, true>(xs + 2LL * (a + lane), g, org0, org1, poly, f[perm[a + lane]],
                              wx + P::XS * lane, wy + P::YS * lane);
    // the task's nodes are in column order: runs of one column
    const int prevc = __shfl_up_sync(0xffffffffu, col, 1);
    unsigned starts = __ballot_sync(0xffffffffu, lane < np && (lane == 0 || col != prevc));
    __syncwarp();
    const float *xrow = wx + r;
    const float2 *ypair = reinterpret_cast<const float2 *>(wy) + h * HP;
    while (starts) {
      const int s = __ffs(starts) - 1;
      starts &= starts - 1;
      const int e = starts ? __ffs(starts) - 1 : np;
      const int c = __shfl_sync(0xffffffffu, col, s);
      // ---- lane (h, r): row r, y pairs h HP .. h HP + HP - 1 of column c
      float2 ar[HP], ai[HP];
#pragma unroll
      for (int q = 0; q < HP; ++q) ar[q] = ai[q] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int j = s; j < e; ++j) {
        const float xw = xrow[j * P::XS];
        const float2 fj = reinterpret_cast<const float2 *>(wy + j * P::YS)[P::YV / 2];
        const float xr = xw * fj.x, xi = xw * fj.y;
        const float2 hr = make_float2(xr, xr), hi = make_float2(xi, xi);
        const float2 *yp = ypair + j * (P::YS / 2);
#pragma unroll
        for (int q = 0; q < HP; ++q) {
          const float2 w = yp[q];
          ar[q] = __ffma2_rn(w, hr, ar[q]);
          ai[q] = __ffma2_rn(w, hi, ai[q]);
        }
      }
      const int xc = c / C2_SLABS, sl = c - xc * C2_SLABS;
      const int off = (CX * xc + r) * SY + C2_CY * sl + 2 * h * HP;
      if (r < P::ROWS) c2_flush<HP, COMP>(sg + off, ar, ai, P::NPOS - 2 * h * HP, sgl + off);
    }
    __syncwarp();  // the next task's set-up reuses the vectors
  }
}

template <int W, bool COMP = false>
__device__ __forceinline__ void c2_bt_item(const WorkItem &it, float2 *__restrict__ grid,
                                           const float *__restrict__ xs, const uint32_t *__restrict__ perm,
                                           const float2 *__restrict__ f, const Geom<float> &g, const WinPoly &poly,
                                           unsigned char *smem_raw, float2 *__restrict__ grid_lo = nullptr)
{
  typedef C2<W> P;
  constexpr int SY = P::SY;
  float *const base = reinterpret_cast<float *>(smem_raw);
  const int warp = threadIdx.x >> 5;
  float *const wx = base + warp * P::WARP_FLOATS_T;  // real, stride XS
  float *const wy = wx + P::XS * C2_CHUNK;
  float2 *const sg = reinterpret_cast<float2 *>(base + C2_WARPS * P::WARP_FLOATS_T);
  float2 *const sgl = sg + P::EXT * SY;  // error plane (COMP only)

  const int org0 = (it.tile / g.ntile[1]) * C2_TILE, org1 = (it.tile % g.ntile[1]) * C2_TILE;
  for (int i = threadIdx.x; i < (COMP ? 2 : 1) * P::EXT * SY; i += C2_THREADS) sg[i] = make_float2(0.f, 0.f);
  __syncthreads();
  c2_bt_nodes<W, COMP, SY>(it, sg, sgl, xs, perm, f, g, poly, wx, wy, org0, org1);
  __syncthreads();
  for (int idx = threadIdx.x; idx < P::EXT * P::EXT; idx += C2_THREADS) {
    const int rx = idx / P::EXT, ry = idx - rx * P::EXT;
    const float2 v = sg[rx * SY + ry];
    const float2 vl = COMP ? sgl[rx * SY + ry] : make_float2(0.f, 0.f);
    if (v.x != 0.f || v.y != 0.f || vl.x != 0.f || vl.y != 0.f) {
      int p0 = org0 + rx, p1 = org1 + ry;
      while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
      while (p1 >= g.n[1]) p1 -= g.n[1];
      const long long q = (long long)p0 * g.n[1] + p1;
      if (COMP) c2_global_add_comp(grid + q, grid_lo + q, v, vl);
      else global_add_c(grid + q, v);
    }
  }
}

// B of one work item by a CTA of C2_THREADS threads with c2_smem_bytes<W>(false)
// bytes of shared memory at smem_raw; writes f of the item's nodes.
// The padded subgrid of the tile at (org0, org1) into sg (rows of SYV complex
// cells) by plain loads, wrapping around the grid edge.
template <int W, int SYV>
__device__ __forceinline__ void c2_stage_plain(float2 *sg, const float2 *__restrict__ grid, const Geom<float> &g,
                                               int org0, int org1)
{
  constexpr int EXT = C2<W>::EXT;
  for (int idx = threadIdx.x; idx < EXT * EXT; idx += C2_THREADS) {
    const int rx = idx / EXT, ry = idx - rx * EXT;
    int p0 = org0 + rx, p1 = org1 + ry;
    while (p0 >= g.n[0]) p0 -= g.n[0];
    while (p1 >= g.n[1]) p1 -= g.n[1];
    sg[rx * SYV + ry] = grid[(long long)p0 * g.n[1] + p1];
  }
}

// B of the nodes of one work item from the staged subgrid sg (rows of SYV
// complex cells), each warp with its vectors at wx / wy.
template <int W, int SYV>
__device__ __forceinline__ void c2_b_nodes(const WorkItem &it, const float2 *sg, const float *__restrict__ xs,
                                           const uint32_t *__restrict__ perm, float2 *__restrict__ f,
                                           const Geom<float> &g, const WinPoly &poly, float *wx, float *wy,
                                           int org0, int org1)
{
  typedef C2<W> P;
  constexpr int CX = P::CX, HP = P::HP, SY = SYV, EXT = P::EXT;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int h = lane >> 4, r = lane & 15;

  for (int a = it.start + warp * C2_CHUNK; a < it.end; a += C2_WARPS * C2_CHUNK) {
    const int np = min(C2_CHUNK, it.end - a);
    int col = -1;
    if (lane < np)
      col = c2_setup<W, false>(xs + 2LL * (a + lane), g, org0, org1, poly, make_float2(0.f, 0.f),
                               wx + P::XS * lane, wy + P::YS * lane);
    const int prevc = __shfl_up_sync(0xffffffffu, col, 1);
    const unsigned starts = __ballot_sync(0xffffffffu, lane < np && (lane == 0 || col != prevc));
    __syncwarp();
    const float *xrow = wx + r;
    const float2 *ypair = reinterpret_cast<const float2 *>(wy) + h * HP;
    // the row's subgrid cells of the current column: real and imaginary
    // parts of y positions (2k, 2k + 1) as pairs
    float2 gr[HP], gi[HP];
#pragma unroll
    for (int q = 0; q < HP; ++q) gr[q] = gi[q] = make_float2(0.f, 0.f);
    for (int j0 = 0; j0 < np; j0 += 8) {
      float pr[8], pi[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const int j = j0 + jj;
        pr[jj] = pi[jj] = 0.f;
        if (j < np) {
          if ((starts >> j) & 1u) {
            const int c = __shfl_sync(0xffffffffu, col, j);
            const int xc = c / C2_SLABS, sl = c - xc * C2_SLABS;
            // rows past the column (zero x weight) read row 0; positions past
            // the subgrid (zero y weight) read its last cell
            const int row = r < P::ROWS ? CX * xc + r : 0;
            const float2 *src = sg + row * SY;
            const int y0 = C2_CY * sl + 2 * h * HP;
#pragma unroll
            for (int q = 0; q < HP; ++q) {
              const float2 c0 = src[min(y0 + 2 * q, EXT - 1)], c1 = src[min(y0 + 2 * q + 1, EXT - 1)];
              gr[q] = make_float2(c0.x, c1.x);
              gi[q] = make_float2(c0.y, c1.y);
            }
          }
          const float xw = xrow[j * P::XS];
          const float2 *yp = ypair + j * (P::YS / 2);
          float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 0; q < HP; ++q) {
            const float2 w = yp[q];
            sr = __ffma2_rn(w, gr[q], sr);
            si = __ffma2_rn(w, gi[q], si);
          }
          pr[jj] = (sr.x + sr.y) * xw;
          pi[jj] = (si.x + si.y) * xw;
        }
      }
      // sum the lanes' partials: lane L ends with node 4 b4 + 2 b3 + b2 of
      // the eight (b_k bit k of L)
#pragma unroll
      for (int o = 16, nv = 4; o >= 4; o >>= 1, nv >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < nv; ++i) {
          const float sr = up ? pr[i] : pr[i + nv], kr = up ? pr[i + nv] : pr[i];
          const float si = up ? pi[i] : pi[i + nv], ki = up ? pi[i + nv] : pi[i];
          pr[i] = kr + __shfl_xor_sync(0xffffffffu, sr, o);
          pi[i] = ki + __shfl_xor_sync(0xffffffffu, si, o);
        }
      }
      pr[0] += __shfl_xor_sync(0xffffffffu, pr[0], 2);
      pi[0] += __shfl_xor_sync(0xffffffffu, pi[0], 2);
      pr[0] += __shfl_xor_sync(0xffffffffu, pr[0], 1);
      pi[0] += __shfl_xor_sync(0xffffffffu, pi[0], 1);
      const int jn = j0 + ((lane >> 2) & 1) + ((lane >> 3) & 1) * 2 + ((lane >> 4) & 1) * 4;
      if ((lane & 3) == 0 && jn < np) f[perm[a + jn]] = make_float2(pr[0], pi[0]);
    }
    __syncwarp();  // the next task's set-up reuses the vectors
  }
}

template <int W>
__device__ __forceinline__ void c2_b_item(const WorkItem &it, const float2 *__restrict__ grid,
                                          const float *__restrict__ xs, const uint32_t *__restrict__ perm,
                                          float2 *__restrict__ f, const Geom<float> &g, const WinPoly &poly,
                                          unsigned char *smem_raw)
{
  typedef C2<W> P;
  float *const base = reinterpret_cast<float *>(smem_raw);
  const int warp = threadIdx.x >> 5;
  float *const wx = base + warp * P::WARP_FLOATS_B;  // real, stride XS
  float *const wy = wx + P::XS * C2_CHUNK;
  float2 *const sg = reinterpret_cast<float2 *>(base + C2_WARPS * P::WARP_FLOATS_B);
  const int org0 = (it.tile / g.ntile[1]) * C2_TILE, org1 = (it.tile % g.ntile[1]) * C2_TILE;
  c2_stage_plain<W, P::SY>(sg, grid, g, org0, org1);
  __syncthreads();
  c2_b_nodes<W, P::SY>(it, sg, xs, perm, f, g, poly, wx, wy, org0, org1);
}

}  // namespace gb
