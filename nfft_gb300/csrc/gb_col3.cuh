// gb_col3.cuh -- single-precision 3-D B^T (adjoint spreading) by z-columns
// and 3-D B (interpolation) by sub-cell units: the hot kernels of the 3-D
// transform.
//
// Both evaluate the Kaiser-Bessel window on the fly from its per-tap
// polynomial form (gb_window.cpp): degree-9 Horner in the node's fractional
// grid offset, single-precision FMAs with the coefficients as kernel
// parameters.
//
// B^T -- reference nfft_adjoint_3d_B (nfft.c:5126-5384) with its blockwise
// scatter (nfft.c:4289-4388): g[l mod n] += phi_0 phi_1 phi_2 f_j over the
// (2m+2)^3 window of every node.
//
// Node set-up sorts the nodes by (8^3 tile, 2x2 column of the tile's x/y
// cells, window start along z), so the nodes of one column sit together,
// ordered by their z window start z0 in [0, 8).  A column's nodes all touch
// the same W+1 by W+1 (x, y) rows of the tile's padded subgrid, over z in
// [0, 8 + W - 1).
//
// A CTA takes one work item (a tile and a range of its nodes) and keeps the
// tile's padded subgrid in shared memory as interleaved complex values.  A
// warp takes a column chunk (at most 32 nodes of one column):
//  * lane j evaluates node j's window into per-warp vectors: x scaled by f_j
//    (complex), y, and z at its offset in an aligned pair; its node record
//    and f_j (read through the node permutation, the one scattered read of
//    the adjoint) were loaded while the warp's previous chunk computed;
//  * lanes own (x, y) rows of the column (two per lane) and hold all
//    8 + W - 1 z values of a row as complex accumulators in registers; for the
//    nodes whose window starts at z0 (a compile-time case, eight of them)
//    each row takes exactly W paired FMAs (fma.rn.f32x2 of the sm_100
//    family: real and imaginary at once);
//  * each row is added to the shared subgrid once per chunk.  Single-precision
//    atomic adds on shared memory are compare-and-swap loops, one value at a
//    time; here a row's complex cells are read, summed and swapped as 64-bit
//    words, all of them before the first result is checked, and only the
//    rare cell another warp changed in between is added again;
//  * the subgrid goes to the global grid once per work item: a tile whose
//    padded box lies inside the grid is copied into a dense box in the
//    warps' (then idle) scratch and added to the grid by one TMA add-reduce
//    (cp.reduce.async.bulk.tensor); a tile whose box wraps around the grid
//    edge adds its cells with vector reductions.
#pragma once

#include "gb_b3group.cuh"  // warp_transpose_reduce
#include "gb_internal.h"
#include "gb_tma.cuh"

namespace gb {

// bounded TMA waits that gave up (read and cleared by read_wait_timeouts);
// this header is compiled into one unit (gb_b3group.cu)
__device__ unsigned long long g_tma_wait_timeouts;

static constexpr int C3_THREADS = 256;
static constexpr int C3_WARPS = C3_THREADS / 32;
static constexpr int C3_CHUNK = 32;  // nodes per column chunk (one per lane at set-up)

template <int W>
struct C3 {
  static constexpr int EXT = 8 + W - 1;                      // padded subgrid edge
  static constexpr int BOX = W + 1;                          // rows per dimension of a column
  static constexpr int BOXP = (BOX + 3) / 4 * 4;             // padded x / y vector length
  static constexpr int ROWS = BOX * BOX;                     // (x, y) rows of a column
  static constexpr int RPL = 2;                              // rows a lane holds at once
  static constexpr int RITER = (ROWS + 32 * RPL - 1) / (32 * RPL);
  static constexpr int ZP = (W + 2 + 3) / 4 * 4;            // z taps with a parity shift, padded
  static constexpr int NPAIR = (EXT + 1) / 2;                // z pairs of a row's accumulators
  // per-warp scratch (floats): x scaled by f [CHUNK][BOXP] complex, y
  // [CHUNK][BOXP], z [CHUNK][ZP] shifted by the parity of the window start
  static constexpr int WXF = 0;
  static constexpr int WY = WXF + 2 * BOXP * C3_CHUNK;
  static constexpr int WZ = WY + BOXP * C3_CHUNK;
  static constexpr int WARP_FLOATS = WZ + ZP * C3_CHUNK;
  static constexpr int INTS = 17 + 1;                        // column starts, task counter
  static_assert(BOXP > BOX, "x / y vectors need one zero slot past the column");
  static_assert(W % 2 == 0, "even window width");
};

template <int W>
inline size_t c3_smem_bytes(const Geom<float> &g)
{
  typedef C3<W> P;
  return (size_t)C3_WARPS * P::WARP_FLOATS * sizeof(float) + (size_t)P::EXT * g.sx2 * sizeof(float2)
         + P::INTS * sizeof(int);
}

__device__ __forceinline__ unsigned long long f2_bits(float2 v)
{
  union {
    float2 f;
    unsigned long long u;
  } c;
  c.f = v;
  return c.u;
}

// Starts a bulk copy of the 16-byte aligned interior of [p, p + bytes) from
// global memory into L2 (cp.async.bulk.prefetch, sm_90 and later): the
// work item's node data arrive while the CTA stages its subgrid.
__device__ __forceinline__ void c3_prefetch_l2(const void *p, long long bytes)
{
  const unsigned long long a = (unsigned long long)p;
  const unsigned long long b = (a + 15) & ~15ull, e = (a + (unsigned long long)bytes) & ~15ull;
  for (unsigned long long q = b; q < e; q += (1u << 20)) {
    const unsigned n = (unsigned)((e - q) < (1u << 20) ? (e - q) : (1u << 20));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q), "r"(n) : "memory");
  }
}

// Adds v[z] to the interleaved complex cells p[z], z < N, ZB cells at a time
// (blocks wholly outside the warp-uniform range [z1, z2) hold zeros and are
// skipped):
// every cell of a block is read, summed (one paired add) and offered by one
// 64-bit compare-and-swap before any result is checked; a cell whose swap
// found a value changed by another warp in between is added again with the
// atomic add of each component.
template <int N, int NP, int ZB>
__device__ __forceinline__ void c3_flush_row(float2 *p, const float2 (&vr)[NP], const float2 (&vi)[NP], int z1,
                                             int z2)
{
  static_assert(N <= 2 * NP, "cells past the accumulators");
  volatile float2 *vp = p;
#pragma unroll
  for (int z0 = 0; z0 < N; z0 += ZB) {
    if (z0 + ZB <= z1 || z0 >= z2) continue;
    float2 cur[ZB], v[ZB];
#pragma unroll
    for (int e = 0; e < ZB; ++e)
      if (z0 + e < N) {
        const int z = z0 + e;
        const volatile float2 &c = vp[z];
        cur[e] = make_float2(c.x, c.y);
        v[e] = make_float2((z & 1) ? vr[z >> 1].y : vr[z >> 1].x, (z & 1) ? vi[z >> 1].y : vi[z >> 1].x);
      }
    unsigned miss = 0;
#pragma unroll
    for (int e = 0; e < ZB; ++e) {
      if (z0 + e < N) {
        const unsigned long long old = f2_bits(cur[e]);
        const unsigned long long want = f2_bits(__fadd2_rn(cur[e], v[e]));
        if (atomicCAS(reinterpret_cast<unsigned long long *>(p + z0 + e), old, want) != old) miss |= 1u << e;
      }
    }
    if (miss) {
#pragma unroll
      for (int e = 0; e < ZB; ++e)
        if (z0 + e < N && (miss >> e) & 1u) {
          atomicAdd(&p[z0 + e].x, v[e].x);
          atomicAdd(&p[z0 + e].y, v[e].y);
        }
    }
  }
}

template <int W>
__global__ void __launch_bounds__(C3_THREADS, 2) k_bt3_col(const WorkItem *__restrict__ items,
                                                            float2 *__restrict__ grid,
                                                            const float4 *__restrict__ rec,
                                                            const uint16_t *__restrict__ cst,
                                                            const uint32_t *__restrict__ perm,
                                                            const float2 *__restrict__ f, Geom<float> g,
                                                            WinPoly poly, const __grid_constant__ CUtensorMap gmap,
                                                            int use_tma)
{
  typedef C3<W> P;
  constexpr int EXT = P::EXT, BOXP = P::BOXP, RPL = P::RPL;
  extern __shared__ __align__(128) unsigned char c3_smem[];
  float *const base = reinterpret_cast<float *>(c3_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *const wsc = base + warp * P::WARP_FLOATS;
  float2 *const wxf = reinterpret_cast<float2 *>(wsc + P::WXF);
  float *const wy = wsc + P::WY;
  float *const wz = wsc + P::WZ;
  float2 *const sg = reinterpret_cast<float2 *>(base + C3_WARPS * P::WARP_FLOATS);
  int *const cstart = reinterpret_cast<int *>(sg + EXT * g.sx2);
  int *const taskctr = cstart + 17;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  {
    int rem = it.tile;
#pragma unroll
    for (int t = 2; t >= 0; --t) {
      org[t] = (rem % g.ntile[t]) * 8;
      rem /= g.ntile[t];
    }
  }
  if (threadIdx.x == 0) {
    c3_prefetch_l2(rec + it.start, 16LL * (it.end - it.start));
    c3_prefetch_l2(perm + it.start, 4LL * (it.end - it.start));
  }
  for (int i = threadIdx.x; i < EXT * g.sx2; i += C3_THREADS) sg[i] = make_float2(0.f, 0.f);
  // column boundaries of the item (node set-up): cstart[c] = first node of column c
  if (threadIdx.x < 17) cstart[threadIdx.x] = cst[17LL * blockIdx.x + threadIdx.x];
  if (threadIdx.x == 0) *taskctr = 0;
  __syncthreads();

  // chunks per column (lanes 0..15), inclusive scan -> task -> column map
  int nch = 0;
  if (lane < 16) nch = (cstart[lane + 1] - cstart[lane] + C3_CHUNK - 1) / C3_CHUNK;
  int incl = nch;
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int ntask = __shfl_sync(0xffffffffu, incl, 15);

  // task -> (column, first node, node count)
  auto locate = [&](int task, int &c, int &a, int &np) {
    c = __popc(__ballot_sync(0xffffffffu, lane < 16 && incl <= task));
    const int prev = __shfl_sync(0xffffffffu, incl, (c + 31) & 31);
    const int before = c > 0 ? prev : 0;
    const int clen = cstart[c + 1] - cstart[c];
    const int nchunk = (clen + C3_CHUNK - 1) / C3_CHUNK;
    const int k = task - before, qn = clen / nchunk, rq = clen - qn * nchunk;
    a = it.start + cstart[c] + k * qn + min(k, rq);
    np = qn + (k < rq ? 1 : 0);
  };
  int task = 0;
  if (lane == 0) task = atomicAdd(taskctr, 1);
  task = __shfl_sync(0xffffffffu, task, 0);
  int c = 0, a = 0, np = 0;
  float4 rn = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 fn = make_float2(0.f, 0.f);
  if (task < ntask) {
    locate(task, c, a, np);
    if (lane < np) {
      rn = rec[a + lane];
      fn = f[perm[a + lane]];
    }
  }
  for (;;) {
    if (task >= ntask) break;
    const int s0 = c >> 2, s1 = c & 3;
    const float4 r = rn;
    const float2 fj = fn;
    const int np_cur = np;
    // the next task's node data, loaded while this one computes
    int ntaskid = 0;
    if (lane == 0) ntaskid = atomicAdd(taskctr, 1);
    ntaskid = __shfl_sync(0xffffffffu, ntaskid, 0);
    int c2 = 0, a2 = 0, np2 = 0;
    if (ntaskid < ntask) {
      locate(ntaskid, c2, a2, np2);
      if (lane < np2) {
        rn = rec[a2 + lane];
        fn = f[perm[a2 + lane]];
      }
    }

    // ---- set-up: lane j evaluates node j's window
    int z0 = 8;
    if (lane < np_cur) {
      const int loc = __float_as_int(r.w);
      float v[W];
      // x, scaled by f_j, at the node's offset in the column's box
      const int ox = (loc & 7) - 2 * s0;
      kb_poly_taps_sym<W>(r.x, poly.c[0], v);
      {
        float4 *dst = reinterpret_cast<float4 *>(wxf + lane * BOXP);
#pragma unroll
        for (int q = 0; q < BOXP / 2; ++q) {
          float e[4];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int b = 2 * q + h;
            float val = 0.f;
            if (b < W && ox == 0) val = v[b];
            if (b >= 1 && b - 1 < W && ox == 1) val = v[b - 1];
            e[2 * h] = val * fj.x;
            e[2 * h + 1] = val * fj.y;
          }
          dst[q] = make_float4(e[0], e[1], e[2], e[3]);
        }
      }
      const int oy = ((loc >> 3) & 7) - 2 * s1;
      kb_poly_taps_sym<W>(r.y, poly.c[1], v);
      {
        float4 *dst = reinterpret_cast<float4 *>(wy + lane * BOXP);
#pragma unroll
        for (int q = 0; q < BOXP / 4; ++q) {
          float e[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int b = 4 * q + h;
            float val = 0.f;
            if (b < W && oy == 0) val = v[b];
            if (b >= 1 && b - 1 < W && oy == 1) val = v[b - 1];
            e[h] = val;
          }
          dst[q] = make_float4(e[0], e[1], e[2], e[3]);
        }
      }
      z0 = loc >> 6;
      kb_poly_taps_sym<W>(r.z, poly.c[2], v);
      {
        // taps at the node's z offset within its aligned pair: a window
        // starting at odd z0 begins in the second half of a pair
        const int oz = z0 & 1;
        float4 *dst = reinterpret_cast<float4 *>(wz + lane * P::ZP);
#pragma unroll
        for (int q = 0; q < P::ZP / 4; ++q) {
          float e[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int b = 4 * q + h;
            float val = 0.f;
            if (b < W && oz == 0) val = v[b];
            if (b >= 1 && b - 1 < W && oz == 1) val = v[b - 1];
            e[h] = val;
          }
          dst[q] = make_float4(e[0], e[1], e[2], e[3]);
        }
      }
    }
    // runs of equal z0 (the chunk is sorted by z0): rs[z] = first lane with z0 >= z
    int rs[9];
#pragma unroll
    for (int z = 0; z <= 8; ++z) rs[z] = __popc(__ballot_sync(0xffffffffu, z0 < z));
    // z range the chunk touches: first z0 .. last z0 + W
    const int zlo = __shfl_sync(0xffffffffu, z0, 0), zhi = __shfl_sync(0xffffffffu, z0, np_cur - 1) + W;
    __syncwarp();

#pragma unroll 1
    for (int ri = 0; ri < P::RITER; ++ri) {
      int bx[RPL], by[RPL];
      bool ok[RPL];
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        const int row = lane + 32 * (ri * RPL + q);
        ok[q] = row < P::ROWS;
        // rows past the column read the zero slot BOXP - 1 of the x vector
        bx[q] = ok[q] ? row / P::BOX : BOXP - 1;
        by[q] = ok[q] ? row - (row / P::BOX) * P::BOX : 0;
      }
      // real and imaginary accumulators of the row's z values, as aligned pairs
      float2 ar[RPL][P::NPAIR], ai[RPL][P::NPAIR];
#pragma unroll
      for (int q = 0; q < RPL; ++q)
#pragma unroll
        for (int z = 0; z < P::NPAIR; ++z) ar[q][z] = ai[q][z] = make_float2(0.f, 0.f);
#pragma unroll
      for (int zz = 0; zz < 8; ++zz) {
        // window start zz: taps in pairs zz/2 .. zz/2 + npr - 1
        const int b = zz >> 1, npr = (zz & 1) ? W / 2 + 1 : W / 2;
#pragma unroll 1
        for (int j = rs[zz]; j < rs[zz + 1]; ++j) {
          // 8-byte broadcast reads: a warp-wide 16-byte read of one address
          // costs four shared-memory wavefronts, an 8-byte read one
          float2 w[P::ZP / 2];
          const float2 *src = reinterpret_cast<const float2 *>(wz + j * P::ZP);
#pragma unroll
          for (int k = 0; k < P::ZP / 2; ++k)
            if (k < npr) w[k] = src[k];
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const float2 xf = wxf[j * BOXP + bx[q]];
            const float yv = wy[j * BOXP + by[q]];
            const float hr = xf.x * yv, hi = xf.y * yv;
            const float2 hr2 = make_float2(hr, hr), hi2 = make_float2(hi, hi);
#pragma unroll
            for (int k = 0; k < W / 2 + 1; ++k)
              if (k < npr) {
                ar[q][b + k] = __ffma2_rn(w[k], hr2, ar[q][b + k]);
                ai[q][b + k] = __ffma2_rn(w[k], hi2, ai[q][b + k]);
              }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < RPL; ++q)
        if (ok[q]) c3_flush_row<EXT, P::NPAIR, 6>(sg + (2 * s0 + bx[q]) * g.sx2 + (2 * s1 + by[q]) * g.sy2, ar[q],
                                                  ai[q], zlo, zhi);
    }
    __syncwarp();
    task = ntaskid;
    c = c2;
    a = a2;
    np = np2;
  }
  __syncthreads();
  // ---- write-back.  A tile whose padded box lies inside the grid: the box
  // goes densely (rows of ZB complex values, the last one zero where EXT is
  // odd) into the warps' scratch, then one TMA add-reduce adds it to the grid.
  constexpr int ZB = (EXT + 1) & ~1;
  static_assert((size_t)EXT * EXT * ZB * 2 <= (size_t)C3_WARPS * P::WARP_FLOATS,
                "the dense padded tile fits in the warps' scratch");
  if (use_tma && org[0] + EXT <= g.n[0] && org[1] + EXT <= g.n[1] && org[2] + EXT <= g.n[2] &&
      (smem_u32(base) & 127u) == 0) {
    float2 *const stg = reinterpret_cast<float2 *>(base);
    for (int r = threadIdx.x; r < EXT * EXT; r += C3_THREADS) {
      const int c0 = r / EXT, c1 = r - c0 * EXT;
      const float2 *src = sg + c0 * g.sx2 + c1 * g.sy2;
      float4 *dst = reinterpret_cast<float4 *>(stg + r * ZB);
#pragma unroll
      for (int z = 0; z < ZB; z += 2) {
        const float2 a = src[z];
        const float2 b = z + 1 < EXT ? src[z + 1] : make_float2(0.f, 0.f);
        dst[z >> 1] = make_float4(a.x, a.y, b.x, b.y);
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_reduce_add_3d(&gmap, stg, 2 * org[2], org[1], org[0]);
      bulk_commit();
      bulk_wait_read_all();  // the scratch stays allocated until the copy has read it
    }
    return;
  }
  // a tile whose padded box wraps around the grid edge: one vector reduction
  // per non-zero cell
  for (int idx = threadIdx.x; idx < EXT * EXT * EXT; idx += C3_THREADS) {
    const int c2 = idx % EXT, r = idx / EXT;
    const int c1 = r % EXT, c0 = r / EXT;
    const float2 v = sg[c0 * g.sx2 + c1 * g.sy2 + c2];
    if (v.x == 0.f && v.y == 0.f) continue;
    int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
    while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
    while (p1 >= g.n[1]) p1 -= g.n[1];
    while (p2 >= g.n[2]) p2 -= g.n[2];
    global_add_c(grid + ((long long)p0 * g.n[1] + p1) * g.n[2] + p2, v);
  }
}

// ---------------------------------------------------------------------------
// B -- 3-D interpolation by sub-cell units: f_j = sum phi_0 phi_1 phi_2 g over
// the window of every node (reference nfft_trafo_3d_B, nfft.c:4687-4914, with
// nfft_trafo_3d_compute, nfft.c:4020-4265).
//
// The nodes of a 2x2x2 sub-cell of a tile share one (W+1)^3 box of the padded
// subgrid.  A CTA stages its tile's padded subgrid in shared memory as real
// and imaginary planes (one TMA copy of the interleaved box, de-interleaved in
// shared memory, for a tile whose padded box lies inside the grid; plain loads
// for one that wraps around the grid edge), finds where each of the tile's 64
// sub-cells starts in the
// item's sorted node range, and its warps take units (at most S3_PM nodes of
// one sub-cell, a sub-cell's nodes split evenly) from a shared counter:
//  * lanes evaluate the unit's windows (one lane per node and dimension) into
//    zero-padded per-warp vectors at each node's offset in the box;
//  * lanes own two (x, y) box rows at a time and hold their W+1 z values in
//    registers; nodes go in pairs, so the paired z FMAs (fma.rn.f32x2) of two
//    nodes and two rows are independent chains;
//  * the per-lane partial sums of the unit's nodes meet in one butterfly
//    transpose-reduction.
static constexpr int S3_PM = 16;  // nodes per unit

template <int W>
struct S3 {
  static constexpr int EXT = 8 + W - 1;
  static constexpr int BOX = W + 1;
  static constexpr int BOXP = (BOX + 3) / 4 * 4;
  static constexpr int ROWS = BOX * BOX;
  static constexpr int RPL = 2;
  static constexpr int RITER = (ROWS + 32 * RPL - 1) / (32 * RPL);
  static constexpr int WARP_FLOATS = 3 * S3_PM * BOXP;  // wx, wy, wz [S3_PM][BOXP]
  static constexpr int INTS = 65 + 1;                   // sub-cell starts, task counter
  // the TMA box of the padded subgrid: rows of ZB (even: 16-byte rows) complex
  // cells, EXTY rows per x-plane -- EXT rounded up to 3 mod 8, so that the
  // row-per-thread de-interleave reads consecutive rows from different banks
  static constexpr int ZB = (EXT + 1) & ~1;
  static constexpr int EXTY = EXT + ((11 - EXT % 8) % 8);
  static_assert(BOXP > BOX, "the x vector needs one zero slot past the box");
};

// warp scratch | real and imaginary planes | ints | (128-byte aligned) TMA
// box | its barrier
template <int W>
__host__ __device__ inline size_t s3_box_offset(const Geom<float> &g)
{
  typedef S3<W> P;
  const size_t b =
      ((size_t)C3_WARPS * P::WARP_FLOATS + 2 * (size_t)P::EXT * g.sx) * sizeof(float) + P::INTS * sizeof(int);
  return (b + 127) / 128 * 128;
}

template <int W>
__host__ __device__ inline size_t s3_smem_bytes(const Geom<float> &g)
{
  typedef S3<W> P;
  return s3_box_offset<W>(g) + (size_t)P::EXT * P::EXTY * P::ZB * sizeof(float2) + sizeof(unsigned long long);
}

template <int W>
__global__ void __launch_bounds__(C3_THREADS, 2) k_b3_cell(const WorkItem *__restrict__ items,
                                                            const float2 *__restrict__ grid,
                                                            const float4 *__restrict__ rec,
                                                            const uint16_t *__restrict__ sst,
                                                            const uint32_t *__restrict__ perm,
                                                            float2 *__restrict__ f, Geom<float> g,
                                                            WinPoly poly, const __grid_constant__ CUtensorMap gmap,
                                                            int use_tma)
{
  typedef S3<W> P;
  constexpr int EXT = P::EXT, BOX = P::BOX, BOXP = P::BOXP, RPL = P::RPL, PM = S3_PM;
  extern __shared__ __align__(128) unsigned char c3_smem[];
  float *const base = reinterpret_cast<float *>(c3_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *const wx = base + warp * P::WARP_FLOATS;
  float *const wy = wx + PM * BOXP;
  float *const wz = wy + PM * BOXP;
  float *const sre = base + C3_WARPS * P::WARP_FLOATS;
  float *const sim = sre + EXT * g.sx;
  int *const sstart = reinterpret_cast<int *>(sim + EXT * g.sx);
  int *const taskctr = sstart + 65;

  const WorkItem it = items[blockIdx.x];
  int org[3];
  {
    int rem = it.tile;
#pragma unroll
    for (int t = 2; t >= 0; --t) {
      org[t] = (rem % g.ntile[t]) * 8;
      rem /= g.ntile[t];
    }
  }
  if (threadIdx.x == 0) {
    c3_prefetch_l2(rec + it.start, 16LL * (it.end - it.start));
    c3_prefetch_l2(perm + it.start, 4LL * (it.end - it.start));
  }
  // the padded subgrid: one TMA copy into the box where the box lies inside
  // the grid (de-interleaved into the planes below), plain loads where it
  // wraps around the grid edge
  constexpr int ZB = P::ZB, EXTY = P::EXTY;
  const size_t off = s3_box_offset<W>(g);
  float2 *const stg = reinterpret_cast<float2 *>(c3_smem + off);
  unsigned long long *const bar = reinterpret_cast<unsigned long long *>(c3_smem + off + (size_t)EXT * EXTY * ZB * sizeof(float2));
  const bool tma = use_tma && org[0] + EXT <= g.n[0] && org[1] + EXT <= g.n[1] && org[2] + EXT <= g.n[2] &&
                   (smem_u32(stg) & 127u) == 0;
  if (threadIdx.x == 0 && tma) {
    mbar_init(bar, 1);
    mbar_expect_tx(bar, (unsigned)(EXT * EXTY * ZB * sizeof(float2)));
    tma_load_3d(stg, &gmap, 2 * org[2], org[1], org[0], bar);
  }
  if (!tma) {
    // several grid loads in flight per thread
#pragma unroll 4
    for (int idx = threadIdx.x; idx < EXT * EXT * EXT; idx += C3_THREADS) {
      const int c2 = idx % EXT, r = idx / EXT;
      const int c1 = r % EXT, c0 = r / EXT;
      int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
      while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
      while (p1 >= g.n[1]) p1 -= g.n[1];
      while (p2 >= g.n[2]) p2 -= g.n[2];
      const float2 v = grid[((long long)p0 * g.n[1] + p1) * g.n[2] + p2];
      const int si = c0 * g.sx + c1 * g.sy + c2;
      sre[si] = v.x;
      sim[si] = v.y;
    }
  }
  // the unused node slots of the weight vectors must hold finite values
  for (int i = lane; i < P::WARP_FLOATS; i += 32) wx[i] = 0.f;
  // sub-cell boundaries of the item (node set-up): sstart[s] = first node of sub-cell s
  if (threadIdx.x < 65) sstart[threadIdx.x] = sst[65LL * blockIdx.x + threadIdx.x];
  if (threadIdx.x == 0) *taskctr = 0;
  __syncthreads();
  if (tma) {
    // a bounded wait: a copy that never arrives costs this tile, not a hang
    const bool ok = mbar_wait(bar, 0, TMA_WAIT_POLLS);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicAdd(&g_tma_wait_timeouts, 1ull);
      return;
    }
    // de-interleave the box into the real and imaginary planes
    for (int r = threadIdx.x; r < EXT * EXT; r += C3_THREADS) {
      const int c0 = r / EXT, c1 = r - c0 * EXT;
      const float2 *src = stg + (c0 * EXTY + c1) * ZB;
      const int si = c0 * g.sx + c1 * g.sy;
#pragma unroll
      for (int z = 0; z < EXT; ++z) {
        const float2 v = src[z];
        sre[si + z] = v.x;
        sim[si + z] = v.y;
      }
    }
    __syncthreads();
  }

  // units per sub-cell: lane l holds sub-cells 2l and 2l+1
  const int l0 = sstart[2 * lane + 1] - sstart[2 * lane], l1 = sstart[2 * lane + 2] - sstart[2 * lane + 1];
  const int n0 = (l0 + PM - 1) / PM, n1 = (l1 + PM - 1) / PM;
  int incl = n0 + n1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int ntask = __shfl_sync(0xffffffffu, incl, 31);

  for (;;) {
    int task = 0;
    if (lane == 0) task = atomicAdd(taskctr, 1);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= ntask) break;
    const int L = __popc(__ballot_sync(0xffffffffu, incl <= task));  // lane holding the task
    const int excl = incl - n0 - n1;
    const bool second = task - excl >= n0;
    const int s_l = 2 * lane + (second ? 1 : 0);
    const int k_l = task - excl - (second ? n0 : 0);
    const int nu_l = second ? n1 : n0;
    const int len_l = second ? l1 : l0;
    const int s = __shfl_sync(0xffffffffu, s_l, L);
    const int k = __shfl_sync(0xffffffffu, k_l, L);
    const int nu = __shfl_sync(0xffffffffu, nu_l, L);
    const int len = __shfl_sync(0xffffffffu, len_l, L);
    // the sub-cell's nodes split evenly into nu units
    const int q = len / nu, rq = len - q * nu;
    const int u0 = it.start + sstart[s] + k * q + min(k, rq);
    const int np = q + (k < rq ? 1 : 0);
    const int b0 = (s >> 4) * 2, b1 = ((s >> 2) & 3) * 2, b2 = (s & 3) * 2;

    // ---- windows: lane k < 3 np takes node k / 3, dimension k mod 3
    for (int kk = lane; kk < 3 * np; kk += 32) {
      const int j = kk / 3, t = kk - 3 * j;
      const float *rj = reinterpret_cast<const float *>(rec + u0 + j);
      const float sj = rj[t];
      const int loc = (__float_as_int(rj[3]) >> (3 * t)) & 7;
      const int o = loc - (t == 0 ? b0 : (t == 1 ? b1 : b2));
      float v[W];
      if (poly.same) kb_poly_taps_sym<W>(sj, poly.c[0], v);
      else kb_poly_taps_sym<W>(sj, poly.c[t], v);
      float *dst = wx + (t * PM + j) * BOXP;
      float e[BOXP];
#pragma unroll
      for (int b = 0; b < BOXP; ++b) {
        float val = 0.f;
        if (b < W && o == 0) val = v[b];
        if (b >= 1 && b - 1 < W && o == 1) val = v[b - 1];
        e[b] = val;
      }
#pragma unroll
      for (int b = 0; b < BOXP; b += 4) *reinterpret_cast<float4 *>(dst + b) = make_float4(e[b], e[b + 1], e[b + 2], e[b + 3]);
    }
    __syncwarp();

    const int sbase = b0 * g.sx + b1 * g.sy + b2;
    float acc[2 * PM];
#pragma unroll
    for (int j = 0; j < 2 * PM; ++j) acc[j] = 0.f;
#pragma unroll 1
    for (int ri = 0; ri < P::RITER; ++ri) {
      int wbx[RPL], by[RPL];
      float gr[RPL][BOX], gi[RPL][BOX];
#pragma unroll
      for (int qq = 0; qq < RPL; ++qq) {
        const int row = lane + 32 * (ri * RPL + qq);
        const bool ok = row < P::ROWS;
        const int rr = ok ? row : 0;
        const int bx = rr / BOX;
        by[qq] = rr - bx * BOX;
        wbx[qq] = ok ? bx : BOXP - 1;  // rows past the box take the zero slot of the x vector
        const float *pr = sre + sbase + bx * g.sx + by[qq] * g.sy;
        const float *pi = sim + sbase + bx * g.sx + by[qq] * g.sy;
        // row starts are even (even plane strides, even sub-cell z origin):
        // pairs of z values load as 8-byte words
#pragma unroll
        for (int z = 0; z + 1 < BOX; z += 2) {
          const float2 a = *reinterpret_cast<const float2 *>(pr + z);
          const float2 b = *reinterpret_cast<const float2 *>(pi + z);
          gr[qq][z] = a.x;
          gr[qq][z + 1] = a.y;
          gi[qq][z] = b.x;
          gi[qq][z + 1] = b.y;
        }
        if (BOX & 1) {
          gr[qq][BOX - 1] = pr[BOX - 1];
          gi[qq][BOX - 1] = pi[BOX - 1];
        }
      }
#pragma unroll
      for (int jb = 0; jb < PM; jb += 2) {
        if (jb < np) {
#pragma unroll
          for (int j = jb; j < jb + 2; ++j) {
            // 8-byte broadcast reads (one shared-memory wavefront each)
            float wzj[BOXP];
#pragma unroll
            for (int b = 0; b < BOX; b += 2) {
              const float2 t = *reinterpret_cast<const float2 *>(wz + j * BOXP + b);
              wzj[b] = t.x;
              wzj[b + 1] = t.y;
            }
#pragma unroll
            for (int qq = 0; qq < RPL; ++qq) {
              float2 r2 = make_float2(0.f, 0.f), i2 = make_float2(0.f, 0.f);
#pragma unroll
              for (int z = 0; z + 1 < BOX; z += 2) {
                const float2 w2 = make_float2(wzj[z], wzj[z + 1]);
                r2 = __ffma2_rn(w2, make_float2(gr[qq][z], gr[qq][z + 1]), r2);
                i2 = __ffma2_rn(w2, make_float2(gi[qq][z], gi[qq][z + 1]), i2);
              }
              float tr = r2.x + r2.y, ti = i2.x + i2.y;
              if (BOX & 1) {
                tr = fmaf(wzj[BOX - 1], gr[qq][BOX - 1], tr);
                ti = fmaf(wzj[BOX - 1], gi[qq][BOX - 1], ti);
              }
              const float wxy = wx[j * BOXP + wbx[qq]] * wy[j * BOXP + by[qq]];
              acc[2 * j] = fmaf(wxy, tr, acc[2 * j]);
              acc[2 * j + 1] = fmaf(wxy, ti, acc[2 * j + 1]);
            }
          }
        }
      }
    }
    if (np > 8) warp_transpose_reduce<float, 32>(acc);
    else warp_transpose_reduce<float, 16>(acc);
    const float re = __shfl_sync(0xffffffffu, acc[0], (2 * lane) & 31);
    const float im = __shfl_sync(0xffffffffu, acc[0], (2 * lane + 1) & 31);
    if (lane < np) f[perm[u0 + lane]] = make_float2(re, im);
    __syncwarp();
  }
}

}  // namespace gb
