// gb_col3.cuh -- single-precision 3-D B^T (adjoint spreading) by z-column
// segments and 3-D B (interpolation) by z-column segments or by sub-cell
// units: the hot kernels of the 3-D transform.
//
// Both evaluate the Kaiser-Bessel window on the fly from its per-tap
// polynomial form (gb_window.cpp): degree-9 Horner in the node's fractional
// grid offset, single-precision FMAs with the coefficients as kernel
// parameters, taps l and W-1-l from one even/odd split.
//
// Both keep a tile's padded subgrid in shared memory in the layout of one TMA
// box of the grid: EXT x-planes of EXTY rows of ZB interleaved complex cells
// (EXT = 8 + W - 1 cells used per dimension; ZB = EXT rounded up to even, so
// that rows are 16-byte multiples; EXTY = EXT rounded up to 3 mod 8, so that
// consecutive rows of a plane fall in different banks).  The cells past EXT
// stay zero.
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
// A CTA takes one work item (a tile and a range of its nodes) and zeroes the
// tile's padded subgrid.  Its warps work in pairs; a pair takes column
// segments (at most C3_SEGN nodes of one column, a long column's nodes split
// evenly) from a shared counter:
//  * the lanes of a pair own the column's rows, two per lane in each warp
//    (row = lane + 32 (2 h + q) for warp h of the pair), and hold all
//    8 + W - 1 z values of a row as real and imaginary accumulator pairs in
//    registers for the whole segment;
//  * the segment goes in chunks of 32 nodes: lane j of one warp evaluates
//    node j's x window scaled by f_j (complex), lane j of the other its y
//    window and its z window at the parity of its start, into the pair's
//    node records in shared memory; the next chunk's node records and f_j
//    (read through the node permutation, the one scattered read of the
//    adjoint) are loaded while the current chunk computes;
//  * for the nodes whose window starts at z0 (a compile-time case, eight of
//    them) each row takes exactly W or W + 2 paired FMAs (fma.rn.f32x2 of the
//    sm_100 family: two z values at once);
//  * at the end of a segment each row is added to the shared subgrid two
//    cells at a time (16-byte read, two paired adds, 16-byte store), one pair
//    at a time under the CTA's flush lock: segments end thousands of cycles
//    apart, so the lock is rarely contended, and a plain read-add-write moves
//    about a third less shared-memory data than a compare-and-swap would
//    (the lock's spin is bounded: a pair that gives up counts a time-out and
//    skips its flush, so a broken lock shows as wrong sums and a non-zero
//    nfft_gb_tma_wait_timeouts, never as a hang);
//  * the subgrid goes to the global grid once per work item: a tile whose box
//    lies inside the grid by one TMA add-reduce (cp.reduce.async.bulk.tensor)
//    straight from the subgrid; a tile whose box wraps around the grid edge
//    adds its cells with vector reductions.
#pragma once

#include "gb_b3group.cuh"  // warp_transpose_reduce
#include "gb_internal.h"
#include "gb_tma.cuh"

namespace gb {

// bounded waits that gave up, on TMA copies or on B^T's flush lock (read and
// cleared by read_wait_timeouts); this header is compiled into one unit
// (gb_b3group.cu)
__device__ unsigned long long g_tma_wait_timeouts;

static constexpr int C3_THREADS = 256;
static constexpr int C3_WARPS = C3_THREADS / 32;
static constexpr int C3_PAIRS = C3_WARPS / 2;
static constexpr int C3_CHUNK = 32;    // nodes per chunk (one per lane at set-up)
static constexpr int C3_SEGN = 256;    // nodes per column segment at most

// the padded subgrid of a tile, as the TMA box of the grid
template <int W>
struct Box3 {
  static constexpr int EXT = 8 + W - 1;
  static constexpr int ZB = (EXT + 1) & ~1;
  static constexpr int EXTY = EXT + ((11 - EXT % 8) % 8);
  static constexpr int SY = ZB, SX = EXTY * ZB;  // row and plane strides (complex cells)
  static constexpr size_t BYTES = (size_t)EXT * SX * sizeof(float2);
};

template <int W>
struct C3 {
  static constexpr int EXT = Box3<W>::EXT;
  static constexpr int BOX = W + 1;                 // rows per dimension of a column
  static constexpr int BOXP = (BOX + 3) / 4 * 4;    // padded x / y vector length
  static constexpr int ROWS = BOX * BOX;            // (x, y) rows of a column
  static constexpr int RQ = 2;                      // rows per lane in each warp of a pair
  static constexpr int ZP = (W + 2 + 3) / 4 * 4;   // z taps with a parity shift, padded
  static constexpr int NPAIR = Box3<W>::ZB / 2;     // z pairs of a row
  // per-node record (floats): x scaled by f [BOXP] complex | y [BOXP] | z
  // [ZP] at the parity of the window start
  static constexpr int NXF = 0, NY = 2 * BOXP, NZ = 3 * BOXP, NF = 3 * BOXP + ZP;
  static constexpr size_t SUBGRID = (Box3<W>::BYTES + 127) / 128 * 128;
  static_assert(BOXP > BOX, "x / y vectors need one zero slot past the column");
  static_assert(W % 2 == 0, "even window width");
  static_assert(ROWS <= 4 * 32, "a pair's lanes hold the column's rows");
  static_assert(NPAIR * 2 >= EXT, "z pairs cover the padded tile");
};

template <int W>
inline size_t c3_smem_bytes()
{
  typedef C3<W> P;
  return P::SUBGRID + (size_t)C3_PAIRS * P::NF * C3_CHUNK * sizeof(float) + (17 + 2 + 2 * C3_PAIRS) * sizeof(int);
}

// Starts a bulk copy of the 16-byte aligned interior of [p, p + bytes) from
// global memory into L2 (cp.async.bulk.prefetch, sm_90 and later): the
// work item's node data arrive while the CTA zeroes or stages its subgrid.
__device__ __forceinline__ void c3_prefetch_l2(const void *p, long long bytes)
{
  const unsigned long long a = (unsigned long long)p;
  const unsigned long long b = (a + 15) & ~15ull, e = (a + (unsigned long long)bytes) & ~15ull;
  for (unsigned long long q = b; q < e; q += (1u << 20)) {
    const unsigned n = (unsigned)((e - q) < (1u << 20) ? (e - q) : (1u << 20));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q), "r"(n) : "memory");
  }
}

// the two warps of pair p (named barrier p + 1; barrier 0 is __syncthreads)
__device__ __forceinline__ void pair_sync(int p)
{
  asm volatile("bar.sync %0, 64;" ::"r"(p + 1) : "memory");
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
  typedef Box3<W> B;
  constexpr int EXT = P::EXT, BOX = P::BOX, BOXP = P::BOXP, RQ = P::RQ, NF = P::NF;
  constexpr int SX = B::SX, SY = B::SY;
  extern __shared__ __align__(128) unsigned char c3_smem[];
  float2 *const sg = reinterpret_cast<float2 *>(c3_smem);
  float *const scratch = reinterpret_cast<float *>(c3_smem + P::SUBGRID);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pair = warp >> 1, half = warp & 1;
  float *const wsc = scratch + pair * NF * C3_CHUNK;
  int *const cstart = reinterpret_cast<int *>(scratch + C3_PAIRS * NF * C3_CHUNK);
  int *const taskctr = cstart + 17;
  int *const nextslot = taskctr + 1 + pair;  // the pair's next task, posted by its first warp

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
  {
    float4 *z4 = reinterpret_cast<float4 *>(sg);
    for (int i = threadIdx.x; i < EXT * SX / 2; i += C3_THREADS) z4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // column boundaries of the item (node set-up): cstart[c] = first node of column c
  if (threadIdx.x < 17) cstart[threadIdx.x] = cst[17LL * blockIdx.x + threadIdx.x];
  if (threadIdx.x == 0) {
    *taskctr = 0;
    taskctr[1 + C3_PAIRS] = 0;  // the flush lock
  }
  __syncthreads();

  // segments per column (lanes 0..15), inclusive scan -> task -> column map
  int nseg = 0;
  if (lane < 16) nseg = (cstart[lane + 1] - cstart[lane] + C3_SEGN - 1) / C3_SEGN;
  int incl = nseg;
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
    const int ns = (clen + C3_SEGN - 1) / C3_SEGN;
    const int k = task - before, qn = clen / ns, rq = clen - qn * ns;
    a = it.start + cstart[c] + k * qn + min(k, rq);
    np = qn + (k < rq ? 1 : 0);
  };

  // byte offsets of the lane's rows' x and y weights in a node record (rows
  // past the column read the zero slot BOXP - 1 of the x vector)
  int xo[RQ], yo[RQ];
#pragma unroll
  for (int q = 0; q < RQ; ++q) {
    const int row = lane + 32 * (2 * half + q);
    const bool ok = row < P::ROWS;
    const int bx = ok ? row / BOX : 0, by = ok ? row - (row / BOX) * BOX : 0;
    xo[q] = 4 * P::NXF + 8 * (ok ? bx : BOXP - 1);
    yo[q] = 4 * P::NY + 4 * by;
  }

  // the pair's first task: its first warp takes it, both read it
  if (half == 0 && lane == 0) *nextslot = atomicAdd(taskctr, 1);
  pair_sync(pair);
  int task = *nextslot;
  pair_sync(pair);
  int c = 0, a = 0, np = 0;
  float4 rn = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 fn = make_float2(0.f, 0.f);
  if (task < ntask) {
    locate(task, c, a, np);
    if (lane < min(np, C3_CHUNK)) {
      rn = rec[a + lane];
      if (half == 0) fn = f[perm[a + lane]];
    }
  }
  while (task < ntask) {
    const int s0 = c >> 2, s1 = c & 3;
    // real and imaginary accumulators of the rows' z values, as aligned pairs
    float2 ar[RQ][P::NPAIR], ai[RQ][P::NPAIR];
#pragma unroll
    for (int q = 0; q < RQ; ++q)
#pragma unroll
      for (int z = 0; z < P::NPAIR; ++z) ar[q][z] = ai[q][z] = make_float2(0.f, 0.f);
    int zlo = 8, zhi = 0;  // z range the segment touches
    int off = 0;
    int ntaskid = task, c2 = c, a2 = a, np2 = np;
    for (;;) {
      const float4 r = rn;
      const float2 fj = fn;
      const int npc = min(C3_CHUNK, np - off);
      int off2 = off + C3_CHUNK;
      const bool last = off2 >= np;  // the segment's last chunk: the next is the next task's first
      if (last && half == 0 && lane == 0) *nextslot = atomicAdd(taskctr, 1);
      // ---- set-up: lane j evaluates node j's windows, x (scaled by f_j) in
      // the pair's first warp, y and z in its second
      const int loc = __float_as_int(r.w);
      int z0 = 8;
      if (lane < npc) {
        float *nd = wsc + lane * NF;
        float v[W];
        z0 = loc >> 6;
        if (half == 0) {
          const int ox = (loc & 7) - 2 * s0;  // the node's x offset in the column's box
          kb_poly_taps_sym<W>(r.x, poly.c[0], v);
          float4 *dst = reinterpret_cast<float4 *>(nd + P::NXF);
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
        } else {
          const int oy = ((loc >> 3) & 7) - 2 * s1;
          kb_poly_taps_sym<W>(r.y, poly.c[1], v);
          {
            float4 *dst = reinterpret_cast<float4 *>(nd + P::NY);
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
          // taps at the node's z offset within its aligned pair: a window
          // starting at odd z0 begins in the second half of a pair
          kb_poly_taps_sym<W>(r.z, poly.c[2], v);
          const int oz = z0 & 1;
          float4 *dst = reinterpret_cast<float4 *>(nd + P::NZ);
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
      zlo = min(zlo, __shfl_sync(0xffffffffu, z0, 0));
      zhi = max(zhi, __shfl_sync(0xffffffffu, z0, npc - 1) + W);
      pair_sync(pair);  // the chunk's node records are written; the next task id is posted
      // the next chunk's node data, loaded while this one computes
      if (last) {
        off2 = 0;
        ntaskid = *nextslot;
        if (ntaskid < ntask) locate(ntaskid, c2, a2, np2);
      }
      if (ntaskid < ntask) {
        const int n2 = min(C3_CHUNK, np2 - off2);
        if (lane < n2) {
          rn = rec[a2 + off2 + lane];
          if (half == 0) fn = f[perm[a2 + off2 + lane]];
        }
      }
      // runs of equal z0 (a chunk is sorted by z0): nodes [j0, j1) start at zz
      int j1 = __popc(__ballot_sync(0xffffffffu, z0 < 1));
      int j0 = 0;
#pragma unroll
      for (int zz = 0; zz < 8; ++zz) {
        if (zz > 0) {
          j0 = j1;
          j1 = __popc(__ballot_sync(0xffffffffu, z0 < zz + 1));
        }
        // window start zz: taps in pairs zz/2 .. zz/2 + npr - 1
        const int b = zz >> 1, npr = (zz & 1) ? W / 2 + 1 : W / 2;
#pragma unroll 1
        for (int j = j0; j < j1; ++j) {
          const char *nd = reinterpret_cast<const char *>(wsc + j * NF);
          // 8-byte broadcast reads (one shared-memory wavefront each)
          float2 w[P::ZP / 2];
#pragma unroll
          for (int k = 0; k < P::ZP / 2; ++k)
            if (k < npr) w[k] = reinterpret_cast<const float2 *>(nd + 4 * P::NZ)[k];
#pragma unroll
          for (int q = 0; q < RQ; ++q) {
            const float2 xf = *reinterpret_cast<const float2 *>(nd + xo[q]);
            const float yv = *reinterpret_cast<const float *>(nd + yo[q]);
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
      pair_sync(pair);  // both warps are done with the node records
      if (last) break;
      off = off2;
    }
    // ---- flush the segment's rows into the subgrid under the CTA's flush lock:
    // one pair at a time, by plain 16-byte read, paired adds and 16-byte store
    // (measured on GB300: 3.41 ms per launch at 512 nodes per tile against
    // 3.74 with a 128-bit compare-and-swap per cell pair and no lock)
    {
      int *const lockp = taskctr + 1 + C3_PAIRS;
      int *const haveslot = lockp + 1 + pair;
      if (half == 0 && lane == 0) {
        int got = 0;
        for (unsigned i = 0; i < (1u << 20); ++i) {
          if (atomicCAS(lockp, 0, 1) == 0) {
            got = 1;
            break;
          }
          __nanosleep(64);
        }
        __threadfence_block();
        if (!got) atomicAdd(&g_tma_wait_timeouts, 1ull);
        *haveslot = got;
      }
      pair_sync(pair);
      if (*haveslot) {
#pragma unroll
        for (int q = 0; q < RQ; ++q) {
          const int row = lane + 32 * (2 * half + q);
          if (row >= P::ROWS) continue;
          const int bx = row / BOX, by = row - bx * BOX;
          float4 *const rowp = reinterpret_cast<float4 *>(sg + (2 * s0 + bx) * SX + (2 * s1 + by) * SY);
#pragma unroll
          for (int p = 0; p < P::NPAIR; ++p) {
            if (2 * p + 2 <= zlo || 2 * p >= zhi) continue;
            const float4 cur = rowp[p];
            const float2 s01 = __fadd2_rn(make_float2(cur.x, cur.y), make_float2(ar[q][p].x, ai[q][p].x));
            const float2 s23 = __fadd2_rn(make_float2(cur.z, cur.w), make_float2(ar[q][p].y, ai[q][p].y));
            rowp[p] = make_float4(s01.x, s01.y, s23.x, s23.y);
          }
        }
      }
      pair_sync(pair);
      if (half == 0 && lane == 0 && *haveslot) {
        __threadfence_block();
        atomicExch(lockp, 0);
      }
    }
    task = ntaskid;
    c = c2;
    a = a2;
    np = np2;
  }
  __syncthreads();
  // ---- write-back.  A tile whose box lies inside the grid: one TMA
  // add-reduce straight from the subgrid (its cells past EXT add zeros).
  if (use_tma && org[0] + EXT <= g.n[0] && org[1] + B::EXTY <= g.n[1] && org[2] + B::ZB <= g.n[2] &&
      (smem_u32(sg) & 127u) == 0) {
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_reduce_add_3d(&gmap, sg, 2 * org[2], org[1], org[0]);
      bulk_commit();
      bulk_wait_read_all();  // the subgrid stays allocated until the copy has read it
    }
    return;
  }
  // a tile whose padded box wraps around the grid edge: one vector reduction
  // per non-zero cell
  for (int idx = threadIdx.x; idx < EXT * EXT * EXT; idx += C3_THREADS) {
    const int c2 = idx % EXT, r = idx / EXT;
    const int c1 = r % EXT, c0 = r / EXT;
    const float2 v = sg[c0 * SX + c1 * SY + c2];
    if (v.x == 0.f && v.y == 0.f) continue;
    int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
    while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
    while (p1 >= g.n[1]) p1 -= g.n[1];
    while (p2 >= g.n[2]) p2 -= g.n[2];
    global_add_c(grid + ((long long)p0 * g.n[1] + p1) * g.n[2] + p2, v);
  }
}

// ---------------------------------------------------------------------------
// B -- 3-D interpolation: f_j = sum phi_0 phi_1 phi_2 g over the window of
// every node (reference nfft_trafo_3d_B, nfft.c:4687-4914, with
// nfft_trafo_3d_compute, nfft.c:4020-4265), in two forms: by sub-cell units
// (k_b3_cell, for plans whose work items hold many nodes) and by column
// segments (k_b3_col, below, for the others).
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
  // the TMA box of the padded subgrid (Box3): its EXTY rows per x-plane let
  // the row-per-thread de-interleave read consecutive rows from different banks
  static constexpr int ZB = Box3<W>::ZB;
  static constexpr int EXTY = Box3<W>::EXTY;
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

// ---------------------------------------------------------------------------
// B by column segments on warp pairs, the gather counterpart of k_bt3_col:
// the CTA stages its tile's padded subgrid in the TMA box layout (one TMA copy
// for a tile whose box lies inside the grid, plain loads for one that wraps
// around the grid edge); its warp pairs take column segments from a shared
// counter:
//  * the lanes of a pair own the column's rows as in k_bt3_col and hold the
//    17 + 1 complex values of each of their two rows as (re, im) register pairs
//    for the whole segment;
//  * per chunk of 32 nodes, lane j of the pair's first warp evaluates node j's
//    x window, lane j of its second warp the y window and the z window as
//    (w, w) pairs;
//  * per node (a compile-time window start z0 per run, as in k_bt3_col) each
//    row's z sum is W paired FMAs of (w, w) with (re, im) in two chains, the
//    nodes of a run taken in pairs so that their chains interleave; the
//    lane's two rows are weighted by x y and summed, the two halves of each
//    warp are folded by one shuffle, and the 32 partial sums of the node go
//    to shared memory;
//  * at the end of a chunk lanes l and l + 16 of each warp sum sixteen
//    partials of one node each, fold them and write f_j through the node
//    permutation;
//  * the pairs take a tile's columns longest first, so that its last
//    segments are short.
template <int W>
struct CB {
  static constexpr int BOX = W + 1;
  static constexpr int BOXP = (BOX + 3) / 4 * 4;
  static constexpr int ROWS = BOX * BOX;
  static constexpr int RQ = 2;
  static constexpr int NZC = 2 * (Box3<W>::ZB / 2);  // z cells of a row held in registers
  // per-node record (floats): x [BOXP] | y [BOXP] | z taps as (w, w) pairs [W]
  static constexpr int NX = 0, NY = BOXP, NZ = 2 * BOXP, NF = 2 * BOXP + 2 * W;
  static constexpr int RS = 33;  // partial sums per node (32) and one pad, complex
  static constexpr size_t PAIR_BYTES =
      (size_t)NF * C3_CHUNK * sizeof(float) + (size_t)C3_CHUNK * RS * sizeof(float2);
  static_assert(NZC >= Box3<W>::EXT, "z cells cover the padded tile");
};

// subgrid box | per pair: node records, partial sums | ints | barrier
template <int W>
inline size_t cb_smem_bytes()
{
  return C3<W>::SUBGRID + (size_t)C3_PAIRS * CB<W>::PAIR_BYTES + (17 + 1 + C3_PAIRS + 3) * sizeof(int) + 8;
}

template <int W>
__global__ void __launch_bounds__(C3_THREADS, 2) k_b3_col(const WorkItem *__restrict__ items,
                                                           const float2 *__restrict__ grid,
                                                           const float4 *__restrict__ rec,
                                                           const uint16_t *__restrict__ cst,
                                                           const uint32_t *__restrict__ perm,
                                                           float2 *__restrict__ f, Geom<float> g, WinPoly poly,
                                                           const __grid_constant__ CUtensorMap gmap, int use_tma)
{
  typedef CB<W> P;
  typedef Box3<W> B;
  constexpr int EXT = B::EXT, BOX = P::BOX, BOXP = P::BOXP, RQ = P::RQ, NF = P::NF, SX = B::SX, SY = B::SY;
  extern __shared__ __align__(128) unsigned char c3_smem[];
  float2 *const sg = reinterpret_cast<float2 *>(c3_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pair = warp >> 1, half = warp & 1;
  unsigned char *const pscr = c3_smem + C3<W>::SUBGRID + pair * P::PAIR_BYTES;
  float *const wsc = reinterpret_cast<float *>(pscr);
  float2 *const red = reinterpret_cast<float2 *>(pscr + (size_t)NF * C3_CHUNK * sizeof(float));
  int *const cstart = reinterpret_cast<int *>(c3_smem + C3<W>::SUBGRID + C3_PAIRS * P::PAIR_BYTES);
  int *const taskctr = cstart + 17;
  int *const nextslot = taskctr + 1 + pair;
  unsigned long long *const bar = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<uintptr_t>(taskctr + 1 + C3_PAIRS + 2) & ~(uintptr_t)7);

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
  // the padded subgrid: one TMA copy where the box lies inside the grid,
  // plain loads where it wraps around the grid edge (the cells past EXT then
  // read as zeros; their weights are zero either way)
  const bool tma = use_tma && org[0] + EXT <= g.n[0] && org[1] + B::EXTY <= g.n[1] && org[2] + B::ZB <= g.n[2] &&
                   (smem_u32(sg) & 127u) == 0;
  if (threadIdx.x == 0 && tma) {
    mbar_init(bar, 1);
    mbar_expect_tx(bar, (unsigned)B::BYTES);
    tma_load_3d(sg, &gmap, 2 * org[2], org[1], org[0], bar);
  }
  if (!tma) {
#pragma unroll 4
    for (int idx = threadIdx.x; idx < EXT * EXT * B::ZB; idx += C3_THREADS) {
      const int c2 = idx % B::ZB, r = idx / B::ZB;
      const int c1 = r % EXT, c0 = r / EXT;
      float2 v = make_float2(0.f, 0.f);
      if (c2 < EXT) {
        int p0 = org[0] + c0, p1 = org[1] + c1, p2 = org[2] + c2;
        while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
        while (p1 >= g.n[1]) p1 -= g.n[1];
        while (p2 >= g.n[2]) p2 -= g.n[2];
        v = grid[((long long)p0 * g.n[1] + p1) * g.n[2] + p2];
      }
      sg[c0 * SX + c1 * SY + c2] = v;
    }
  }
  if (threadIdx.x < 17) cstart[threadIdx.x] = cst[17LL * blockIdx.x + threadIdx.x];
  if (threadIdx.x == 0) *taskctr = 0;
  __syncthreads();
  if (tma) {
    // a bounded wait: a copy that never arrives costs this tile, not a hang
    const bool ok = mbar_wait(bar, 0, TMA_WAIT_POLLS);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicAdd(&g_tma_wait_timeouts, 1ull);
      return;
    }
  }

  // columns ordered by length, longest first (16-lane bitonic sort of
  // (length, column)): the pairs take the long columns first, so that the
  // tile's last segments are short ones (measured: 3.83 -> 3.70 ms at 512
  // nodes per tile; B^T, whose flushes then overlap differently, lost by it)
  int ckey = -1, ccol = lane;
  if (lane < 16) ckey = cstart[lane + 1] - cstart[lane];
#pragma unroll
  for (int k = 2; k <= 16; k <<= 1) {
#pragma unroll
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      const int pk = __shfl_xor_sync(0xffffffffu, ckey, jj);
      const int pc = __shfl_xor_sync(0xffffffffu, ccol, jj);
      const bool lower = (lane & jj) == 0;
      const bool desc = (lane & k) == 0;
      // descending blocks keep the larger key in the lower lane
      const bool take = desc ? (lower ? pk > ckey : pk < ckey) : (lower ? pk < ckey : pk > ckey);
      if (lane < 16 && take) {
        ckey = pk;
        ccol = pc;
      }
    }
  }
  int nseg = 0;
  if (lane < 16) nseg = (ckey + C3_SEGN - 1) / C3_SEGN;
  int incl = nseg;
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int ntask = __shfl_sync(0xffffffffu, incl, 15);
  auto locate = [&](int task, int &c, int &a, int &np) {
    const int pos = __popc(__ballot_sync(0xffffffffu, lane < 16 && incl <= task));
    const int prev = __shfl_sync(0xffffffffu, incl, (pos + 31) & 31);
    const int before = pos > 0 ? prev : 0;
    c = __shfl_sync(0xffffffffu, ccol, pos);
    const int clen = cstart[c + 1] - cstart[c];
    const int ns = (clen + C3_SEGN - 1) / C3_SEGN;
    const int k = task - before, qn = clen / ns, rq = clen - qn * ns;
    a = it.start + cstart[c] + k * qn + min(k, rq);
    np = qn + (k < rq ? 1 : 0);
  };

  // byte offsets of the lane's rows' x and y weights in a node record (rows
  // past the column read the zero slot BOXP - 1 of the x vector)
  int xo[RQ], yo[RQ];
#pragma unroll
  for (int q = 0; q < RQ; ++q) {
    const int row = lane + 32 * (2 * half + q);
    const bool ok = row < P::ROWS;
    const int bx = ok ? row / BOX : 0, by = ok ? row - (row / BOX) * BOX : 0;
    xo[q] = 4 * P::NX + 4 * (ok ? bx : BOXP - 1);
    yo[q] = 4 * P::NY + 4 * by;
  }

  if (half == 0 && lane == 0) *nextslot = atomicAdd(taskctr, 1);
  pair_sync(pair);
  int task = *nextslot;
  pair_sync(pair);
  int c = 0, a = 0, np = 0;
  float4 rn = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t pn = 0;
  if (task < ntask) {
    locate(task, c, a, np);
    if (lane < min(np, C3_CHUNK)) {
      rn = rec[a + lane];
      pn = perm[a + lane];
    }
  }
  while (task < ntask) {
    const int s0 = c >> 2, s1 = c & 3;
    // the rows' grid values as (re, im) pairs
    float2 gv[RQ][P::NZC];
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
      const int row = lane + 32 * (2 * half + q);
      const int rr = row < P::ROWS ? row : 0;
      const int bx = rr / BOX, by = rr - bx * BOX;
      const float2 *rowp = sg + (2 * s0 + bx) * SX + (2 * s1 + by) * SY;
#pragma unroll
      for (int z = 0; z < P::NZC; ++z) gv[q][z] = rowp[z];
    }
    int off = 0;
    int ntaskid = task, c2 = c, a2 = a, np2 = np;
    for (;;) {
      const float4 r = rn;
      const uint32_t pj = pn;
      const int npc = min(C3_CHUNK, np - off);
      int off2 = off + C3_CHUNK;
      const bool last = off2 >= np;  // the segment's last chunk: the next is the next task's first
      if (last && half == 0 && lane == 0) *nextslot = atomicAdd(taskctr, 1);
      // ---- set-up: lane j evaluates node j's windows, x in the pair's first
      // warp, y and z in its second
      const int loc = __float_as_int(r.w);
      int z0 = 8;
      if (lane < npc) {
        float *nd = wsc + lane * NF;
        float v[W];
        z0 = loc >> 6;
        if (half == 0) {
          const int ox = (loc & 7) - 2 * s0;
          kb_poly_taps_sym<W>(r.x, poly.c[0], v);
          float4 *dst = reinterpret_cast<float4 *>(nd + P::NX);
#pragma unroll
          for (int q = 0; q < BOXP / 4; ++q) {
            float e[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const int b = 4 * q + h;
              float val = 0.f;
              if (b < W && ox == 0) val = v[b];
              if (b >= 1 && b - 1 < W && ox == 1) val = v[b - 1];
              e[h] = val;
            }
            dst[q] = make_float4(e[0], e[1], e[2], e[3]);
          }
        } else {
          const int oy = ((loc >> 3) & 7) - 2 * s1;
          kb_poly_taps_sym<W>(r.y, poly.c[1], v);
          {
            float4 *dst = reinterpret_cast<float4 *>(nd + P::NY);
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
          kb_poly_taps_sym<W>(r.z, poly.c[2], v);
          float4 *dst = reinterpret_cast<float4 *>(nd + P::NZ);
#pragma unroll
          for (int q = 0; q < W / 2; ++q) dst[q] = make_float4(v[2 * q], v[2 * q], v[2 * q + 1], v[2 * q + 1]);
        }
      }
      pair_sync(pair);  // the chunk's node records are written; the next task id is posted
      // the next chunk's node data, loaded while this one computes
      if (last) {
        off2 = 0;
        ntaskid = *nextslot;
        if (ntaskid < ntask) locate(ntaskid, c2, a2, np2);
      }
      if (ntaskid < ntask) {
        const int n2 = min(C3_CHUNK, np2 - off2);
        if (lane < n2) {
          rn = rec[a2 + off2 + lane];
          pn = perm[a2 + off2 + lane];
        }
      }
      // runs of equal z0 (a chunk is sorted by z0): nodes [j0, j1) start at zz
      int j1 = __popc(__ballot_sync(0xffffffffu, z0 < 1));
      int j0 = 0;
#pragma unroll
      for (int zz = 0; zz < 8; ++zz) {
        if (zz > 0) {
          j0 = j1;
          j1 = __popc(__ballot_sync(0xffffffffu, z0 < zz + 1));
        }
        // nodes in pairs: the z sums of two nodes are independent chains
        // (measured: 3.70 -> 3.58 ms at 512 nodes per tile, 3.65 -> 3.43 ms
        // clustered); an odd run's last node goes alone below, and both keep
        // each node's order of additions
#pragma unroll 1
        for (int j = j0; j + 1 < j1; j += 2) {
          const char *na = reinterpret_cast<const char *>(wsc + j * NF);
          const char *nb = na + 4 * NF;
          float2 ta[RQ][2], tb[RQ][2];
#pragma unroll
          for (int q = 0; q < RQ; ++q) ta[q][0] = ta[q][1] = tb[q][0] = tb[q][1] = make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 0; k < W; k += 2) {
            const float4 wa = reinterpret_cast<const float4 *>(na + 4 * P::NZ)[k / 2];
            const float4 wb = reinterpret_cast<const float4 *>(nb + 4 * P::NZ)[k / 2];
#pragma unroll
            for (int q = 0; q < RQ; ++q) {
              ta[q][0] = __ffma2_rn(make_float2(wa.x, wa.y), gv[q][zz + k], ta[q][0]);
              ta[q][1] = __ffma2_rn(make_float2(wa.z, wa.w), gv[q][zz + k + 1], ta[q][1]);
              tb[q][0] = __ffma2_rn(make_float2(wb.x, wb.y), gv[q][zz + k], tb[q][0]);
              tb[q][1] = __ffma2_rn(make_float2(wb.z, wb.w), gv[q][zz + k + 1], tb[q][1]);
            }
          }
          float par = 0.f, pai = 0.f, pbr = 0.f, pbi = 0.f;
#pragma unroll
          for (int q = 0; q < RQ; ++q) {
            const float2 sa = __fadd2_rn(ta[q][0], ta[q][1]), sb = __fadd2_rn(tb[q][0], tb[q][1]);
            const float wxa = *reinterpret_cast<const float *>(na + xo[q]) * *reinterpret_cast<const float *>(na + yo[q]);
            const float wxb = *reinterpret_cast<const float *>(nb + xo[q]) * *reinterpret_cast<const float *>(nb + yo[q]);
            par = fmaf(wxa, sa.x, par);
            pai = fmaf(wxa, sa.y, pai);
            pbr = fmaf(wxb, sb.x, pbr);
            pbi = fmaf(wxb, sb.y, pbi);
          }
          par += __shfl_xor_sync(0xffffffffu, par, 16);
          pai += __shfl_xor_sync(0xffffffffu, pai, 16);
          pbr += __shfl_xor_sync(0xffffffffu, pbr, 16);
          pbi += __shfl_xor_sync(0xffffffffu, pbi, 16);
          if (lane < 16) {
            red[j * P::RS + 16 * half + lane + half] = make_float2(par, pai);
            red[(j + 1) * P::RS + 16 * half + lane + half] = make_float2(pbr, pbi);
          }
        }
        if ((j1 - j0) & 1) {
          const int j = j1 - 1;
          const char *nd = reinterpret_cast<const char *>(wsc + j * NF);
          float2 w[W];
#pragma unroll
          for (int k = 0; k < W; ++k) w[k] = reinterpret_cast<const float2 *>(nd + 4 * P::NZ)[k];
          float pr = 0.f, pi = 0.f;
#pragma unroll
          for (int q = 0; q < RQ; ++q) {
            float2 t0 = make_float2(0.f, 0.f), t1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < W; k += 2) {
              t0 = __ffma2_rn(w[k], gv[q][zz + k], t0);
              t1 = __ffma2_rn(w[k + 1], gv[q][zz + k + 1], t1);
            }
            const float2 t = __fadd2_rn(t0, t1);
            const float wxy =
                *reinterpret_cast<const float *>(nd + xo[q]) * *reinterpret_cast<const float *>(nd + yo[q]);
            pr = fmaf(wxy, t.x, pr);
            pi = fmaf(wxy, t.y, pi);
          }
          pr += __shfl_xor_sync(0xffffffffu, pr, 16);
          pi += __shfl_xor_sync(0xffffffffu, pi, 16);
          // partial 16 half + lane of node j, at slot 16 half + lane + half
          // (lanes l and l + 16 of the summing warp read different banks)
          if (lane < 16) red[j * P::RS + 16 * half + lane + half] = make_float2(pr, pi);
        }
      }
      pair_sync(pair);  // the partial sums are stored; both warps are done with the node records
      // node n = 16 half + (lane & 15): lanes l and l + 16 each sum sixteen
      // partials (those of one warp), then fold
      {
        const int n = 16 * half + (lane & 15), hh = lane >> 4;
        float sr = 0.f, si = 0.f;
        if (n < npc) {
          const float2 *src = red + n * P::RS + 16 * hh + hh;
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const float2 v = src[k];
            sr += v.x;
            si += v.y;
          }
        }
        sr += __shfl_xor_sync(0xffffffffu, sr, 16);
        si += __shfl_xor_sync(0xffffffffu, si, 16);
        const uint32_t pw = __shfl_sync(0xffffffffu, pj, n);
        if (lane < 16 && n < npc) f[pw] = make_float2(sr, si);
      }
      // (the next chunk stores partial sums only after its first pair
      // barrier, which both warps reach after these reads)
      if (last) break;
      off = off2;
    }
    task = ntaskid;
    c = c2;
    a = a2;
    np = np2;
  }
}

}  // namespace gb
