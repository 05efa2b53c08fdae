// gb_col2.cu -- 2-D B^T (adjoint spreading, single and double precision)
// and B (interpolation) by x-row strips of sub-cell columns: the per-plan
// kernels.  The single-precision work-item functions and their design are in
// gb_col2.cuh.
#include <algorithm>

#include "gb_col2.cuh"
#include "gb_tma.cuh"

namespace gb {

// bounded TMA waits that gave up (read and cleared with the 3-D kernels' count
// by read_wait_timeouts)
__device__ unsigned long long g_tma_wait_timeouts_2d;

unsigned long long read_wait_timeouts_2d()
{
  unsigned long long v = 0, z = 0;
  GB_CUDA(cudaMemcpyFromSymbol(&v, g_tma_wait_timeouts_2d, sizeof(v)));
  GB_CUDA(cudaMemcpyToSymbol(g_tma_wait_timeouts_2d, &z, sizeof(z)));
  return v;
}

// The per-plan single-precision B with a TMA copy of the subgrid: the
// subgrid in the layout of one box of the grid's 2-D tensor map, EXT rows of
// ZB complex cells (ZB = EXT rounded up to even, so that rows are 16-byte
// multiples; the cells past EXT are not read), at the start of shared memory,
// the warps' vectors after it.  A tile whose box lies inside the grid is
// staged by one TMA copy (cp.async.bulk.tensor, an mbarrier with the box's
// byte count, a bounded wait), an edge tile by plain loads.  (The same layout
// for B^T, with one TMA add-reduce as its write-back, was slower: the even
// row stride costs its flush bank conflicts, and the box adds the zero cells
// of sparse tiles, which the cell-by-cell write-back skips.)
template <int W>
struct C2T {
  static constexpr int EXT = C2<W>::EXT;
  static constexpr int ZB = (EXT + 1) & ~1;
  static constexpr size_t SUBGRID = ((size_t)EXT * ZB * sizeof(float2) + 127) / 128 * 128;
};

template <int W>
inline size_t c2t_smem_bytes()
{
  return C2T<W>::SUBGRID + (size_t)C2_WARPS * C2<W>::WARP_FLOATS_B * sizeof(float) + sizeof(unsigned long long);
}

template <int W>
__global__ void __launch_bounds__(C2_THREADS, 3) k_b2_col_tma(const WorkItem *__restrict__ items,
                                                               const float2 *__restrict__ grid,
                                                               const float *__restrict__ xs,
                                                               const uint32_t *__restrict__ perm,
                                                               float2 *__restrict__ f, Geom<float> g, WinPoly poly,
                                                               const __grid_constant__ CUtensorMap gmap)
{
  typedef C2<W> P;
  typedef C2T<W> T;
  constexpr int EXT = T::EXT, ZB = T::ZB;
  extern __shared__ __align__(128) unsigned char c2_smem[];
  float2 *const sg = reinterpret_cast<float2 *>(c2_smem);
  float *const base = reinterpret_cast<float *>(c2_smem + T::SUBGRID);
  const int warp = threadIdx.x >> 5;
  float *const wx = base + warp * P::WARP_FLOATS_B;
  float *const wy = wx + P::XS * C2_CHUNK;
  unsigned long long *const bar =
      reinterpret_cast<unsigned long long *>(base + C2_WARPS * P::WARP_FLOATS_B);
  const WorkItem it = items[blockIdx.x];
  const int org0 = (it.tile / g.ntile[1]) * C2_TILE, org1 = (it.tile % g.ntile[1]) * C2_TILE;
  const bool tma = org0 + EXT <= g.n[0] && org1 + ZB <= g.n[1] && (smem_u32(sg) & 127u) == 0;
  if (tma) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      mbar_expect_tx(bar, (unsigned)(EXT * ZB * sizeof(float2)));
      tma_load_2d(sg, &gmap, 2 * org1, org0, bar);
    }
    __syncthreads();
    // a bounded wait: a copy that never arrives costs this tile, not a hang
    const bool ok = mbar_wait(bar, 0, TMA_WAIT_POLLS);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicAdd(&g_tma_wait_timeouts_2d, 1ull);
      return;
    }
  } else {
    c2_stage_plain<W, ZB>(sg, grid, g, org0, org1);
    __syncthreads();
  }
  c2_b_nodes<W, ZB>(it, sg, xs, perm, f, g, poly, wx, wy, org0, org1);
}

// per-plan kernels: one CTA per work item
template <int W, bool COMP>
__global__ void __launch_bounds__(C2_THREADS, 3) k_bt2_col(const WorkItem *__restrict__ items,
                                                            float2 *__restrict__ grid,
                                                            const float *__restrict__ xs,
                                                            const uint32_t *__restrict__ perm,
                                                            const float2 *__restrict__ f, Geom<float> g,
                                                            WinPoly poly, float2 *__restrict__ grid_lo)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  c2_bt_item<W, COMP>(items[blockIdx.x], grid, xs, perm, f, g, poly, smem_raw, grid_lo);
}

// grid += grid_lo: the compensated B^T's rounding errors folded in before the FFT
__global__ void k_fold_lo(float2 *__restrict__ grid, const float2 *__restrict__ lo, long long n)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const float2 a = grid[k], b = lo[k];
    grid[k] = make_float2(a.x + b.x, a.y + b.y);
  }
}

template <int W>
__global__ void __launch_bounds__(C2_THREADS, 3) k_b2_col(const WorkItem *__restrict__ items,
                                                           const float2 *__restrict__ grid,
                                                           const float *__restrict__ xs,
                                                           const uint32_t *__restrict__ perm,
                                                           float2 *__restrict__ f, Geom<float> g, WinPoly poly)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  c2_b_item<W>(items[blockIdx.x], grid, xs, perm, f, g, poly, smem_raw);
}

// ---------------------------------------------------------------- double
// The B^T above in double precision (the FP64 transforms of the
// mixed-precision solver and of double plans): the same columns and lane
// roles, FP64 accumulators (one FMA per y position and component), the
// window from its degree-16 form (gb_window.cpp), four warps per CTA for the
// larger vectors.
static constexpr int C2D_THREADS = 128;
static constexpr int C2D_WARPS = C2D_THREADS / 32;

template <int W>
struct C2D {
  typedef C2<W> P;
  static constexpr int NP = 2 * P::HP;       // y positions per half-warp
  static constexpr int XS = 17;              // x vector stride (complex)
  static constexpr int YS = 2 * NP + 2;      // y vector stride (doubles; even: 16-byte pairs)
  static constexpr int WARP_DOUBLES = 2 * XS * C2_CHUNK + YS * C2_CHUNK;
};

template <int W>
static size_t c2d_smem_bytes()
{
  typedef C2<W> P;
  return (size_t)C2D_WARPS * C2D<W>::WARP_DOUBLES * sizeof(double) + (size_t)P::EXT * P::SY * sizeof(double2);
}

template <int W>
__global__ void __launch_bounds__(C2D_THREADS) k_bt2_col_d(const WorkItem *__restrict__ items,
                                                           double2 *__restrict__ grid,
                                                           const double *__restrict__ xs,
                                                           const uint32_t *__restrict__ perm,
                                                           const double2 *__restrict__ f, Geom<double> g,
                                                           WinPolyD poly)
{
  typedef C2<W> P;
  typedef C2D<W> Q;
  constexpr int CX = P::CX, NP = Q::NP, SY = P::SY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *const base = reinterpret_cast<double *>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double2 *const wx = reinterpret_cast<double2 *>(base + warp * Q::WARP_DOUBLES);  // stride XS
  double *const wy = base + warp * Q::WARP_DOUBLES + 2 * Q::XS * C2_CHUNK;           // stride YS
  double2 *const sg = reinterpret_cast<double2 *>(base + C2D_WARPS * Q::WARP_DOUBLES);

  const WorkItem it = items[blockIdx.x];
  const int org0 = (it.tile / g.ntile[1]) * C2_TILE, org1 = (it.tile % g.ntile[1]) * C2_TILE;
  for (int i = threadIdx.x; i < P::EXT * SY; i += C2D_THREADS) sg[i] = make_double2(0.0, 0.0);
  __syncthreads();
  const int h = lane >> 4, r = lane & 15;

  for (int a = it.start + warp * C2_CHUNK; a < it.end; a += C2D_WARPS * C2_CHUNK) {
    const int np = min(C2_CHUNK, it.end - a);
    int col = -1;
    if (lane < np) {
      const int i = a + lane;
      const double xn0 = xs[2LL * i] * g.nR[0], xn1 = xs[2LL * i + 1] * g.nR[1];
      const int u0 = (int)floor(xn0) - g.m, u1 = (int)floor(xn1) - g.m;  // node_u
      const double s0 = fma(2.0, xn0 - (double)u0, -(double)(2 * g.m + 1));
      const double s1 = fma(2.0, xn1 - (double)u1, -(double)(2 * g.m + 1));
      const int ux = min(max(wrap(u0, g.n[0]) - org0, 0), C2_TILE - 1);
      const int uy = min(max(wrap(u1, g.n[1]) - org1, 0), C2_TILE - 1);
      const int ox = ux % CX, oy = uy % C2_CY;
      col = (ux / CX) * C2_SLABS + uy / C2_CY;
      const double2 fj = f[perm[i]];
      double v[W];
      double2 *xv = wx + Q::XS * lane;
#pragma unroll
      for (int q = 0; q < 16; ++q) xv[q] = make_double2(0.0, 0.0);
      kb_polyd_taps_s<W>(s0, poly.c[0], v);
#pragma unroll
      for (int l = 0; l < W; ++l) xv[ox + l] = make_double2(v[l] * fj.x, v[l] * fj.y);
      double *yv = wy + Q::YS * lane;
#pragma unroll
      for (int q = 0; q < 2 * NP; ++q) yv[q] = 0.0;
      kb_polyd_taps_s<W>(s1, poly.c[1], v);
#pragma unroll
      for (int l = 0; l < W; ++l) yv[oy + l] = v[l];
    }
    const int prevc = __shfl_up_sync(0xffffffffu, col, 1);
    unsigned starts = __ballot_sync(0xffffffffu, lane < np && (lane == 0 || col != prevc));
    __syncwarp();
    while (starts) {
      const int s = __ffs(starts) - 1;
      starts &= starts - 1;
      const int e = starts ? __ffs(starts) - 1 : np;
      const int c = __shfl_sync(0xffffffffu, col, s);
      double ar[NP], ai[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) ar[q] = ai[q] = 0.0;
      for (int j = s; j < e; ++j) {
        const double2 xf = wx[Q::XS * j + r];
        const double2 *yp = reinterpret_cast<const double2 *>(wy + Q::YS * j + h * NP);
#pragma unroll
        for (int q = 0; q < NP / 2; ++q) {
          const double2 w = yp[q];
          ar[2 * q] = fma(w.x, xf.x, ar[2 * q]);
          ai[2 * q] = fma(w.x, xf.y, ai[2 * q]);
          ar[2 * q + 1] = fma(w.y, xf.x, ar[2 * q + 1]);
          ai[2 * q + 1] = fma(w.y, xf.y, ai[2 * q + 1]);
        }
      }
      const int xc = c / C2_SLABS, sl = c - xc * C2_SLABS;
      if (r < P::ROWS) {
        double2 *p = sg + (CX * xc + r) * SY + C2_CY * sl + h * NP;
        const int nv = P::NPOS - h * NP;
#pragma unroll
        for (int q = 0; q < NP; ++q)
          if (q < nv && (ar[q] != 0.0 || ai[q] != 0.0)) {
            atomicAdd(&p[q].x, ar[q]);
            atomicAdd(&p[q].y, ai[q]);
          }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < P::EXT * P::EXT; idx += C2D_THREADS) {
    const int rx = idx / P::EXT, ry = idx - rx * P::EXT;
    const double2 v = sg[rx * SY + ry];
    if (v.x != 0.0 || v.y != 0.0) {
      int p0 = org0 + rx, p1 = org1 + ry;
      while (p0 >= g.n[0]) p0 -= g.n[0];
      while (p1 >= g.n[1]) p1 -= g.n[1];
      global_add_c(grid + (long long)p0 * g.n[1] + p1, v);
    }
  }
}

template <int W>
static void run_bt2_d(const WorkItem *items, int nitems, double2 *grid, const double *xs, const uint32_t *perm,
                      const double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s)
{
  const size_t smem = c2d_smem_bytes<W>();
  set_smem_limit((const void *)k_bt2_col_d<W>, smem);
  k_bt2_col_d<W><<<nitems, C2D_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly);
  GB_LAUNCHED("bt2_col_d");
}

// Double-precision 2-D B, one node per thread over a 128-node work item: the
// tile's padded subgrid in shared memory, the node's taps from the degree-16
// form, the w^2 gather in row order.
template <int W>
__global__ void __launch_bounds__(C2D_THREADS) k_b2_node_d(const WorkItem *__restrict__ items,
                                                           const double2 *__restrict__ grid,
                                                           const double *__restrict__ xs,
                                                           const uint32_t *__restrict__ perm,
                                                           double2 *__restrict__ f, Geom<double> g, WinPolyD poly)
{
  typedef C2<W> P;
  constexpr int EXT = P::EXT, SY = P::SY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *const sg = reinterpret_cast<double2 *>(smem_raw);
  const WorkItem it = items[blockIdx.x];
  const int org0 = (it.tile / g.ntile[1]) * C2_TILE, org1 = (it.tile % g.ntile[1]) * C2_TILE;
  for (int idx = threadIdx.x; idx < EXT * EXT; idx += C2D_THREADS) {
    const int rx = idx / EXT, ry = idx - rx * EXT;
    int p0 = org0 + rx, p1 = org1 + ry;
    while (p0 >= g.n[0]) p0 -= g.n[0];  // a padded tile can wrap more than once on small grids
    while (p1 >= g.n[1]) p1 -= g.n[1];
    sg[rx * SY + ry] = grid[(long long)p0 * g.n[1] + p1];
  }
  __syncthreads();
  for (int i = it.start + threadIdx.x; i < it.end; i += C2D_THREADS) {
    const double xn0 = xs[2LL * i] * g.nR[0], xn1 = xs[2LL * i + 1] * g.nR[1];
    const int u0 = (int)floor(xn0) - g.m, u1 = (int)floor(xn1) - g.m;  // node_u
    const double s0 = fma(2.0, xn0 - (double)u0, -(double)(2 * g.m + 1));
    const double s1 = fma(2.0, xn1 - (double)u1, -(double)(2 * g.m + 1));
    const int l0 = min(max(wrap(u0, g.n[0]) - org0, 0), C2_TILE - 1);
    const int l1 = min(max(wrap(u1, g.n[1]) - org1, 0), C2_TILE - 1);
    double v0[W], v1[W];
    kb_polyd_taps_s<W>(s0, poly.c[0], v0);
    kb_polyd_taps_s<W>(s1, poly.c[1], v1);
    double ar = 0.0, ai = 0.0;
#pragma unroll
    for (int a = 0; a < W; ++a) {
      const double2 *row = sg + (l0 + a) * SY + l1;
      double rr = 0.0, ri = 0.0;
#pragma unroll
      for (int b = 0; b < W; ++b) {
        const double2 c = row[b];
        rr = fma(v1[b], c.x, rr);
        ri = fma(v1[b], c.y, ri);
      }
      ar = fma(v0[a], rr, ar);
      ai = fma(v0[a], ri, ai);
    }
    f[perm[i]] = make_double2(ar, ai);
  }
}

template <int W>
static void run_b2_d(const WorkItem *items, int nitems, const double2 *grid, const double *xs,
                     const uint32_t *perm, double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s)
{
  const size_t smem = (size_t)C2<W>::EXT * C2<W>::SY * sizeof(double2);
  set_smem_limit((const void *)k_b2_node_d<W>, smem);
  k_b2_node_d<W><<<nitems, C2D_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly);
  GB_LAUNCHED("b2_node_d");
}

template <int W>
static void run_bt2(const WorkItem *items, int nitems, float2 *grid, const float *xs, const uint32_t *perm,
                    const float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s, float2 *grid_lo)
{
  if (grid_lo) {
    const size_t smem = c2_smem_bytes<W>(true, true);
    set_smem_limit((const void *)k_bt2_col<W, true>, smem);
    k_bt2_col<W, true><<<nitems, C2_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly, grid_lo);
    GB_LAUNCHED("bt2_col (compensated)");
    const long long n = (long long)g.n[0] * g.n[1];
    k_fold_lo<<<(unsigned)std::min<long long>((n + 255) / 256, 1216), 256, 0, s>>>(grid, grid_lo, n);
    GB_LAUNCHED("fold_lo");
    return;
  }
  const size_t smem = c2_smem_bytes<W>(true);
  set_smem_limit((const void *)k_bt2_col<W, false>, smem);
  k_bt2_col<W, false><<<nitems, C2_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly, nullptr);
  GB_LAUNCHED("bt2_col");
}

template <int W>
static void run_b2(const WorkItem *items, int nitems, const float2 *grid, const float *xs, const uint32_t *perm,
                   float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s, const CUtensorMap *gmap)
{
  if (gmap) {
    const size_t smem = c2t_smem_bytes<W>();
    set_smem_limit((const void *)k_b2_col_tma<W>, smem);
    k_b2_col_tma<W><<<nitems, C2_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly, *gmap);
    GB_LAUNCHED("b2_col_tma");
    return;
  }
  const size_t smem = c2_smem_bytes<W>(false);
  set_smem_limit((const void *)k_b2_col<W>, smem);
  k_b2_col<W><<<nitems, C2_THREADS, smem, s>>>(items, grid, xs, perm, f, g, poly);
  GB_LAUNCHED("b2_col");
}

#define GB_COL2_WIDTHS(X) X(6) X(8) X(10) X(12) X(14) X(16)

int col2_column_width(int w)
{
  switch (w) {
#define GB_C2_CX(W) \
  case W:           \
    return C2<W>::CX;
    GB_COL2_WIDTHS(GB_C2_CX)
#undef GB_C2_CX
    default:
      return 0;
  }
}

int col2_box_zb(int w)
{
  return (C2_TILE + w - 1 + 1) & ~1;  // the padded tile edge rounded up to even
}

void launch_bt2_col(const WorkItem *items, int nitems, float2 *grid, const float *xs, const uint32_t *perm,
                    const float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s, float2 *grid_lo)
{
  if (nitems <= 0) return;
  switch (g.w) {
#define GB_C2_RUN(W)                                                          \
  case W:                                                                     \
    run_bt2<W>(items, nitems, grid, xs, perm, f, g, poly, s, grid_lo); \
    return;
    GB_COL2_WIDTHS(GB_C2_RUN)
#undef GB_C2_RUN
    default:
      fatal("no 2-D column kernel for w=%d", g.w);
  }
}

void launch_b2_col(const WorkItem *items, int nitems, const float2 *grid, const float *xs, const uint32_t *perm,
                   float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s, const CUtensorMap *gmap)
{
  if (nitems <= 0) return;
  switch (g.w) {
#define GB_C2_RUN(W)                                                      \
  case W:                                                                 \
    run_b2<W>(items, nitems, grid, xs, perm, f, g, poly, s, gmap); \
    return;
    GB_COL2_WIDTHS(GB_C2_RUN)
#undef GB_C2_RUN
    default:
      fatal("no 2-D column kernel for w=%d", g.w);
  }
}

}  // namespace gb

namespace gb {

void launch_bt2_col_d(const WorkItem *items, int nitems, double2 *grid, const double *xs, const uint32_t *perm,
                      const double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s)
{
  if (nitems <= 0) return;
  switch (g.w) {
#define GB_C2D_RUN(W)                                               \
  case W:                                                           \
    run_bt2_d<W>(items, nitems, grid, xs, perm, f, g, poly, s); \
    return;
    GB_COL2_WIDTHS(GB_C2D_RUN)
#undef GB_C2D_RUN
    default:
      fatal("no 2-D column kernel for w=%d", g.w);
  }
}

void launch_b2_node_d(const WorkItem *items, int nitems, const double2 *grid, const double *xs,
                      const uint32_t *perm, double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s)
{
  if (nitems <= 0) return;
  switch (g.w) {
#define GB_C2D_RUN(W)                                              \
  case W:                                                          \
    run_b2_d<W>(items, nitems, grid, xs, perm, f, g, poly, s); \
    return;
    GB_COL2_WIDTHS(GB_C2D_RUN)
#undef GB_C2D_RUN
    default:
      fatal("no 2-D double-precision kernel for w=%d", g.w);
  }
}

}  // namespace gb
