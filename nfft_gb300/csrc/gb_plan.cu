// gb_plan.cu -- the nfft_plan C API on the GPU.
//
// Reference: init_help (nfft.c:5950-6046), nfft_init / init_guru / init_1d..3d
// (nfft.c:6048-6166), precompute_one_psi and friends (nfft.c:5776-5948),
// nfft_trafo / nfft_adjoint (nfft.c:5655-5749) and their d-specialisations
// (nfft.c:2775-2903, 3808-3998, 5387-5651), the direct transforms
// (nfft.c:145-297), nfft_check (nfft.c:6169-6207), nfft_finalize
// (nfft.c:6209-6270).
//
// Design: the plan struct keeps the reference layout and host-array
// semantics; its device state (a Ctx) hangs off my_fftw_plan1.  A transform
// copies its input vector to HBM, runs D -> cuFFT -> B (trafo) or
// B^T -> cuFFT -> D^T (adjoint) on the plan's stream and copies the result
// back before returning, so callers read f / f_hat immediately, as with the
// reference.  Node set-up (precompute_one_psi) uploads x once, bins the
// nodes by grid tile on the GPU and, when NFFT_SORT_NODES is set, also
// produces the reference's sorted index_x bit-exactly.
#include <cufft.h>

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/nfft3.h"
#include "gb_internal.h"

namespace gb {

template <typename R> struct Api;
template <> struct Api<double> {
  typedef nfft_plan plan;
  typedef fftw_complex cx;
  static void *mal(size_t n) { return nfft_malloc(n); }
  static void fre(void *p) { nfft_free(p); }
  static const cufftType fft_type = CUFFT_Z2Z;
  static void set_mv(plan *p)
  {
    p->mv_trafo = (void (*)(void *))nfft_trafo;
    p->mv_adjoint = (void (*)(void *))nfft_adjoint;
  }
};
template <> struct Api<float> {
  typedef nfftf_plan plan;
  typedef fftwf_complex cx;
  static void *mal(size_t n) { return nfftf_malloc(n); }
  static void fre(void *p) { nfftf_free(p); }
  static const cufftType fft_type = CUFFT_C2C;
  static void set_mv(plan *p)
  {
    p->mv_trafo = (void (*)(void *))nfftf_trafo;
    p->mv_adjoint = (void (*)(void *))nfftf_adjoint;
  }
};

static void check_fft(cufftResult r, const char *what)
{
  if (r != CUFFT_SUCCESS) fatal("cuFFT %s failed (cufftResult %d)", what, (int)r);
}

// Device state of one plan.
template <typename R>
struct Ctx {
  typedef typename Cx<R>::T C;
  Geom<R> g;
  unsigned flags = 0;
  bool direct = false;   // reference switches to the NDFT (nfft.c:5658-5665)
  bool tiled = false;
  bool group3 = false;  // 3-D sub-cell group kernels
  WinPoly poly = {};     // polynomial window of the single-precision 2-D / 3-D kernels
  WinPolyD polyd = {};   // the same in double precision (2-D double-precision kernels)
  bool col2 = false;     // 2-D column kernels (nodes keyed by column)
  int comp = 0;          // compensated 2-D single-precision B^T (nfftf_gb_set_compensated), off by default
  int b3mode = 0;        // 3-D single-precision B (nfftf_gb_set_b3_kernel): 0 or 1 column segments, 2 sub-cell units
  void *grid_lo = nullptr;  // its error grid (n_total complex), allocated on first use
  bool col3 = false;     // single-precision column / sub-cell kernels (node records below)
  float4 *c3rec = nullptr;
  uint16_t *c3cst = nullptr, *c3sst = nullptr;
  CUtensorMap grid_map;      // TMA view of `grid` for the 3-D column kernels (B^T, B)
  CUtensorMap grid_map2;     // TMA view of `grid` for the 2-D single-precision column B
  bool grid_map2_ok = false;
  bool grid_map_ok = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // FFT: one plan for d <= 3; for d > 3 a rank-3 plan over the last three
  // dimensions plus strided rank-1 plans for the leading ones
  cufftHandle fft_main = 0;
  bool fft_ok = false;
  int fft_lead = 0;             // number of leading dims done by 1-D plans
  cufftHandle fft_lead_plan[GB_MAXD] = {};
  long long fft_lead_outer[GB_MAXD] = {};
  long long fft_lead_stride[GB_MAXD] = {};
  // device buffers
  R *x_dev = nullptr;       // caller-order copy of x
  R *xs = nullptr;          // tile-ordered x
  uint32_t *perm = nullptr; // tile order -> caller order
  C *grid = nullptr;
  C *fhat_dev = nullptr;
  C *f_dev = nullptr;
  double *cphi = nullptr;
  uint32_t *tile_start = nullptr;
  WorkItem *items = nullptr;
  int nitems = 0;
  int ntiles = 1;
  int force_T = 0;  // 2-D tile edge set by the batch autotuner (0 = automatic)
  bool nodes_ready = false;
  unsigned long long gen = 0;  // bumped whenever node set-up rebuilds the node order and work items
  cudaEvent_t ev[7] = {};
  // optional per-call event ring for timing a sequence of device calls
  std::vector<cudaEvent_t> ring;  // 7 events per slot
  std::vector<char> ring_kind;    // 1 = trafo, 0 = adjoint
  int ring_slots = 0, ring_used = 0;
  bool ring_on = false;
  bool last_trafo = true;
  bool timed = false;
  float stage_ms[4] = {0, 0, 0, 0};
  int launches = 0;
};

template <typename R>
static Ctx<R> *ctx_of(const typename Api<R>::plan *p)
{
  Ctx<R> *c = reinterpret_cast<Ctx<R> *>(p->my_fftw_plan1);
  if (!c) fatal("plan has no device context (not initialised by this library)");
  return c;
}

static int ceil_log2(long long v)
{
  int b = 0;
  while ((1LL << b) < v) ++b;
  return b;
}

// Nodes per work item of the transform kernels: the 3-D group kernels take
// large items; 2-D plans take small ones so that crowded tiles spread over
// many SMs (double precision, bound by FP64 arithmetic, the smallest).
template <typename R>
static int item_chunk(const Ctx<R> *c)
{
  if (c->group3) return group3_max_item();
  if (std::is_same<R, double>::value && c->g.d == 2) return 128;
  if (c->col2) return 256;  // 2-D column kernels: eight warp tasks of 32 nodes
  return 1024;
}

// Tile edge per dimension for the shared-memory kernels: the largest
// candidate whose padded subgrid fits the shared-memory budget.
template <typename R>
static void choose_tiles(Ctx<R> *c)
{
  Geom<R> &g = c->g;
  const size_t cap = 96 * 1024;
  const int cand1[] = {512, 256, 128, 64};
  const int cand2[] = {32, 16, 8};
  const int cand3[] = {8, 4, 2};
  const int *cand = g.d == 1 ? cand1 : (g.d == 2 ? cand2 : cand3);
  const int ncand = g.d == 1 ? 4 : 3;
  c->tiled = false;
  int T = 0;
  if (g.d <= 3 && tiled_supported<R>(g.d, g.w)) {
    for (int i = 0; i < ncand; ++i) {
      size_t cells = 1;
      for (int t = 0; t < g.d; ++t) cells *= (size_t)(cand[i] + g.w - 1);
      if (cells * sizeof(typename Cx<R>::T) <= cap) {
        T = cand[i];
        break;
      }
    }
    c->tiled = T > 0;
    if (c->tiled && c->force_T > 0 && g.d == 2) T = c->force_T;  // chosen by the batch autotuner
  }
  if (!c->tiled) T = g.d == 1 ? 256 : (g.d == 2 ? 32 : 8);  // binning only, for locality
  // 3-D: sub-cell group kernels on 8^3 tiles where the grid allows
  const int cs = group3_subcell_edge();
  c->group3 = false;
  g.cs = 1;
  g.csz = 1;
  g.sub = 1;
  if (g.d == 3 && group3_supported<R>(g.w) && g.n[0] >= 8 && g.n[1] >= 8 && g.n[2] >= 8) {
    Geom<R> h = g;
    for (int t = 0; t < 3; ++t) h.ext[t] = 8 + g.w - 1;
    h.sx = h.ext[0] * (h.ext[0] + 8) + 40;  // upper bound of the padded plane stride
    if (group3_smem_bytes<R>(h) <= 200 * 1024) {
      c->group3 = true;
      c->tiled = true;
      T = 8;
      g.cs = cs;
      // the z-column B^T kernel wants its columns' nodes ordered by window
      // start along z; the sub-cell B kernel only needs them grouped by
      // sub-cell, which that finer order also gives
      g.csz = group3_column_supported<R>(g.w) ? 1 : cs;
      g.sub = (8 / cs) * (8 / cs) * (8 / g.csz);
      // plane strides: rows of a box taken 32 at a time by a warp should hit
      // distinct banks; search the padding that minimises the worst case
      const int ext = 8 + g.w - 1, box = g.w + cs - 1, rows = box * box;
      int best = 1 << 30;
      g.sy = ext;
      g.sx = ext * ext;
      // (even strides: the sub-cell kernel reads rows as 8-byte pairs)
      for (int sy = ext + (ext & 1); sy < ext + 8; sy += 2)
        for (int sx = ext * sy; sx < ext * sy + 40; sx += 2) {
          int cost = 0;
          for (int r0 = 0; r0 < rows; r0 += 32) {
            int cnt[32] = {0}, worst = 0;
            for (int l = 0; l < 32 && r0 + l < rows; ++l) {
              const int r = r0 + l, bx = r / box, by = r % box;
              worst = std::max(worst, ++cnt[(bx * sx + by * sy) & 31]);
            }
            cost += worst;
          }
          cost = cost * 4096 + (sx * ext);  // then the smallest footprint
          if (cost < best) {
            best = cost;
            g.sy = sy;
            g.sx = sx;
          }
        }
    }
  }
  // 2-D: column B^T (and B in single precision) on 32^2 tiles, nodes keyed by
  // (tile, column of CX x-cells by 8 y-cells); not under the batch engine,
  // which sets its own tiles
  c->col2 = false;
  {
    const int cx = col2_column_width(g.w);
    if (g.d == 2 && c->tiled && c->force_T == 0 && T == 32 && cx > 0 && g.n[0] >= 32 && g.n[1] >= 32) {
      c->col2 = true;
      g.cs = cx;
      g.csz = 8;
      g.sub = (32 / cx) * (32 / 8);
    }
  }
  c->ntiles = 1;
  for (int t = 0; t < g.d; ++t) {
    g.T[t] = std::min(T, g.n[t]);
    g.ntile[t] = (g.n[t] + g.T[t] - 1) / g.T[t];
    g.ext[t] = g.T[t] + g.w - 1;
    c->ntiles *= g.ntile[t];
  }
  for (int t = g.d; t < GB_MAXD; ++t) {
    g.T[t] = 1;
    g.ntile[t] = 1;
    g.ext[t] = 1;
  }
}

template <typename R>
static void make_fft(Ctx<R> *c)
{
  const Geom<R> &g = c->g;
  const cufftType ty = Api<R>::fft_type;
  if (g.d <= 3) {
    int n[3];
    for (int t = 0; t < g.d; ++t) n[t] = g.n[t];
    check_fft(cufftPlanMany(&c->fft_main, g.d, n, nullptr, 1, 0, nullptr, 1, 0, ty, 1), "plan");
    c->fft_lead = 0;
  } else {
    // last three dimensions batched, leading dimensions one at a time
    int n3[3] = {g.n[g.d - 3], g.n[g.d - 2], g.n[g.d - 1]};
    long long inner3 = (long long)n3[0] * n3[1] * n3[2];
    int batch = (int)(g.n_total / inner3);
    check_fft(cufftPlanMany(&c->fft_main, 3, n3, nullptr, 1, (int)inner3, nullptr, 1, (int)inner3,
                            ty, batch),
              "plan");
    c->fft_lead = g.d - 3;
    for (int t = 0; t < g.d - 3; ++t) {
      long long inner = 1, outer = 1;
      for (int s = t + 1; s < g.d; ++s) inner *= g.n[s];
      for (int s = 0; s < t; ++s) outer *= g.n[s];
      int nt = g.n[t];
      check_fft(cufftPlanMany(&c->fft_lead_plan[t], 1, &nt, &nt, (int)inner, 1, &nt, (int)inner, 1,
                              ty, (int)inner),
                "plan");
      c->fft_lead_outer[t] = outer;
      c->fft_lead_stride[t] = (long long)nt * inner;
    }
  }
  c->fft_ok = true;
}

static void exec_fft_one(cufftHandle h, float2 *a, int dir)
{
  check_fft(cufftExecC2C(h, reinterpret_cast<cufftComplex *>(a), reinterpret_cast<cufftComplex *>(a),
                         dir),
            "exec");
}
static void exec_fft_one(cufftHandle h, double2 *a, int dir)
{
  check_fft(cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex *>(a),
                         reinterpret_cast<cufftDoubleComplex *>(a), dir),
            "exec");
}

template <typename R>
static void run_fft(Ctx<R> *c, int dir)
{
  check_fft(cufftSetStream(c->fft_main, c->stream), "set stream");
  exec_fft_one(c->fft_main, c->grid, dir);
  for (int t = 0; t < c->fft_lead; ++t) {
    check_fft(cufftSetStream(c->fft_lead_plan[t], c->stream), "set stream");
    for (long long o = 0; o < c->fft_lead_outer[t]; ++o)
      exec_fft_one(c->fft_lead_plan[t], c->grid + o * c->fft_lead_stride[t], dir);
  }
}

template <typename R>
static void dev_alloc(void **p, size_t bytes)
{
  if (bytes == 0) bytes = 16;
  GB_CUDA(cudaMalloc(p, bytes));
}

// ------------------------------------------------------------ init
template <typename R>
static void init_help(typename Api<R>::plan *ths)
{
  typedef typename Cx<R>::T C;
  const int d = (int)ths->d;
  if (d < 1 || d > GB_MAXD) fatal("dimension d=%d outside 1..%d", d, GB_MAXD);
  if (ths->m < 0 || 2 * ths->m + 2 > GB_MAXW) fatal("cut-off m=%td outside 0..%d", ths->m, (GB_MAXW - 2) / 2);
  if (ths->flags & NFFT_OMP_BLOCKWISE_ADJOINT) ths->flags |= NFFT_SORT_NODES;  // nfft.c:5955-5956

  ths->N_total = 1;
  ths->n_total = 1;
  for (int t = 0; t < d; ++t) {
    ths->N_total *= ths->N[t];
    ths->n_total *= ths->n[t];
  }
  ths->sigma = (R *)Api<R>::mal((size_t)d * sizeof(R));
  ths->b = (R *)Api<R>::mal((size_t)d * sizeof(R));
  for (int t = 0; t < d; ++t) {
    ths->sigma[t] = ((R)ths->n[t]) / (R)ths->N[t];
    ths->b[t] = (R)3.1415926535897932384626433832795028841971693993751 *
                ((R)2.0 - (R)1.0 / ths->sigma[t]);  // include/infft.h:216-222
  }
  if (ths->flags & MALLOC_X) ths->x = (R *)Api<R>::mal((size_t)(d * ths->M_total) * sizeof(R));
  if (ths->flags & MALLOC_F_HAT)
    ths->f_hat = (typename Api<R>::cx *)Api<R>::mal((size_t)ths->N_total * 2 * sizeof(R));
  if (ths->flags & MALLOC_F)
    ths->f = (typename Api<R>::cx *)Api<R>::mal((size_t)ths->M_total * 2 * sizeof(R));
  ths->psi = nullptr;
  ths->psi_index_g = nullptr;
  ths->psi_index_f = nullptr;
  ths->g = ths->g_hat = ths->g1 = ths->g2 = nullptr;
  ths->spline_coeffs = nullptr;
  ths->c_phi_inv = nullptr;
  if (ths->flags & PRE_LIN_PSI) {
    if (ths->K == 0) {
      // m2K (kernel/util/window.c:37-41), Kaiser-Bessel table
      static const int m2K_[] = {1, 3, 7, 9, 14, 17, 20, 23, 24};
      int j = (int)std::min<long long>(ths->m, 8);
      ths->K = (NFFT_INT)((1U << m2K_[j]) * (ths->m + 2));
    }
  }
  ths->index_x = (ths->flags & NFFT_SORT_NODES)
                     ? (NFFT_INT *)Api<R>::mal(sizeof(NFFT_INT) * 2U * (size_t)ths->M_total)
                     : nullptr;
  ths->MEASURE_TIME_t[0] = ths->MEASURE_TIME_t[1] = ths->MEASURE_TIME_t[2] = 0;
  Api<R>::set_mv(ths);  // nfft.c:6044-6045

  Ctx<R> *c = new Ctx<R>();
  Geom<R> &g = c->g;
  memset(&g, 0, sizeof(g));
  g.d = d;
  g.m = (int)ths->m;
  g.w = 2 * g.m + 2;
  g.M = ths->M_total;
  g.n_total = ths->n_total;
  g.N_total = ths->N_total;
  g.mm = (R)g.m * (R)g.m;
  for (int t = 0; t < d; ++t) {
    g.n[t] = (int)ths->n[t];
    g.N[t] = (int)ths->N[t];
    g.nR[t] = (R)ths->n[t];
    g.b[t] = ths->b[t];
    if (g.N[t] <= g.m || g.n[t] <= 2 * g.m + 2) c->direct = true;
  }
  for (int t = d; t < GB_MAXD; ++t) {
    g.n[t] = g.N[t] = 1;
    g.nR[t] = 1;
  }
  if (g.w <= KB_POLY_WMAX) {
    c->poly.same = 1;
    for (int t = 0; t < std::min(d, 3); ++t) {
      kb_poly_fit(g.m, (double)ths->b[t], g.w, &c->poly.c[t][0][0]);
      if (ths->b[t] != ths->b[0]) c->poly.same = 0;
    }
    if (std::is_same<R, double>::value && d == 2)
      for (int t = 0; t < 2; ++t) kb_polyd_fit(g.m, (double)ths->b[t], g.w, &c->polyd.c[t][0][0]);
  }
  c->flags = ths->flags;
  choose_tiles<R>(c);

  GB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->own_stream = true;
  for (int i = 0; i < 7; ++i) GB_CUDA(cudaEventCreate(&c->ev[i]));
  const size_t M = (size_t)std::max<long long>(g.M, 1);
  dev_alloc<R>((void **)&c->x_dev, M * d * sizeof(R));
  dev_alloc<R>((void **)&c->fhat_dev, (size_t)g.N_total * sizeof(C));
  dev_alloc<R>((void **)&c->f_dev, M * sizeof(C));
  size_t ncphi = 0;
  for (int t = 0; t < d; ++t) ncphi += g.N[t];
  dev_alloc<R>((void **)&c->cphi, ncphi * sizeof(double));
  if (!c->direct) {
    dev_alloc<R>((void **)&c->grid, (size_t)g.n_total * sizeof(C));
    dev_alloc<R>((void **)&c->xs, M * d * sizeof(R));
    dev_alloc<R>((void **)&c->perm, M * sizeof(uint32_t));
    dev_alloc<R>((void **)&c->tile_start, ((size_t)c->ntiles + 1) * sizeof(uint32_t));
    const int chunk = std::min(item_chunk(c), 1024);  // the item buffers hold any chunk >= this
    dev_alloc<R>((void **)&c->items, ((size_t)c->ntiles + M / chunk + 2) * sizeof(WorkItem));
    c->col3 = c->group3 && sizeof(R) == 4 && group3_column_supported<R>(g.w);
    if (c->col3) {
      const size_t cap = (size_t)c->ntiles + M / chunk + 2;
      dev_alloc<R>((void **)&c->c3rec, M * sizeof(float4));
      dev_alloc<R>((void **)&c->c3cst, cap * 17 * sizeof(uint16_t));
      dev_alloc<R>((void **)&c->c3sst, cap * 65 * sizeof(uint16_t));
      c->grid_map_ok = encode_grid_map(&c->grid_map, c->grid, g.n, g.ext[0], col3_box_ext_y(g.w));
    }
    if (c->col2 && sizeof(R) == 4)
      c->grid_map2_ok = encode_grid_map_2d(&c->grid_map2, c->grid, g.n, 32 + g.w - 1, col2_box_zb(g.w));
    make_fft<R>(c);
  }
  launch_cphi<R>(g, c->cphi, c->stream);
  if (ths->flags & PRE_PHI_HUT) {
    ths->c_phi_inv = (R **)Api<R>::mal((size_t)d * sizeof(R *));
    double *tmp = (double *)malloc(ncphi * sizeof(double));
    GB_CUDA(cudaMemcpyAsync(tmp, c->cphi, ncphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GB_CUDA(cudaStreamSynchronize(c->stream));
    size_t off = 0;
    for (int t = 0; t < d; ++t) {
      ths->c_phi_inv[t] = (R *)Api<R>::mal((size_t)g.N[t] * sizeof(R));
      for (int k = 0; k < g.N[t]; ++k) ths->c_phi_inv[t][k] = (R)tmp[off + k];
      off += g.N[t];
    }
    free(tmp);
  }
  ths->my_fftw_plan1 = reinterpret_cast<decltype(ths->my_fftw_plan1)>(c);
  ths->my_fftw_plan2 = reinterpret_cast<decltype(ths->my_fftw_plan2)>(c);
}

// ------------------------------------------------------------ node set-up
template <typename R>
static void nodes_from_device(typename Api<R>::plan *ths, Ctx<R> *c)
{
  Geom<R> &g = c->g;
  const long long M = g.M;
  cudaStream_t s = c->stream;
  const bool want_index = (ths->flags & NFFT_SORT_NODES) && ths->index_x && M > 0;
  ++c->gen;
  if (c->direct && !want_index) {
    c->nodes_ready = true;
    return;
  }
  // scratch for keys and the sort
  const size_t Mz = (size_t)std::max<long long>(M, 1);
  uint32_t *k1, *v1, *k2, *v2, *rk;
  dev_alloc<R>((void **)&k1, Mz * 4);
  dev_alloc<R>((void **)&v1, Mz * 4);
  dev_alloc<R>((void **)&k2, Mz * 4);
  dev_alloc<R>((void **)&v2, Mz * 4);
  dev_alloc<R>((void **)&rk, Mz * 4);
  const size_t tb = std::max(radix_temp_bytes(Mz), scan_temp_bytes((size_t)c->ntiles + 1)) + 1024;
  void *temp;
  dev_alloc<R>(&temp, tb);
  launch_node_keys<R>(c->x_dev, g, k1, want_index ? rk : nullptr, v1, s);
  if (want_index) {
    // reference order: stable sort of (key, j) by key (nfft.c:75-109)
    if (g.n_total > 0xffffffffLL) fatal("NFFT_SORT_NODES needs n_total < 2^32");
    uint32_t *idx;
    dev_alloc<R>((void **)&idx, Mz * 4);
    GB_CUDA(cudaMemcpyAsync(idx, v1, Mz * 4, cudaMemcpyDeviceToDevice, s));
    // rhigh = ceil(log2(n_total)) - 1 (nfft.c:100); sorting all those bits
    radix_sort_pairs(rk, idx, k2, v2, (size_t)M, std::max(ceil_log2(g.n_total), 1), temp, s);
    long long *pairs;
    dev_alloc<R>((void **)&pairs, (size_t)M * 16);
    launch_ref_index_to_int64(rk, idx, M, pairs, s);
    static_assert(sizeof(NFFT_INT) == 8, "NFFT_INT must be 64-bit");
    GB_CUDA(cudaMemcpyAsync(ths->index_x, pairs, (size_t)M * 16, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    GB_CUDA(cudaFree(pairs));
    GB_CUDA(cudaFree(idx));
  }
  if (!c->direct) {
    // tile order used by the transform kernels
    radix_sort_pairs(k1, v1, k2, v2, (size_t)M, std::max(ceil_log2((long long)c->ntiles * g.sub), 1),
                     temp, s);
    GB_CUDA(cudaMemcpyAsync(c->perm, v1, Mz * 4, cudaMemcpyDeviceToDevice, s));
    launch_gather_x<R>(c->x_dev, c->perm, c->xs, g, s);
    launch_tile_starts(k1, M, c->ntiles, (uint32_t)g.sub, c->tile_start, s);
    uint32_t *cnt = k2, *off = v2;  // reuse (>= ntiles entries needed)
    uint32_t *total;
    dev_alloc<R>((void **)&total, 16);
    if ((size_t)c->ntiles > Mz) {
      dev_alloc<R>((void **)&cnt, (size_t)c->ntiles * 4);
      dev_alloc<R>((void **)&off, (size_t)c->ntiles * 4);
    }
    const int chunk = item_chunk(c);
    c->nitems = c->tiled ? build_work_items(c->tile_start, c->ntiles, chunk, c->items, cnt, off,
                                            total, temp, s)
                         : 0;
    if constexpr (std::is_same<R, float>::value)
      if (c->col3) launch_c3_setup(c->xs, g, c->items, c->nitems, k1, c->c3rec, c->c3cst, c->c3sst, s);
    // dense work items favour B by sub-cell units (per-unit work shared by
    // more nodes), sparse ones B by column segments
    if (cnt != k2) {
      GB_CUDA(cudaFree(cnt));
      GB_CUDA(cudaFree(off));
    }
    GB_CUDA(cudaFree(total));
  }
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaFree(k1));
  GB_CUDA(cudaFree(v1));
  GB_CUDA(cudaFree(k2));
  GB_CUDA(cudaFree(v2));
  GB_CUDA(cudaFree(rk));
  GB_CUDA(cudaFree(temp));
  c->nodes_ready = true;
}

template <typename R>
static void upload_x(typename Api<R>::plan *ths, Ctx<R> *c)
{
  if (c->g.M == 0) return;
  if (!ths->x) fatal("member x not initialized");
  GB_CUDA(cudaMemcpyAsync(c->x_dev, ths->x, (size_t)c->g.M * c->g.d * sizeof(R),
                          cudaMemcpyHostToDevice, c->stream));
}

template <typename R>
static void precompute(typename Api<R>::plan *ths)
{
  Ctx<R> *c = ctx_of<R>(ths);
  upload_x<R>(ths, c);
  nodes_from_device<R>(ths, c);
}

// Without any PRE_*PSI flag the reference evaluates the window and sorts the
// nodes inside every B call (nfft.c:1231-1268); mirror that by refreshing the
// node set-up per transform.  With a precompute flag the state of the last
// precompute_one_psi call is used, as the reference uses its psi table.
template <typename R>
static void ensure_nodes(typename Api<R>::plan *ths, Ctx<R> *c)
{
  if (!(ths->flags & PRE_ONE_PSI) || !c->nodes_ready) precompute<R>(ths);
}

// ------------------------------------------------------------ transforms
// Events: ev[0] call start, ev[1] stage 1 start, ev[6] after the grid
// memset of B^T, ev[2] stage 1 end, ev[3] FFT end, ev[4] stage 3 end,
// ev[5] call end (after the result copy).
template <typename R>
static Col3Bufs col3_bufs(Ctx<R> *c)
{
  Col3Bufs b;
  b.rec = c->c3rec;
  b.cst = c->c3cst;
  b.sst = c->c3sst;
  b.grid_map = c->grid_map_ok ? &c->grid_map : nullptr;
  // column segments unless the sub-cell form is asked for (measured on GB300
  // at 2^24 nodes, 128^3 / 256^3, m = 4: the column form is as fast or faster
  // from uniform nodes (3.58 against 3.97 ms) to 32 tight clusters of spread
  // 0.005 (3.16 against 3.20 ms))
  b.b_column = c->b3mode != 2;
  return b;
}

// the 2-D column B where the plan selected it (double precision: a per-node
// gather on the same work items, whose FP64 arithmetic is the smaller); false
// otherwise
template <typename R>
static bool b2_stage(Ctx<R> *c, typename Cx<R>::T *f)
{
  if (!c->col2) return false;
  if constexpr (std::is_same<R, float>::value)
    launch_b2_col(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->poly, c->stream,
                  c->grid_map2_ok ? &c->grid_map2 : nullptr);
  else
    launch_b2_node_d(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->polyd, c->stream);
  return true;
}

template <typename R>
static void b_stage(Ctx<R> *c, typename Cx<R>::T *f)
{
  if (c->group3) launch_b3_group<R>(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->poly, col3_bufs(c), c->stream);
  else if (b2_stage(c, f)) return;
  else if (c->tiled) launch_b_tiled<R>(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->stream);
  else launch_b_generic<R>(c->grid, c->xs, c->perm, f, c->g, c->stream);
}

template <typename R>
static cudaEvent_t *events_for_call(Ctx<R> *c, bool trafo)
{
  if (c->ring_on && c->ring_used < c->ring_slots) {
    c->ring_kind[c->ring_used] = trafo ? 1 : 0;
    return &c->ring[7 * (size_t)c->ring_used++];
  }
  return c->ev;
}

// the 2-D column B^T where the plan selected it; false otherwise
template <typename R>
static bool bt2_stage(Ctx<R> *c, const typename Cx<R>::T *f)
{
  if (!c->col2) return false;
  if constexpr (std::is_same<R, float>::value) {
    float2 *lo = nullptr;
    if (c->comp == 1) {
      if (!c->grid_lo) dev_alloc<R>(&c->grid_lo, (size_t)c->g.n_total * sizeof(float2));
      lo = (float2 *)c->grid_lo;
      GB_CUDA(cudaMemsetAsync(lo, 0, (size_t)c->g.n_total * sizeof(float2), c->stream));
    }
    launch_bt2_col(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->poly, c->stream, lo);
  } else
    launch_bt2_col_d(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->polyd, c->stream);
  return true;
}

template <typename R>
static void bt_stage(Ctx<R> *c, const typename Cx<R>::T *f, cudaEvent_t *E)
{
  GB_CUDA(cudaMemsetAsync(c->grid, 0, (size_t)c->g.n_total * sizeof(typename Cx<R>::T), c->stream));
  GB_CUDA(cudaEventRecord(E[6], c->stream));
  if (c->group3) launch_bt3_group<R>(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->poly, col3_bufs(c), c->stream);
  else if (bt2_stage(c, f)) return;
  else if (c->tiled) launch_bt_tiled<R>(c->items, c->nitems, c->grid, c->xs, c->perm, f, c->g, c->stream);
  else launch_bt_generic<R>(c->grid, c->xs, c->perm, f, c->g, c->stream);
}

// f = A fhat, device vectors
template <typename R>
static void trafo_device(Ctx<R> *c, const typename Cx<R>::T *fhat, typename Cx<R>::T *f)
{
  c->last_trafo = true;
  c->timed = !c->direct;
  if (c->direct) {
    launch_ndft_trafo<R>(c->x_dev, fhat, f, c->g, c->stream);
    c->launches = 1;
    return;
  }
  cudaEvent_t *E = events_for_call(c, true);
  GB_CUDA(cudaEventRecord(E[1], c->stream));
  launch_d_pad<R>(fhat, c->cphi, c->grid, c->g, c->stream);
  GB_CUDA(cudaEventRecord(E[2], c->stream));
  run_fft<R>(c, CUFFT_FORWARD);
  GB_CUDA(cudaEventRecord(E[3], c->stream));
  b_stage<R>(c, f);
  GB_CUDA(cudaEventRecord(E[4], c->stream));
  c->launches = 2;
}

// fhat = A^H f, device vectors
template <typename R>
static void adjoint_device(Ctx<R> *c, const typename Cx<R>::T *f, typename Cx<R>::T *fhat)
{
  c->last_trafo = false;
  c->timed = !c->direct;
  if (c->direct) {
    launch_ndft_adjoint<R>(c->x_dev, f, fhat, c->g, c->stream);
    c->launches = 1;
    return;
  }
  cudaEvent_t *E = events_for_call(c, false);
  GB_CUDA(cudaEventRecord(E[1], c->stream));
  bt_stage<R>(c, f, E);
  GB_CUDA(cudaEventRecord(E[2], c->stream));
  run_fft<R>(c, CUFFT_INVERSE);
  GB_CUDA(cudaEventRecord(E[3], c->stream));
  launch_d_crop<R>(c->grid, c->cphi, fhat, c->g, c->stream);
  GB_CUDA(cudaEventRecord(E[4], c->stream));
  c->launches = 2;
}

// Stage times of the last transform (the caller has synchronised or the
// events are waited on here): [0] D or D^T, [1] FFT, [2] B or B^T (kernel
// only, without the grid memset), [3] the rest of the call (copies, memset).
template <typename R>
static void stage_times(Ctx<R> *c, bool host_call)
{
  if (!c->timed) {
    for (int i = 0; i < 4; ++i) c->stage_ms[i] = 0;
    return;
  }
  GB_CUDA(cudaEventSynchronize(c->ev[host_call ? 5 : 4]));
  float a = 0, b = 0, d = 0, tot = 0, ms = 0;
  GB_CUDA(cudaEventElapsedTime(&a, c->ev[1], c->ev[2]));
  GB_CUDA(cudaEventElapsedTime(&b, c->ev[2], c->ev[3]));
  GB_CUDA(cudaEventElapsedTime(&d, c->ev[3], c->ev[4]));
  if (!c->last_trafo) GB_CUDA(cudaEventElapsedTime(&ms, c->ev[1], c->ev[6]));
  if (host_call) GB_CUDA(cudaEventElapsedTime(&tot, c->ev[0], c->ev[5]));
  else GB_CUDA(cudaEventElapsedTime(&tot, c->ev[1], c->ev[4]));
  c->stage_ms[0] = c->last_trafo ? a : d;
  c->stage_ms[1] = b;
  c->stage_ms[2] = c->last_trafo ? d : a - ms;
  c->stage_ms[3] = std::max(0.0f, tot - a - b - d + ms);
}

// Per-call event ring: time a sequence of device transforms on the plan's
// stream without synchronising between them.
template <typename R>
static int timing_begin(Ctx<R> *c, int max_calls)
{
  GB_CUDA(cudaStreamSynchronize(c->stream));
  if (max_calls > c->ring_slots) {
    for (int i = 7 * c->ring_slots; i < 7 * max_calls; ++i) {
      cudaEvent_t e;
      GB_CUDA(cudaEventCreate(&e));
      c->ring.push_back(e);
    }
    c->ring_slots = max_calls;
    c->ring_kind.resize(max_calls);
  }
  c->ring_used = 0;
  c->ring_on = true;
  return 0;
}

// sums[7] (ms): trafo D, trafo FFT, trafo B, adjoint memset, adjoint B^T,
// adjoint FFT, adjoint D^T; counts[2]: trafo calls, adjoint calls
template <typename R>
static int timing_end(Ctx<R> *c, float *sums, int *counts)
{
  c->ring_on = false;
  for (int i = 0; i < 7; ++i) sums[i] = 0;
  counts[0] = counts[1] = 0;
  for (int k = 0; k < c->ring_used; ++k) {
    cudaEvent_t *E = &c->ring[7 * (size_t)k];
    GB_CUDA(cudaEventSynchronize(E[4]));
    float a = 0, b = 0, d = 0, ms = 0;
    GB_CUDA(cudaEventElapsedTime(&a, E[1], E[2]));
    GB_CUDA(cudaEventElapsedTime(&b, E[2], E[3]));
    GB_CUDA(cudaEventElapsedTime(&d, E[3], E[4]));
    if (c->ring_kind[k]) {
      sums[0] += a;
      sums[1] += b;
      sums[2] += d;
      counts[0]++;
    } else {
      GB_CUDA(cudaEventElapsedTime(&ms, E[1], E[6]));
      sums[3] += ms;
      sums[4] += a - ms;
      sums[5] += b;
      sums[6] += d;
      counts[1]++;
    }
  }
  return c->ring_used;
}

template <typename R>
static void finish_times(typename Api<R>::plan *ths, Ctx<R> *c)
{
  stage_times<R>(c, true);
  // MEASURE_TIME_t[0] = D, [1] = FFT, [2] = B, in seconds (include/infft.h:1376-1410)
  ths->MEASURE_TIME_t[0] = (R)(c->stage_ms[0] * 1e-3);
  ths->MEASURE_TIME_t[1] = (R)(c->stage_ms[1] * 1e-3);
  ths->MEASURE_TIME_t[2] = (R)(c->stage_ms[2] * 1e-3);
}

template <typename R>
static void trafo(typename Api<R>::plan *ths)
{
  typedef typename Cx<R>::T C;
  Ctx<R> *c = ctx_of<R>(ths);
  if (c->direct) upload_x<R>(ths, c);
  ensure_nodes<R>(ths, c);
  GB_CUDA(cudaEventRecord(c->ev[0], c->stream));
  if (c->g.N_total > 0)
    GB_CUDA(cudaMemcpyAsync(c->fhat_dev, ths->f_hat, (size_t)c->g.N_total * sizeof(C),
                            cudaMemcpyHostToDevice, c->stream));
  trafo_device<R>(c, c->fhat_dev, c->f_dev);
  if (c->g.M > 0)
    GB_CUDA(cudaMemcpyAsync(ths->f, c->f_dev, (size_t)c->g.M * sizeof(C), cudaMemcpyDeviceToHost,
                            c->stream));
  GB_CUDA(cudaEventRecord(c->ev[5], c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  finish_times<R>(ths, c);
}

template <typename R>
static void adjoint(typename Api<R>::plan *ths)
{
  typedef typename Cx<R>::T C;
  Ctx<R> *c = ctx_of<R>(ths);
  if (c->direct) upload_x<R>(ths, c);
  ensure_nodes<R>(ths, c);
  GB_CUDA(cudaEventRecord(c->ev[0], c->stream));
  if (c->g.M > 0)
    GB_CUDA(cudaMemcpyAsync(c->f_dev, ths->f, (size_t)c->g.M * sizeof(C), cudaMemcpyHostToDevice,
                            c->stream));
  adjoint_device<R>(c, c->f_dev, c->fhat_dev);
  if (c->g.N_total > 0)
    GB_CUDA(cudaMemcpyAsync(ths->f_hat, c->fhat_dev, (size_t)c->g.N_total * sizeof(C),
                            cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaEventRecord(c->ev[5], c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  finish_times<R>(ths, c);
}

template <typename R>
static void trafo_direct(const typename Api<R>::plan *ths)
{
  typedef typename Cx<R>::T C;
  Ctx<R> *c = ctx_of<R>(ths);
  upload_x<R>(const_cast<typename Api<R>::plan *>(ths), c);
  if (c->g.N_total > 0)
    GB_CUDA(cudaMemcpyAsync(c->fhat_dev, ths->f_hat, (size_t)c->g.N_total * sizeof(C),
                            cudaMemcpyHostToDevice, c->stream));
  launch_ndft_trafo<R>(c->x_dev, c->fhat_dev, c->f_dev, c->g, c->stream);
  if (c->g.M > 0)
    GB_CUDA(cudaMemcpyAsync(ths->f, c->f_dev, (size_t)c->g.M * sizeof(C), cudaMemcpyDeviceToHost,
                            c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
}

template <typename R>
static void adjoint_direct(const typename Api<R>::plan *ths)
{
  typedef typename Cx<R>::T C;
  Ctx<R> *c = ctx_of<R>(ths);
  upload_x<R>(const_cast<typename Api<R>::plan *>(ths), c);
  if (c->g.M > 0)
    GB_CUDA(cudaMemcpyAsync(c->f_dev, ths->f, (size_t)c->g.M * sizeof(C), cudaMemcpyHostToDevice,
                            c->stream));
  launch_ndft_adjoint<R>(c->x_dev, c->f_dev, c->fhat_dev, c->g, c->stream);
  if (c->g.N_total > 0)
    GB_CUDA(cudaMemcpyAsync(ths->f_hat, c->fhat_dev, (size_t)c->g.N_total * sizeof(C),
                            cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
}

template <typename R>
static const char *check(typename Api<R>::plan *ths)
{
  // nfft.c:6169-6207
  if (!ths->f) return "Member f not initialized.";
  if (!ths->x) return "Member x not initialized.";
  if (!ths->f_hat) return "Member f_hat not initialized.";
  if ((ths->flags & PRE_LIN_PSI) && ths->K < ths->M_total)
    return "Number of nodes too small to use PRE_LIN_PSI.";
  for (NFFT_INT j = 0; j < ths->M_total * ths->d; j++)
    if ((ths->x[j] < (R)-0.5) || (ths->x[j] >= (R)0.5)) return "ths->x out of range [-0.5,0.5)";
  for (NFFT_INT j = 0; j < ths->d; j++) {
    if (ths->sigma[j] <= 1) return "Oversampling factor too small";
    if (ths->N[j] % 2 == 1) return "polynomial degree N has to be even";
  }
  return 0;
}

template <typename R>
static void finalize(typename Api<R>::plan *ths)
{
  Ctx<R> *c = reinterpret_cast<Ctx<R> *>(ths->my_fftw_plan1);
  if (c) {
    cudaStreamSynchronize(c->stream);
    if (c->fft_ok) {
      cufftDestroy(c->fft_main);
      for (int t = 0; t < c->fft_lead; ++t) cufftDestroy(c->fft_lead_plan[t]);
    }
    cudaFree(c->x_dev);
    cudaFree(c->xs);
    cudaFree(c->perm);
    cudaFree(c->grid);
    cudaFree(c->grid_lo);
    cudaFree(c->fhat_dev);
    cudaFree(c->f_dev);
    cudaFree(c->cphi);
    cudaFree(c->tile_start);
    cudaFree(c->items);
    cudaFree(c->c3rec);
    cudaFree(c->c3cst);
    cudaFree(c->c3sst);
    for (int i = 0; i < 7; ++i)
      if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (cudaEvent_t e : c->ring) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    ths->my_fftw_plan1 = nullptr;
    ths->my_fftw_plan2 = nullptr;
  }
  // nfft.c:6209-6270: free what init allocated
  if (ths->index_x) Api<R>::fre(ths->index_x);
  if (ths->c_phi_inv) {
    for (NFFT_INT t = 0; t < ths->d; ++t) Api<R>::fre(ths->c_phi_inv[t]);
    Api<R>::fre(ths->c_phi_inv);
  }
  if (ths->flags & MALLOC_F) Api<R>::fre(ths->f);
  if (ths->flags & MALLOC_F_HAT) Api<R>::fre(ths->f_hat);
  if (ths->flags & MALLOC_X) Api<R>::fre(ths->x);
  Api<R>::fre(ths->b);
  Api<R>::fre(ths->sigma);
  Api<R>::fre(ths->n);
  Api<R>::fre(ths->N);
  ths->index_x = nullptr;
  ths->c_phi_inv = nullptr;
}

template <typename R>
static void init_guru(typename Api<R>::plan *ths, int d, int *N, int M, int *n, int m,
                      unsigned flags, unsigned fftw_flags)
{
  ths->d = d;
  ths->M_total = M;
  ths->N = (NFFT_INT *)Api<R>::mal((size_t)d * sizeof(NFFT_INT));
  ths->n = (NFFT_INT *)Api<R>::mal((size_t)d * sizeof(NFFT_INT));
  for (int t = 0; t < d; ++t) {
    ths->N[t] = N[t];
    ths->n[t] = n[t];
  }
  ths->m = m;
  ths->flags = flags;
  ths->fftw_flags = fftw_flags;
  ths->K = 0;
  init_help<R>(ths);
}

// nfft_init defaults (nfft.c:6048-6087): n = 2 next_pow2(N), default m, and
// the default flags of an OpenMP build for d > 1.
template <typename R>
static void init_default(typename Api<R>::plan *ths, int d, int *N, int M, int mdef)
{
  int n[GB_MAXD];
  for (int t = 0; t < d && t < GB_MAXD; ++t) n[t] = 2 * (int)nfft_next_power_of_2(N[t]);
  unsigned flags = (d > 1) ? (PRE_PHI_HUT | PRE_PSI | MALLOC_X | MALLOC_F_HAT | MALLOC_F |
                              FFTW_INIT | NFFT_SORT_NODES | NFFT_OMP_BLOCKWISE_ADJOINT)
                           : (PRE_PHI_HUT | PRE_PSI | MALLOC_X | MALLOC_F_HAT | MALLOC_F |
                              FFTW_INIT | FFT_OUT_OF_PLACE);
  init_guru<R>(ths, d, N, M, n, mdef, flags, FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
}

// ------------------------------------------------------------ extensions
// mode 1 (on) / 0 (off, the default) / -1 (the default) for the compensated
// single-precision 2-D column B^T; -1 returned where the plan runs no such kernel
template <typename R>
static int set_compensated(typename Api<R>::plan *ths, int mode)
{
  Ctx<R> *c = ctx_of<R>(ths);
  if (!std::is_same<R, float>::value || c->g.d != 2 || c->direct || !c->col2 || mode < -1 || mode > 1) return -1;
  c->comp = mode == 1 ? 1 : 0;
  return 0;
}

// mode 0 (the default) or 1 (column segments), or 2 (sub-cell units) for the
// 3-D single-precision B; -1 returned where the plan runs no such kernel
template <typename R>
static int set_b3_kernel(typename Api<R>::plan *ths, int mode)
{
  Ctx<R> *c = ctx_of<R>(ths);
  if (!std::is_same<R, float>::value || c->direct || !c->col3 || mode < 0 || mode > 2) return -1;
  c->b3mode = mode;
  return 0;
}

// the B kernel the plan runs now: 1 column segments, 2 sub-cell units, -1 none
// of these
template <typename R>
static int b3_kernel(typename Api<R>::plan *ths)
{
  Ctx<R> *c = ctx_of<R>(ths);
  if (!std::is_same<R, float>::value || c->direct || !c->col3) return -1;
  return col3_bufs(c).b_column ? 1 : 2;
}

template <typename R>
static int set_stream(typename Api<R>::plan *ths, void *stream)
{
  Ctx<R> *c = ctx_of<R>(ths);
  cudaStreamSynchronize(c->stream);
  if (c->own_stream) {
    cudaStreamDestroy(c->stream);
    c->own_stream = false;
  }
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    GB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return 0;
}

}  // namespace gb

using namespace gb;

extern "C" {

#define GB_PLAN_API(X, R, MDEF)                                                                    \
  void X##init_guru(X##plan *ths, int d, int *N, int M, int *n, int m, unsigned flags,             \
                    unsigned fftw_flags)                                                           \
  {                                                                                                \
    init_guru<R>(ths, d, N, M, n, m, flags, fftw_flags);                                           \
  }                                                                                                \
  void X##init_lin(X##plan *ths, int d, int *N, int M, int *n, int m, int K, unsigned flags,       \
                   unsigned fftw_flags)                                                            \
  {                                                                                                \
    ths->d = d;                                                                                    \
    ths->M_total = M;                                                                              \
    ths->N = (NFFT_INT *)Api<R>::mal((size_t)d * sizeof(NFFT_INT));                                \
    ths->n = (NFFT_INT *)Api<R>::mal((size_t)d * sizeof(NFFT_INT));                                \
    for (int t = 0; t < d; ++t) {                                                                  \
      ths->N[t] = N[t];                                                                            \
      ths->n[t] = n[t];                                                                            \
    }                                                                                              \
    ths->m = m;                                                                                    \
    ths->flags = flags;                                                                            \
    ths->fftw_flags = fftw_flags;                                                                  \
    ths->K = K;                                                                                    \
    init_help<R>(ths);                                                                             \
  }                                                                                                \
  void X##init(X##plan *ths, int d, int *N, int M) { init_default<R>(ths, d, N, M, MDEF); }        \
  void X##init_1d(X##plan *ths, int N1, int M)                                                     \
  {                                                                                                \
    int N[1] = {N1};                                                                               \
    init_default<R>(ths, 1, N, M, MDEF);                                                           \
  }                                                                                                \
  void X##init_2d(X##plan *ths, int N1, int N2, int M)                                             \
  {                                                                                                \
    int N[2] = {N1, N2};                                                                           \
    init_default<R>(ths, 2, N, M, MDEF);                                                           \
  }                                                                                                \
  void X##init_3d(X##plan *ths, int N1, int N2, int N3, int M)                                     \
  {                                                                                                \
    int N[3] = {N1, N2, N3};                                                                       \
    init_default<R>(ths, 3, N, M, MDEF);                                                           \
  }                                                                                                \
  void X##precompute_one_psi(X##plan *ths) { precompute<R>(ths); }                                 \
  void X##precompute_psi(X##plan *ths) { precompute<R>(ths); }                                     \
  void X##precompute_full_psi(X##plan *ths) { precompute<R>(ths); }                                \
  void X##precompute_fg_psi(X##plan *ths) { precompute<R>(ths); }                                  \
  void X##precompute_lin_psi(X##plan *ths) { precompute<R>(ths); }                                 \
  void X##trafo(X##plan *ths) { trafo<R>(ths); }                                                   \
  void X##adjoint(X##plan *ths) { adjoint<R>(ths); }                                               \
  void X##trafo_1d(X##plan *ths) { trafo<R>(ths); }                                                \
  void X##trafo_2d(X##plan *ths) { trafo<R>(ths); }                                                \
  void X##trafo_3d(X##plan *ths) { trafo<R>(ths); }                                                \
  void X##adjoint_1d(X##plan *ths) { adjoint<R>(ths); }                                            \
  void X##adjoint_2d(X##plan *ths) { adjoint<R>(ths); }                                            \
  void X##adjoint_3d(X##plan *ths) { adjoint<R>(ths); }                                            \
  void X##trafo_direct(const X##plan *ths) { trafo_direct<R>(ths); }                               \
  void X##adjoint_direct(const X##plan *ths) { adjoint_direct<R>(ths); }                           \
  const char *X##check(X##plan *ths) { return check<R>(ths); }                                     \
  void X##finalize(X##plan *ths) { finalize<R>(ths); }                                             \
  int X##gb_set_stream(X##plan *ths, void *stream) { return set_stream<R>(ths, stream); }          \
  int X##gb_set_compensated(X##plan *ths, int mode) { return set_compensated<R>(ths, mode); }      \
  int X##gb_set_b3_kernel(X##plan *ths, int mode) { return set_b3_kernel<R>(ths, mode); }          \
  int X##gb_b3_kernel(X##plan *ths) { return b3_kernel<R>(ths); }                                    \
  void *X##gb_get_stream(X##plan *ths) { return (void *)ctx_of<R>(ths)->stream; }                  \
  void *X##gb_device_f_hat(X##plan *ths) { return (void *)ctx_of<R>(ths)->fhat_dev; }              \
  void *X##gb_device_f(X##plan *ths) { return (void *)ctx_of<R>(ths)->f_dev; }                     \
  void *X##gb_device_x(X##plan *ths) { return (void *)ctx_of<R>(ths)->x_dev; }                     \
  void X##gb_precompute_device(X##plan *ths)                                                       \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    nodes_from_device<R>(ths, c);                                                                  \
  }                                                                                                \
  void X##gb_trafo_device(X##plan *ths)                                                            \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    if (!c->nodes_ready) nodes_from_device<R>(ths, c);                                             \
    trafo_device<R>(c, c->fhat_dev, c->f_dev);                                                     \
  }                                                                                                \
  void X##gb_adjoint_device(X##plan *ths)                                                          \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    if (!c->nodes_ready) nodes_from_device<R>(ths, c);                                             \
    adjoint_device<R>(c, c->f_dev, c->fhat_dev);                                                   \
  }                                                                                                \
  void X##gb_trafo_ptr(X##plan *ths, const void *f_hat_dev, void *f_dev)                           \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    if (!c->nodes_ready) nodes_from_device<R>(ths, c);                                             \
    trafo_device<R>(c, (const Cx<R>::T *)f_hat_dev, (Cx<R>::T *)f_dev);                            \
  }                                                                                                \
  void X##gb_adjoint_ptr(X##plan *ths, const void *f_dev, void *f_hat_dev)                         \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    if (!c->nodes_ready) nodes_from_device<R>(ths, c);                                             \
    adjoint_device<R>(c, (const Cx<R>::T *)f_dev, (Cx<R>::T *)f_hat_dev);                          \
  }                                                                                                \
  void X##gb_stage_times(X##plan *ths, float *ms4)                                                 \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    for (int i = 0; i < 4; ++i) ms4[i] = c->stage_ms[i];                                           \
  }                                                                                                \
  void X##gb_device_stage_times(X##plan *ths, float *ms4)                                          \
  {                                                                                                \
    Ctx<R> *c = ctx_of<R>(ths);                                                                    \
    stage_times<R>(c, false);                                                                      \
    for (int i = 0; i < 4; ++i) ms4[i] = c->stage_ms[i];                                           \
  }                                                                                                \
  int X##gb_last_launch_count(X##plan *ths) { return ctx_of<R>(ths)->launches; }                  \
  unsigned long long X##gb_generation(X##plan *ths) { return ctx_of<R>(ths)->gen; }              \
  int X##gb_timing_begin(X##plan *ths, int max_calls) { return timing_begin<R>(ctx_of<R>(ths), max_calls); } \
  int X##gb_timing_end(X##plan *ths, float *sums7, int *counts2)                                    \
  {                                                                                                \
    return timing_end<R>(ctx_of<R>(ths), sums7, counts2);                                          \
  }

GB_PLAN_API(nfft_, double, 8)
GB_PLAN_API(nfftf_, float, 4)

}  // extern "C"


namespace gb {

bool plan_view_f(void *pp, PlanViewF *v)
{
  nfftf_plan *p = reinterpret_cast<nfftf_plan *>(pp);
  Ctx<float> *c = ctx_of<float>(p);
  v->g = c->g;
  v->xs = c->xs;
  v->perm = c->perm;
  v->cphi = c->cphi;
  v->items = c->items;
  v->nitems = c->nitems;
  v->fhat = c->fhat_dev;
  v->f = c->f_dev;
  v->tiled = c->tiled;
  v->group3 = c->group3;
  v->direct = c->direct;
  v->ready = c->nodes_ready;
  v->col2 = c->col2;
  v->poly = &c->poly;
  v->stream = c->stream;
  v->c3 = col3_bufs<float>(c);
  v->grid = c->grid;
  return true;
}

void plan_retile_f(void *pp, int T)
{
  nfftf_plan *p = reinterpret_cast<nfftf_plan *>(pp);
  Ctx<float> *c = ctx_of<float>(p);
  if (c->g.d != 2 || c->direct) return;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  c->force_T = T;
  choose_tiles<float>(c);
  GB_CUDA(cudaFree(c->tile_start));
  GB_CUDA(cudaFree(c->items));
  const size_t M = (size_t)std::max<long long>(c->g.M, 1);
  dev_alloc<float>((void **)&c->tile_start, ((size_t)c->ntiles + 1) * sizeof(uint32_t));
  dev_alloc<float>((void **)&c->items, ((size_t)c->ntiles + M / std::min(item_chunk(c), 1024) + 2) * sizeof(WorkItem));
  nodes_from_device<float>(p, c);
}

}  // namespace gb
