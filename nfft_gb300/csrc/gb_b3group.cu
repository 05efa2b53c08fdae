// gb_b3group.cu -- instantiations and launchers of the 3-D sub-cell group
// kernels (see gb_b3group.cuh).
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "gb_b3group.cuh"
#include "gb_col3.cuh"

namespace gb {

int col3_box_ext_y(int w)
{
  return w == 10 ? Box3<10>::EXTY : 8 + w - 1;
}

unsigned long long read_wait_timeouts()
{
  unsigned long long v = 0, z = 0;
  GB_CUDA(cudaMemcpyFromSymbol(&v, g_tma_wait_timeouts, sizeof(v)));
  GB_CUDA(cudaMemcpyToSymbol(g_tma_wait_timeouts, &z, sizeof(z)));
  return v;
}

static constexpr int G3_CS = 2;  // sub-cell edge

template <typename R, int W>
static void run_g3(bool adjoint, const WorkItem *items, int nitems, typename Cx<R>::T *grid,
                   const R *xs, const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g,
                   const WinPoly &poly, const Col3Bufs &cb, cudaStream_t s)
{
  (void)poly;
  if constexpr (std::is_same<R, float>::value && W == 10) {
    // the grid's TMA view (a zeroed map and use_tma = 0 where there is none)
    CUtensorMap gmap;
    memset(&gmap, 0, sizeof(gmap));
    const int use_tma = cb.grid_map ? 1 : 0;
    if (use_tma) gmap = *cb.grid_map;
    if (adjoint) {
      set_smem_limit((const void *)k_bt3_col<W>, c3_smem_bytes<W>());
      k_bt3_col<W><<<nitems, C3_THREADS, c3_smem_bytes<W>(), s>>>(items, grid, cb.rec, cb.cst, perm, f, g, poly,
                                                                  gmap, use_tma);
      GB_LAUNCHED("bt3_col");
      return;
    }
    if (cb.b_column) {
      set_smem_limit((const void *)k_b3_col<W>, cb_smem_bytes<W>());
      k_b3_col<W><<<nitems, C3_THREADS, cb_smem_bytes<W>(), s>>>(items, grid, cb.rec, cb.cst, perm, f, g, poly, gmap,
                                                                 use_tma);
      GB_LAUNCHED("b3_col");
      return;
    }
    set_smem_limit((const void *)k_b3_cell<W>, s3_smem_bytes<W>(g));
    k_b3_cell<W><<<nitems, C3_THREADS, s3_smem_bytes<W>(g), s>>>(items, grid, cb.rec, cb.sst, perm, f, g, poly,
                                                                 gmap, use_tma);
    GB_LAUNCHED("b3_cell");
    return;
  }
  const size_t smem = adjoint ? g3_smem_bytes<R, W, G3_CS, true>(g) : g3_smem_bytes<R, W, G3_CS, false>(g);
  if (adjoint) {
    set_smem_limit((const void *)k_bt3_group<R, W, G3_CS>, smem);
    k_bt3_group<R, W, G3_CS><<<nitems, G3_THREADS, smem, s>>>(items, grid, xs, perm, f, g);
    GB_LAUNCHED("bt3_group");
  } else {
    set_smem_limit((const void *)k_b3_group<R, W, G3_CS>, smem);
    k_b3_group<R, W, G3_CS><<<nitems, G3_THREADS, smem, s>>>(items, grid, xs, perm, f, g);
    GB_LAUNCHED("b3_group");
  }
}

template <typename R> struct G3Set;
template <> struct G3Set<float> {
  static bool has(int w) { return w == 8 || w == 10 || w == 14; }
  static size_t smem(const Geom<float> &g)
  {
    switch (g.w) {
      case 8: return g3_smem_max<float, 8, G3_CS>(g);
      case 10: return std::max({g3_smem_max<float, 10, G3_CS>(g), c3_smem_bytes<10>(), cb_smem_bytes<10>(), s3_smem_bytes<10>(g)});
      case 14: return g3_smem_max<float, 14, G3_CS>(g);
    }
    return 0;
  }
  static bool column(int w) { return w == 10; }
  static void run(bool adj, const WorkItem *it, int ni, float2 *grid, const float *xs, const uint32_t *perm,
                  float2 *f, const Geom<float> &g, const WinPoly &poly, const Col3Bufs &cb, cudaStream_t s)
  {
    switch (g.w) {
      case 8: run_g3<float, 8>(adj, it, ni, grid, xs, perm, f, g, poly, cb, s); return;
      case 10: run_g3<float, 10>(adj, it, ni, grid, xs, perm, f, g, poly, cb, s); return;
      case 14: run_g3<float, 14>(adj, it, ni, grid, xs, perm, f, g, poly, cb, s); return;
    }
    fatal("no 3-D group kernel for w=%d", g.w);
  }
};
template <> struct G3Set<double> {
  static bool has(int w) { return w == 10 || w == 14; }
  static bool column(int) { return false; }
  static size_t smem(const Geom<double> &g)
  {
    switch (g.w) {
      case 10: return g3_smem_max<double, 10, G3_CS>(g);
      case 14: return g3_smem_max<double, 14, G3_CS>(g);
    }
    return 0;
  }
  static void run(bool adj, const WorkItem *it, int ni, double2 *grid, const double *xs,
                  const uint32_t *perm, double2 *f, const Geom<double> &g, const WinPoly &poly, const Col3Bufs &cb, cudaStream_t s)
  {
    switch (g.w) {
      case 10: run_g3<double, 10>(adj, it, ni, grid, xs, perm, f, g, poly, cb, s); return;
      case 14: run_g3<double, 14>(adj, it, ni, grid, xs, perm, f, g, poly, cb, s); return;
    }
    fatal("no 3-D group kernel for w=%d", g.w);
  }
};

template <typename R>
bool group3_supported(int w) { return G3Set<R>::has(w); }
template <typename R>
size_t group3_smem_bytes(const Geom<R> &g) { return G3Set<R>::smem(g); }
int group3_subcell_edge() { return G3_CS; }
template <typename R>
bool group3_column_supported(int w) { return G3Set<R>::column(w); }
int group3_max_item() { return G3_MAXITEM; }

template <typename R>
void launch_b3_group(const WorkItem *items, int nitems, const typename Cx<R>::T *grid, const R *xs,
                     const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g, const WinPoly &poly,
                     const Col3Bufs &cb, cudaStream_t s)
{
  if (nitems > 0)
    G3Set<R>::run(false, items, nitems, const_cast<typename Cx<R>::T *>(grid), xs, perm, f, g, poly, cb, s);
}

template <typename R>
void launch_bt3_group(const WorkItem *items, int nitems, typename Cx<R>::T *grid, const R *xs,
                      const uint32_t *perm, const typename Cx<R>::T *f, const Geom<R> &g, const WinPoly &poly,
                      const Col3Bufs &cb, cudaStream_t s)
{
  if (nitems > 0)
    G3Set<R>::run(true, items, nitems, grid, xs, perm, const_cast<typename Cx<R>::T *>(f), g, poly, cb, s);
}

template bool group3_supported<float>(int);
template bool group3_supported<double>(int);
template size_t group3_smem_bytes<float>(const Geom<float> &);
template bool group3_column_supported<float>(int);
template bool group3_column_supported<double>(int);
template size_t group3_smem_bytes<double>(const Geom<double> &);
template void launch_b3_group<float>(const WorkItem *, int, const float2 *, const float *, const uint32_t *,
                                     float2 *, const Geom<float> &, const WinPoly &, const Col3Bufs &, cudaStream_t);
template void launch_b3_group<double>(const WorkItem *, int, const double2 *, const double *,
                                      const uint32_t *, double2 *, const Geom<double> &, const WinPoly &,
                                      const Col3Bufs &, cudaStream_t);
template void launch_bt3_group<float>(const WorkItem *, int, float2 *, const float *, const uint32_t *,
                                      const float2 *, const Geom<float> &, const WinPoly &, const Col3Bufs &, cudaStream_t);
template void launch_bt3_group<double>(const WorkItem *, int, double2 *, const double *, const uint32_t *,
                                       const double2 *, const Geom<double> &, const WinPoly &, const Col3Bufs &, cudaStream_t);

}  // namespace gb
