// gb_internal.h -- host-side interfaces between the library's translation units.
#pragma once

#include <cuda.h>  // CUtensorMap (type only; the encoder comes through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <stddef.h>

#include "gb_common.cuh"

namespace gb {

// ---------------------------------------------------------------- scans/sort
size_t scan_temp_bytes(size_t n);
// out[i] = sum_{k<i} in[k]; out may not alias in.  total (device, nullable)
// receives the sum of all n values.
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *total,
                        void *temp, cudaStream_t s);

size_t radix_temp_bytes(size_t n);
// Stable LSD radix sort of (keys, vals) by the low key_bits bits of keys.
// keys2/vals2 are n-element ping-pong buffers.  The sorted result ends in
// keys/vals.
void radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2,
                      size_t n, int key_bits, void *temp, cudaStream_t s);

// node binning
template <typename R>
void launch_node_keys(const R *x, const Geom<R> &g, uint32_t *tile_key, uint32_t *ref_key,
                      uint32_t *idx, cudaStream_t s);
template <typename R>
void launch_gather_x(const R *x, const uint32_t *perm, R *xs, const Geom<R> &g, cudaStream_t s);
// start[t] = first sorted position whose key / div >= t, t in [0, ntiles]
void launch_tile_starts(const uint32_t *sorted_keys, long long M, int ntiles, uint32_t div,
                        uint32_t *start, cudaStream_t s);
// fills items (capacity >= ntiles + M/chunk + 1); returns the item count
// (synchronises the stream once)
int build_work_items(const uint32_t *start, int ntiles, int chunk, WorkItem *items,
                     uint32_t *cnt_tmp, uint32_t *off_tmp, uint32_t *total_dev, void *scan_temp,
                     cudaStream_t s);
void launch_ref_index_to_int64(const uint32_t *keys, const uint32_t *vals, long long M,
                               long long *out, cudaStream_t s);

// ---------------------------------------------------------------- D stage
template <typename R>
void launch_cphi(const Geom<R> &g, double *cphi, cudaStream_t s);
template <typename R>
void launch_d_pad(const typename Cx<R>::T *fhat, const double *cphi, typename Cx<R>::T *grid,
                  const Geom<R> &g, cudaStream_t s);
template <typename R>
void launch_d_crop(const typename Cx<R>::T *grid, const double *cphi, typename Cx<R>::T *fhat,
                   const Geom<R> &g, cudaStream_t s);

// ---------------------------------------------------------------- B stage
// tiled shared-memory kernels; return false when (d, w) has no tiled variant
template <typename R>
bool tiled_supported(int d, int w);
template <typename R>
size_t tiled_smem_bytes(const Geom<R> &g);
template <typename R>
void launch_b_tiled(const WorkItem *items, int nitems, const typename Cx<R>::T *grid,
                    const R *xs, const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g,
                    cudaStream_t s);
template <typename R>
void launch_bt_tiled(const WorkItem *items, int nitems, typename Cx<R>::T *grid, const R *xs,
                     const uint32_t *perm, const typename Cx<R>::T *f, const Geom<R> &g,
                     cudaStream_t s);
// 3-D sub-cell group kernels (fast path of the 3-D transform)
template <typename R>
bool group3_supported(int w);
template <typename R>
size_t group3_smem_bytes(const Geom<R> &g);
int group3_subcell_edge();
// z-column B^T kernel (nodes keyed by (x sub-cell, y sub-cell, z cell))
template <typename R>
bool group3_column_supported(int w);
// node-set data of the single-precision column / sub-cell kernels
struct Col3Bufs {
  const float4 *rec;    // per sorted node: s_0, s_1, s_2, packed window starts in the tile
  const uint16_t *cst;  // per work item: 17 column starts
  const uint16_t *sst;  // per work item: 65 sub-cell starts
  // TMA view of the oversampled grid as f32 [n_0][n_1][2 n_2] with a box of
  // the padded tile: ext x ext_y x 2 zb floats, zb = ext rounded up to even,
  // ext_y = col3_box_ext_y(w) (Box3 in gb_col3.cuh).  Null where it could
  // not be encoded (the kernels then use plain loads and reductions).
  const CUtensorMap *grid_map;
  // B by column segments (k_b3_col) instead of sub-cell units (k_b3_cell)
  int b_column;
};
// Encodes such a view for a plan's grid (false: not representable, e.g. an
// odd n_2, whose rows are not 16-byte multiples).
bool encode_grid_map(CUtensorMap *map, void *grid, const int *n, int ext, int ext_y);
// the 2-D view f32 [n_0][2 n_1] with boxes of ext rows of zb complex values
// (zb even); false where it cannot be encoded (odd n_1)
bool encode_grid_map_2d(CUtensorMap *map, void *grid, const int *n, int ext, int zb);
// y extent of the 3-D column kernels' subgrid box for window width w
int col3_box_ext_y(int w);
// Device-side wait time-outs recorded since the last call (bounded waits on
// TMA copies; non-zero means a copy did not arrive and the kernel gave up).
unsigned long long read_wait_timeouts();
void launch_c3_setup(const float *xs, const Geom<float> &g, const WorkItem *items, int nitems,
                     const uint32_t *keys, float4 *rec, uint16_t *cst, uint16_t *sst, cudaStream_t s);
int group3_max_item();
template <typename R>
void launch_b3_group(const WorkItem *items, int nitems, const typename Cx<R>::T *grid, const R *xs,
                     const uint32_t *perm, typename Cx<R>::T *f, const Geom<R> &g, const WinPoly &poly,
                     const Col3Bufs &cb, cudaStream_t s);
template <typename R>
void launch_bt3_group(const WorkItem *items, int nitems, typename Cx<R>::T *grid, const R *xs,
                      const uint32_t *perm, const typename Cx<R>::T *f, const Geom<R> &g, const WinPoly &poly,
                      const Col3Bufs &cb, cudaStream_t s);
// single-precision 2-D B^T and B by sub-cell columns (nodes keyed by (32^2 tile,
// column of CX x-cells by 8 y-cells)); col2_column_width(w) = CX, 0 where
// the width has no such kernel
int col2_column_width(int w);
// grid_lo non-null: the compensated form (B^T's rounding errors gathered in
// grid_lo, n_0 n_1 complex, zeroed by the caller, then folded into grid).
// B's gmap non-null: the grid's 2-D TMA view (encode_grid_map_2d with ext =
// 32 + w - 1 and zb = col2_box_zb(w)); without it B stages the subgrid cell by
// cell.
void launch_bt2_col(const WorkItem *items, int nitems, float2 *grid, const float *xs, const uint32_t *perm,
                    const float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s,
                    float2 *grid_lo = nullptr);
void launch_b2_col(const WorkItem *items, int nitems, const float2 *grid, const float *xs, const uint32_t *perm,
                   float2 *f, const Geom<float> &g, const WinPoly &poly, cudaStream_t s,
                   const CUtensorMap *gmap = nullptr);
// row length (complex cells, even) of the 2-D column kernels' TMA box
int col2_box_zb(int w);
// bounded TMA waits of the 2-D kernels that gave up (read and cleared)
unsigned long long read_wait_timeouts_2d();
// the B^T of the same layout in double precision, and a per-node B on the
// same work items (both with the window's degree-16 form)
void launch_bt2_col_d(const WorkItem *items, int nitems, double2 *grid, const double *xs, const uint32_t *perm,
                      const double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s);
void launch_b2_node_d(const WorkItem *items, int nitems, const double2 *grid, const double *xs,
                      const uint32_t *perm, double2 *f, const Geom<double> &g, const WinPolyD &poly, cudaStream_t s);
// generic global-memory kernels for any d and m
template <typename R>
void launch_b_generic(const typename Cx<R>::T *grid, const R *xs, const uint32_t *perm,
                      typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s);
template <typename R>
void launch_bt_generic(typename Cx<R>::T *grid, const R *xs, const uint32_t *perm,
                       const typename Cx<R>::T *f, const Geom<R> &g, cudaStream_t s);

// ---------------------------------------------------------------- plan views
// Device state of a single-precision plan, for the batched transforms.
struct PlanViewF {
  Geom<float> g;
  const float *xs;
  const uint32_t *perm;
  const double *cphi;
  const WorkItem *items;
  int nitems;
  float2 *fhat;
  float2 *f;
  bool tiled, group3, direct, ready;
  bool col2;           // nodes keyed by 2-D column (the column kernels apply)
  const WinPoly *poly; // the plan's polynomial window (host copy)
  cudaStream_t stream;
  Col3Bufs c3;         // node records of the 3-D single-precision kernels (null elsewhere)
  float2 *grid;        // the oversampled grid
};
bool plan_view_f(void *nfftf_plan_ptr, PlanViewF *v);
// re-bin a 2-D plan's nodes on tiles of edge T (8, 16 or 32), or with T = 0
// as the plan would by itself (32^2 tiles keyed by column where it can)
void plan_retile_f(void *nfftf_plan_ptr, int T);

// ---------------------------------------------------------------- NDFT
template <typename R>
void launch_ndft_trafo(const R *x, const typename Cx<R>::T *fhat, typename Cx<R>::T *f,
                       const Geom<R> &g, cudaStream_t s);
template <typename R>
void launch_ndft_adjoint(const R *x, const typename Cx<R>::T *f, typename Cx<R>::T *fhat,
                         const Geom<R> &g, cudaStream_t s);

}  // namespace gb
