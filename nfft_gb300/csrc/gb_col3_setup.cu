// gb_col3_setup.cu -- node set-up for the single-precision 3-D kernels of
// gb_col3.cuh, done once per node set (in precompute_one_psi).
//
// The reference precomputes per-node window data once per node set as well
// (PRE_PSI tables, nfft.c:5819-5844); here a node keeps 16 bytes: its three
// polynomial arguments s_t = 2 frac(n_t x_t) - 1 and its window start inside
// its 8^3 tile, three 3-bit fields.  Per work item the start of every z-column
// (17 entries) and of every 2x2x2 sub-cell (65 entries) within the item's
// node range is kept, so the transform kernels need no pass over the nodes to
// find them.
#include <mutex>

#include "gb_internal.h"

namespace gb {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool encode_grid_map(CUtensorMap *map, void *grid, const int *n, int ext, int ext_y)
{
  static std::once_flag once;
  static EncodeTiledFn enc = nullptr;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      enc = (EncodeTiledFn)fn;
  });
  // rows of 2 n_2 floats must be 16-byte multiples, the box within 256 per dimension
  const int zb = (ext + 1) & ~1;
  if (!enc || !grid || (n[2] & 1) || ext > 256 || ext_y > 256 || 2 * zb > 256) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * n[2], (cuuint64_t)n[1], (cuuint64_t)n[0]};
  const cuuint64_t strides[2] = {(cuuint64_t)8 * n[2], (cuuint64_t)8 * n[2] * n[1]};
  const cuuint32_t box[3] = {(cuuint32_t)(2 * zb), (cuuint32_t)ext_y, (cuuint32_t)ext};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, grid, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_grid_map_2d(CUtensorMap *map, void *grid, const int *n, int ext, int zb)
{
  // rows of 2 n_1 floats must be 16-byte multiples, the box within 256 per dimension
  if (!grid || (n[1] & 1) || (zb & 1) || ext > 256 || 2 * zb > 256) return false;
  static std::once_flag once;
  static EncodeTiledFn enc = nullptr;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      enc = (EncodeTiledFn)fn;
  });
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)2 * n[1], (cuuint64_t)n[0]};
  const cuuint64_t strides[1] = {(cuuint64_t)8 * n[1]};
  const cuuint32_t box[2] = {(cuuint32_t)(2 * zb), (cuuint32_t)ext};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, grid, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

__global__ void k_c3_records(const float *__restrict__ xs, Geom<float> g, float4 *__restrict__ rec)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.M) return;
  float s[3];
  int loc = 0;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const float xn = xs[3 * i + t] * g.nR[t];
    const int u = (int)floorf(xn) - g.m;  // node_u: the binning used the same expression
    const float t0 = xn - (float)u;       // in [m, m + 1), exact
    s[t] = fmaf(2.f, t0, -(float)(2 * g.m + 1));
    loc |= (wrap(u, g.n[t]) & 7) << (3 * t);
  }
  rec[i] = make_float4(s[0], s[1], s[2], __int_as_float(loc));
}

// one block per work item; keys are the sorted node keys tile * sub + k with
// k = (x sub-cell * 4 + y sub-cell) * 8 + z cell
__global__ void k_c3_item_starts(const WorkItem *__restrict__ items, const uint32_t *__restrict__ keys,
                                 uint32_t sub, uint16_t *__restrict__ cst, uint16_t *__restrict__ sst)
{
  const WorkItem it = items[blockIdx.x];
  const int n = it.end - it.start;
  uint16_t *c = cst + 17LL * blockIdx.x;
  uint16_t *s = sst + 65LL * blockIdx.x;
  for (int k = threadIdx.x; k <= n; k += blockDim.x) {
    const int kc = k < n ? (int)(keys[it.start + k] % sub) : 128;
    const int kp = k > 0 ? (int)(keys[it.start + k - 1] % sub) : -2;
    for (int q = (kp >> 3) + 1; q <= (kc >> 3); ++q) c[q] = (uint16_t)k;
    for (int q = (kp >> 1) + 1; q <= (kc >> 1); ++q) s[q] = (uint16_t)k;
  }
}


void launch_c3_setup(const float *xs, const Geom<float> &g, const WorkItem *items, int nitems,
                     const uint32_t *keys, float4 *rec, uint16_t *cst, uint16_t *sst, cudaStream_t s)
{
  if (g.M > 0) {
    k_c3_records<<<(unsigned)((g.M + 255) / 256), 256, 0, s>>>(xs, g, rec);
    GB_LAUNCHED("c3_records");
  }
  if (nitems > 0) {
    k_c3_item_starts<<<nitems, 128, 0, s>>>(items, keys, (uint32_t)g.sub, cst, sst);
    GB_LAUNCHED("c3_item_starts");
  }
}


}  // namespace gb
