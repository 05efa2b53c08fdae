// gb_batch.cu -- many independent 2-D single-precision plans of uneven N, M
// and m transformed together: one persistent kernel per stage pulls
// (plan, tile, node range) work items from a device queue, the D stages run
// as one launch over all plans, the FFTs as one batched cuFFT call per grid
// shape, and the whole trafo + adjoint sequence can be captured once as a
// CUDA graph and replayed.  An autotuner picks, per class of plans
// (m, oversampling, node density), the tile edge and the number of threads
// that share one node.
//
// No counterpart in the reference: the reference runs plans one at a time
// (nfft_trafo / nfft_adjoint, kernel/nfft/nfft.c:5655-5749); every plan's
// result here is the same transform as its own nfftf_trafo / nfftf_adjoint.
#include <cufft.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/nfft_gb300.h"
#include "gb_col2.cuh"
#include "gb_internal.h"

namespace gb {

// per-plan entry of the device table
struct BPlan {
  Geom<float> g;
  const float *xs;        // tile-ordered nodes
  const uint32_t *perm;   // tile order -> caller order
  const double *cphi;     // FP64 1/phi_hat
  const float2 *fhat_in;  // trafo input (N_total)
  float2 *f_out;          // trafo output (M)
  const float2 *f_in;     // adjoint input (M)
  float2 *fhat_out;       // adjoint output (N_total)
  float2 *grid;           // this plan's grid in the batch arena
  long long grid_off;     // offset of grid in the arena (complex elements)
  long long fhat_off;     // offset of this plan in the concatenated f_hat index space
  int tpn;                // threads per node of the B / B^T kernels (1, 4, 16); 0: column kernels
  int pad;
  const WinPoly *poly;    // the plan's polynomial window (device copy; column kernels)
};

struct BItem {
  int plan, tile, start, end;
};

static constexpr int BT_THREADS = 256;

// smallest k with off[k + 1] > i (off ascending, off[0] = 0)
__device__ __forceinline__ int find_plan(const long long *off, int n, long long i)
{
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// D + zero pad for all plans: one thread per arena cell
__global__ void k_batch_pad(const BPlan *__restrict__ plans, const long long *__restrict__ grid_off, int np,
                            long long total, float2 *__restrict__ arena)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int k = find_plan(grid_off, np, i);
  const BPlan &P = plans[k];
  const long long cell = i - grid_off[k];
  const int n1 = P.g.n[1], n0 = P.g.n[0];
  const int i0 = (int)(cell / n1), i1 = (int)(cell - (long long)i0 * n1);
  const int k0 = i0 < n0 / 2 ? i0 : i0 - n0, k1 = i1 < n1 / 2 ? i1 : i1 - n1;
  const int kk0 = k0 + P.g.N[0] / 2, kk1 = k1 + P.g.N[1] / 2;
  float2 out = make_float2(0.f, 0.f);
  if (kk0 >= 0 && kk0 < P.g.N[0] && kk1 >= 0 && kk1 < P.g.N[1]) {
    const double c = P.cphi[kk0] * P.cphi[P.g.N[0] + kk1];
    const float2 v = P.fhat_in[(long long)kk0 * P.g.N[1] + kk1];
    out = make_float2((float)(v.x * c), (float)(v.y * c));
  }
  arena[i] = out;
}

// crop + D^T for all plans: one thread per coefficient of the concatenation
__global__ void k_batch_crop(const BPlan *__restrict__ plans, const long long *__restrict__ fhat_off, int np,
                             long long total, const float2 *__restrict__ arena)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int k = find_plan(fhat_off, np, i);
  const BPlan &P = plans[k];
  const long long kl = i - fhat_off[k];
  const int kk0 = (int)(kl / P.g.N[1]), kk1 = (int)(kl - (long long)kk0 * P.g.N[1]);
  const int k0 = kk0 - P.g.N[0] / 2, k1 = kk1 - P.g.N[1] / 2;
  const int i0 = k0 < 0 ? k0 + P.g.n[0] : k0, i1 = k1 < 0 ? k1 + P.g.n[1] : k1;
  const float2 v = arena[P.grid_off + (long long)i0 * P.g.n[1] + i1];
  const double c = P.cphi[kk0] * P.cphi[P.g.N[0] + kk1];
  P.fhat_out[kl] = make_float2((float)(v.x * c), (float)(v.y * c));
}

}  // namespace gb

namespace gb {

// Window values of one node shared by a group of TPN lanes: lane q of the
// group evaluates the taps l = q, q + TPN, ... of both dimensions; psi1 is
// then gathered in full by every lane (W shuffles), psi0 stays with the lane
// that owns those rows.
template <int W, int TPN>
__device__ __forceinline__ void b2_weights(float x0, float x1, int u0, int u1, const Geom<float> &g, int q,
                                           int base, float (&p0)[(W + TPN - 1) / TPN], float (&p1)[W])
{
  constexpr int S = (W + TPN - 1) / TPN;
  float mine1[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int l = q + s * TPN;
    p0[s] = l < W ? kb_phi<float>(x0 - float(u0 + l) / g.nR[0], g.nR[0], g.mm, g.b[0]) : 0.f;
    mine1[s] = l < W ? kb_phi<float>(x1 - float(u1 + l) / g.nR[1], g.nR[1], g.mm, g.b[1]) : 0.f;
  }
  if (TPN == 1) {
#pragma unroll
    for (int l = 0; l < W; ++l) p1[l] = mine1[l];
  } else {
    const unsigned mask = 0xffffffffu;
#pragma unroll
    for (int l = 0; l < W; ++l) p1[l] = __shfl_sync(mask, mine1[l / TPN], base + (l % TPN));
  }
}

template <int W, int TPN>
__device__ void b2_gather_item(const BItem &it, const BPlan &P, const float2 *sg, const int *org)
{
  constexpr int S = (W + TPN - 1) / TPN;
  const Geom<float> &g = P.g;
  const int q = threadIdx.x % TPN, base = (threadIdx.x & 31) - q;
  const int e1 = g.ext[1];
  // every lane of a group walks the same node sequence; whole warps stay converged
  for (int i0 = it.start; i0 < it.end; i0 += BT_THREADS / TPN) {
    const int i = i0 + threadIdx.x / TPN;
    const bool valid = i < it.end;
    const int ii = valid ? i : it.start;
    const float x0 = P.xs[2 * (long long)ii], x1 = P.xs[2 * (long long)ii + 1];
    const int u0 = node_u<float>(x0, g.nR[0], g.m), u1 = node_u<float>(x1, g.nR[1], g.m);
    const int l0 = wrap(u0, g.n[0]) - org[0], l1 = wrap(u1, g.n[1]) - org[1];
    float p0[S], p1[W];
    b2_weights<W, TPN>(x0, x1, u0, u1, g, q, base, p0, p1);
    float ar = 0.f, ai = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int r = q + s * TPN;
      if (r < W) {
        const float2 *row = sg + (l0 + r) * e1 + l1;
        float rr = 0.f, ri = 0.f;
#pragma unroll
        for (int c = 0; c < W; ++c) {
          const float2 v = row[c];
          rr += p1[c] * v.x;
          ri += p1[c] * v.y;
        }
        ar += p0[s] * rr;
        ai += p0[s] * ri;
      }
    }
#pragma unroll
    for (int o = TPN / 2; o >= 1; o >>= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o);
      ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (valid && q == 0) P.f_out[P.perm[i]] = make_float2(ar, ai);
  }
}

template <int W, int TPN>
__device__ void b2_spread_item(const BItem &it, const BPlan &P, float2 *sg, const int *org)
{
  constexpr int S = (W + TPN - 1) / TPN;
  const Geom<float> &g = P.g;
  const int q = threadIdx.x % TPN, base = (threadIdx.x & 31) - q;
  const int e1 = g.ext[1];
  for (int i0 = it.start; i0 < it.end; i0 += BT_THREADS / TPN) {
    const int i = i0 + threadIdx.x / TPN;
    const bool valid = i < it.end;
    const int ii = valid ? i : it.start;
    const float x0 = P.xs[2 * (long long)ii], x1 = P.xs[2 * (long long)ii + 1];
    const int u0 = node_u<float>(x0, g.nR[0], g.m), u1 = node_u<float>(x1, g.nR[1], g.m);
    const int l0 = wrap(u0, g.n[0]) - org[0], l1 = wrap(u1, g.n[1]) - org[1];
    float p0[S], p1[W];
    b2_weights<W, TPN>(x0, x1, u0, u1, g, q, base, p0, p1);
    if (!valid) continue;
    const float2 fj = P.f_in[P.perm[i]];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int r = q + s * TPN;
      if (r < W) {
        float2 *row = sg + (l0 + r) * e1 + l1;
        const float wr = p0[s] * fj.x, wi = p0[s] * fj.y;
#pragma unroll
        for (int c = 0; c < W; ++c) {
          atomicAdd(&row[c].x, p1[c] * wr);
          atomicAdd(&row[c].y, p1[c] * wi);
        }
      }
    }
  }
}

__device__ __forceinline__ void b2_item_origin(const BItem &it, const Geom<float> &g, int *org)
{
  const int t1 = it.tile % g.ntile[1], t0 = it.tile / g.ntile[1];
  org[0] = t0 * g.T[0];
  org[1] = t1 * g.T[1];
}

__device__ __forceinline__ long long b2_cell(int idx, const int *org, const Geom<float> &g)
{
  const int c1 = idx % g.ext[1], c0 = idx / g.ext[1];
  int p0 = org[0] + c0, p1 = org[1] + c1;
  while (p0 >= g.n[0]) p0 -= g.n[0];
  while (p1 >= g.n[1]) p1 -= g.n[1];
  return (long long)p0 * g.n[1] + p1;
}

#define GB_B2_DISPATCH(FN, ...)                                                  \
  switch (P.g.w * 100 + P.tpn) {                                                 \
    case 1001: FN<10, 1>(__VA_ARGS__); break;                                    \
    case 1004: FN<10, 4>(__VA_ARGS__); break;                                    \
    case 1016: FN<10, 16>(__VA_ARGS__); break;                                   \
    case 1401: FN<14, 1>(__VA_ARGS__); break;                                    \
    case 1404: FN<14, 4>(__VA_ARGS__); break;                                    \
    case 1416: FN<14, 16>(__VA_ARGS__); break;                                   \
    default: break;                                                              \
  }

// Persistent B over all plans: CTAs take items from the queue in order
// (largest first) until it is empty.
__global__ void __launch_bounds__(BT_THREADS) k_batch_b2(const BPlan *__restrict__ plans,
                                                         const BItem *__restrict__ items, int nitems,
                                                         int *__restrict__ counter)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *sg = reinterpret_cast<float2 *>(smem_raw);
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int k = s_item;
    if (k >= nitems) break;
    const BItem it = items[k];
    const BPlan &P = plans[it.plan];
    int org[2];
    b2_item_origin(it, P.g, org);
    const int cells = P.g.ext[0] * P.g.ext[1];
    for (int idx = threadIdx.x; idx < cells; idx += BT_THREADS) sg[idx] = P.grid[b2_cell(idx, org, P.g)];
    __syncthreads();
    GB_B2_DISPATCH(b2_gather_item, it, P, sg, org)
    __syncthreads();
  }
}

// Persistent B^T over all plans; each item adds its padded subgrid to its
// plan's grid once.
__global__ void __launch_bounds__(BT_THREADS) k_batch_bt2(const BPlan *__restrict__ plans,
                                                          const BItem *__restrict__ items, int nitems,
                                                          int *__restrict__ counter)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *sg = reinterpret_cast<float2 *>(smem_raw);
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int k = s_item;
    if (k >= nitems) break;
    const BItem it = items[k];
    const BPlan &P = plans[it.plan];
    int org[2];
    b2_item_origin(it, P.g, org);
    const int cells = P.g.ext[0] * P.g.ext[1];
    for (int idx = threadIdx.x; idx < cells; idx += BT_THREADS) sg[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    GB_B2_DISPATCH(b2_spread_item, it, P, sg, org)
    __syncthreads();
    for (int idx = threadIdx.x; idx < cells; idx += BT_THREADS) {
      const float2 v = sg[idx];
      if (v.x != 0.f || v.y != 0.f) global_add_c(P.grid + b2_cell(idx, org, P.g), v);
    }
    __syncthreads();
  }
}

// Persistent column B / B^T (gb_col2.cuh) over the items of the plans in
// column mode: the same queue discipline, one work item per CTA pass.
#define GB_C2_DISPATCH(FN, ...)          \
  switch (P.g.w) {                       \
    case 10: FN<10>(__VA_ARGS__); break; \
    case 14: FN<14>(__VA_ARGS__); break; \
    default: break;                      \
  }

__global__ void __launch_bounds__(C2_THREADS, 2) k_batch_b2c(const BPlan *__restrict__ plans,
                                                              const BItem *__restrict__ items, int nitems,
                                                              int *__restrict__ counter)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int k = s_item;
    if (k >= nitems) break;
    const BItem bi = items[k];
    const BPlan &P = plans[bi.plan];
    const WorkItem it = {bi.tile, bi.start, bi.end, 0};
    GB_C2_DISPATCH(c2_b_item, it, P.grid, P.xs, P.perm, P.f_out, P.g, *P.poly, smem_raw)
    __syncthreads();
  }
}

__global__ void __launch_bounds__(C2_THREADS, 2) k_batch_bt2c(const BPlan *__restrict__ plans,
                                                               const BItem *__restrict__ items, int nitems,
                                                               int *__restrict__ counter)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int k = s_item;
    if (k >= nitems) break;
    const BItem bi = items[k];
    const BPlan &P = plans[bi.plan];
    const WorkItem it = {bi.tile, bi.start, bi.end, 0};
    GB_C2_DISPATCH(c2_bt_item, it, P.grid, P.xs, P.perm, P.f_in, P.g, *P.poly, smem_raw)
    __syncthreads();
  }
}

}  // namespace gb

