// gb_sort.cu -- node keys, stable radix sort and tile binning on the GPU.
//
// Two orders of the nodes are produced at node set-up:
//  * the reference's sorted index (reference nfft.c:75-109, sort0): key_j is
//    the row-major index of ((floor(n_t x_jt - m) mod n_t) + n_t) mod n_t,
//    evaluated in plan precision without contraction, and (key, j) pairs are
//    sorted stably by key (reference kernel/util/sort.c:91-171 uses an LSD
//    radix sort; any stable sort gives the same permutation).  Exposed as
//    index_x when NFFT_SORT_NODES is set;
//  * the tile order used by the transform kernels: nodes grouped by the tile
//    of the oversampled grid that holds their wrapped window start, so that
//    one CTA works on one tile's padded subgrid in shared memory.
#include "gb_internal.h"

namespace gb {

// ============================================================== scan
// Block-wide exclusive scan of 4 values per thread, 1024 threads per block.
static constexpr int SCAN_THREADS = 1024;
static constexpr int SCAN_ITEMS = 4;
static constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__global__ void k_scan_tiles(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                             uint32_t *__restrict__ sums, size_t n)
{
  __shared__ uint32_t wsum[SCAN_THREADS / 32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    acc += v[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = warp_incl_scan(acc);
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = wsum[lane];
    uint32_t si = warp_incl_scan(s);
    wsum[lane] = si - s;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + incl - acc;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == SCAN_THREADS - 1 && sums) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, const uint32_t *__restrict__ offs, size_t n)
{
  const size_t i = (size_t)blockIdx.x * SCAN_TILE + threadIdx.x;
  const uint32_t o = offs[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    size_t j = i + (size_t)k * SCAN_THREADS;
    if (j < n) out[j] += o;
  }
}

__global__ void k_scan_total(const uint32_t *in, const uint32_t *out, size_t n, uint32_t *total)
{
  if (threadIdx.x == 0 && blockIdx.x == 0) *total = (n ? out[n - 1] + in[n - 1] : 0u);
}

size_t scan_temp_bytes(size_t n)
{
  size_t bytes = 0;
  while (n > 1) {
    n = (n + SCAN_TILE - 1) / SCAN_TILE;
    bytes += 2 * n * sizeof(uint32_t) + 256;
  }
  return bytes + 256;
}

static void scan_rec(const uint32_t *in, uint32_t *out, size_t n, char *temp, cudaStream_t s)
{
  const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb <= 1) {
    k_scan_tiles<<<1, SCAN_THREADS, 0, s>>>(in, out, nullptr, n);
    GB_LAUNCHED("scan_tiles");
    return;
  }
  uint32_t *sums = (uint32_t *)temp;
  uint32_t *sums_scan = sums + nb;
  char *next = temp + ((2 * nb * sizeof(uint32_t) + 255) / 256) * 256;
  k_scan_tiles<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, sums, n);
  GB_LAUNCHED("scan_tiles");
  scan_rec(sums, sums_scan, nb, next, s);
  k_scan_add<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(out, sums_scan, n);
  GB_LAUNCHED("scan_add");
}

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *total, void *temp,
                        cudaStream_t s)
{
  if (n == 0) {
    if (total) GB_CUDA(cudaMemsetAsync(total, 0, sizeof(uint32_t), s));
    return;
  }
  scan_rec(in, out, n, (char *)temp, s);
  if (total) {
    k_scan_total<<<1, 32, 0, s>>>(in, out, n, total);
    GB_LAUNCHED("scan_total");
  }
}

// ============================================================== radix sort
// 8-bit digits; a block owns RS_TILE consecutive elements.  The scatter
// ranks elements stably: rounds of RS_THREADS consecutive elements, ranked
// inside each warp with __match_any_sync and across warps by per-digit
// prefix sums, so that equal keys keep their input order.
static constexpr int RS_THREADS = 256;
static constexpr int RS_ROUNDS = 16;
static constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
static constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__(RS_THREADS) k_rs_count(const uint32_t *__restrict__ keys, size_t n,
                                                         int shift, uint32_t *__restrict__ hist,
                                                         int nblk)
{
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    size_t i = base + (size_t)r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(
    const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout,
    uint32_t *__restrict__ vout, const uint32_t *__restrict__ offs, size_t n, int shift, int nblk)
{
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcnt[RS_WARPS][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base[tid] = offs[(size_t)tid * nblk + blockIdx.x];
  const uint32_t lt_mask = (1u << lane) - 1u;
  const size_t start = (size_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const size_t i0 = start + (size_t)r * RS_THREADS;
    if (i0 >= n) break;  // uniform across the block
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const size_t idx = i0 + tid;
    const bool valid = idx < n;
    const uint32_t k = valid ? kin[idx] : 0u;
    const uint32_t v = valid ? vin[idx] : 0u;
    const uint32_t dig = valid ? ((k >> shift) & 255u) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, dig);
    const uint32_t lrank = __popc(peers & lt_mask);
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][dig] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = base[tid];
#pragma unroll
      for (int w = 0; w < RS_WARPS; ++w) {
        uint32_t c = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += c;
      }
      base[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = wcnt[warp][dig] + lrank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

size_t radix_temp_bytes(size_t n)
{
  const size_t nblk = (n + RS_TILE - 1) / RS_TILE;
  const size_t h = 256 * nblk;
  return 2 * h * sizeof(uint32_t) + scan_temp_bytes(h) + 512;
}

void radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, size_t n,
                      int key_bits, void *temp, cudaStream_t s)
{
  if (n <= 1 || key_bits <= 0) return;
  const int nblk = (int)((n + RS_TILE - 1) / RS_TILE);
  const size_t h = (size_t)256 * nblk;
  uint32_t *hist = (uint32_t *)temp;
  uint32_t *offs = hist + h;
  void *stemp = (void *)(((uintptr_t)(offs + h) + 255) & ~(uintptr_t)255);
  uint32_t *ka = keys, *va = vals, *kb = keys2, *vb = vals2;
  int passes = 0;
  for (int shift = 0; shift < key_bits; shift += 8) {
    k_rs_count<<<nblk, RS_THREADS, 0, s>>>(ka, n, shift, hist, nblk);
    GB_LAUNCHED("rs_count");
    exclusive_scan_u32(hist, offs, h, nullptr, stemp, s);
    k_rs_scatter<<<nblk, RS_THREADS, 0, s>>>(ka, va, kb, vb, offs, n, shift, nblk);
    GB_LAUNCHED("rs_scatter");
    uint32_t *t;
    t = ka; ka = kb; kb = t;
    t = va; va = vb; vb = t;
    ++passes;
  }
  if (passes & 1) {
    GB_CUDA(cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    GB_CUDA(cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
}

// ============================================================== node keys
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <typename R>
__global__ void k_node_keys(const R *__restrict__ x, Geom<R> g, uint32_t *__restrict__ tile_key,
                            uint32_t *__restrict__ ref_key, uint32_t *__restrict__ idx)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.M) return;
  uint32_t tk = 0, rk = 0, sk = 0;
  for (int t = 0; t < g.d; ++t) {
    const R xt = x[j * g.d + t];
    const int u = wrap(node_u<R>(xt, g.nR[t], g.m), g.n[t]);
    const int tile = u / g.T[t];
    tk = tk * (uint32_t)g.ntile[t] + (uint32_t)tile;
    // sub-cell of the window start inside its tile (group kernels)
    const int cst = (t == g.d - 1) ? g.csz : g.cs;
    sk = sk * (uint32_t)(g.T[t] / cst) + (uint32_t)((u - tile * g.T[t]) / cst);
    // reference sort key: floor(n*x - m) in plan precision, no contraction
    const int help = (int)gb_floor(sub_rn(mul_rn(g.nR[t], xt), (R)g.m));
    const int ut = ((help % g.n[t]) + g.n[t]) % g.n[t];
    rk = rk * (uint32_t)g.n[t] + (uint32_t)ut;
  }
  tile_key[j] = g.sub > 1 ? tk * (uint32_t)g.sub + sk : tk;
  if (ref_key) ref_key[j] = rk;
  idx[j] = (uint32_t)j;
}

template <typename R>
void launch_node_keys(const R *x, const Geom<R> &g, uint32_t *tile_key, uint32_t *ref_key,
                      uint32_t *idx, cudaStream_t s)
{
  if (g.M == 0) return;
  const int th = 256;
  const long long nb = (g.M + th - 1) / th;
  k_node_keys<R><<<(unsigned)nb, th, 0, s>>>(x, g, tile_key, ref_key, idx);
  GB_LAUNCHED("node_keys");
}

template <typename R>
__global__ void k_gather_x(const R *__restrict__ x, const uint32_t *__restrict__ perm,
                           R *__restrict__ xs, long long M, int d)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const long long j = perm[i];
  for (int t = 0; t < d; ++t) xs[i * d + t] = x[j * d + t];
}

template <typename R>
void launch_gather_x(const R *x, const uint32_t *perm, R *xs, const Geom<R> &g, cudaStream_t s)
{
  if (g.M == 0) return;
  const int th = 256;
  k_gather_x<R><<<(unsigned)((g.M + th - 1) / th), th, 0, s>>>(x, perm, xs, g.M, g.d);
  GB_LAUNCHED("gather_x");
}

// start[t] = first sorted position with key >= t, for t in [0, ntiles]
__global__ void k_tile_starts(const uint32_t *__restrict__ key, long long M, int ntiles,
                              uint32_t div, uint32_t *__restrict__ start)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > M) return;
  const long long lo = (i == 0) ? -1 : (long long)(key[i - 1] / div);
  const long long hi = (i == M) ? (long long)ntiles : (long long)(key[i] / div);
  for (long long t = lo + 1; t <= hi; ++t) start[t] = (uint32_t)i;
}

void launch_tile_starts(const uint32_t *sorted_keys, long long M, int ntiles, uint32_t div,
                        uint32_t *start, cudaStream_t s)
{
  const int th = 256;
  k_tile_starts<<<(unsigned)((M + 1 + th - 1) / th), th, 0, s>>>(sorted_keys, M, ntiles, div, start);
  GB_LAUNCHED("tile_starts");
}

__global__ void k_chunk_counts(const uint32_t *__restrict__ start, int ntiles, int chunk,
                               uint32_t *__restrict__ cnt)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint32_t c = start[t + 1] - start[t];
  cnt[t] = (c + chunk - 1) / chunk;
}

__global__ void k_fill_items(const uint32_t *__restrict__ start, const uint32_t *__restrict__ off,
                             int ntiles, int chunk, WorkItem *__restrict__ items)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint32_t s0 = start[t], s1 = start[t + 1];
  uint32_t o = off[t];
  for (uint32_t a = s0; a < s1; a += chunk, ++o) {
    WorkItem w;
    w.tile = t;
    w.start = (int)a;
    w.end = (int)min(s1, a + (uint32_t)chunk);
    w.pad = 0;
    items[o] = w;
  }
}

int build_work_items(const uint32_t *start, int ntiles, int chunk, WorkItem *items,
                     uint32_t *cnt_tmp, uint32_t *off_tmp, uint32_t *total_dev, void *scan_temp,
                     cudaStream_t s)
{
  const int th = 256;
  const int nb = (ntiles + th - 1) / th;
  k_chunk_counts<<<nb, th, 0, s>>>(start, ntiles, chunk, cnt_tmp);
  GB_LAUNCHED("chunk_counts");
  exclusive_scan_u32(cnt_tmp, off_tmp, (size_t)ntiles, total_dev, scan_temp, s);
  k_fill_items<<<nb, th, 0, s>>>(start, off_tmp, ntiles, chunk, items);
  GB_LAUNCHED("fill_items");
  uint32_t total = 0;
  GB_CUDA(cudaMemcpyAsync(&total, total_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  return (int)total;
}

__global__ void k_ref_index(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                            long long M, long long *__restrict__ out)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  out[2 * i] = (long long)keys[i];
  out[2 * i + 1] = (long long)vals[i];
}

void launch_ref_index_to_int64(const uint32_t *keys, const uint32_t *vals, long long M,
                               long long *out, cudaStream_t s)
{
  if (M == 0) return;
  const int th = 256;
  k_ref_index<<<(unsigned)((M + th - 1) / th), th, 0, s>>>(keys, vals, M, out);
  GB_LAUNCHED("ref_index");
}

template void launch_node_keys<float>(const float *, const Geom<float> &, uint32_t *, uint32_t *,
                                      uint32_t *, cudaStream_t);
template void launch_node_keys<double>(const double *, const Geom<double> &, uint32_t *,
                                       uint32_t *, uint32_t *, cudaStream_t);
template void launch_gather_x<float>(const float *, const uint32_t *, float *, const Geom<float> &,
                                     cudaStream_t);
template void launch_gather_x<double>(const double *, const uint32_t *, double *,
                                      const Geom<double> &, cudaStream_t);

}  // namespace gb
