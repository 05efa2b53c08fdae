// gb_noalloc.cu -- the node sort without any device allocation.
//
// Some callers cannot call cudaMalloc (or anything that does) on the path
// where they sort their nodes: a process whose device memory is owned by a
// caching allocator or a fixed budget, a real-time loop that cannot take the
// implicit device synchronisation of cudaMalloc / cudaFree, or code that runs
// where a new allocation would be an error.  The regular node set-up
// (nfft_precompute_one_psi) allocates its sort buffers per call; this entry
// point computes the same sorted node index from caller-owned device buffers
// and keeps every intermediate buffer (keys, values, their ping-pong copies,
// the radix histograms and scan blocks) in one statically sized device array.
//
// Limits and behaviour:
//  * at most NOALLOC_MAX_NODES (2^18 = 262144) nodes per call; larger M is rejected
//    with an error (return -1, message in nfft_gb_last_error) before any work;
//  * the scratch array is a file-scope __device__ array: every GPU that loads
//    the library holds it (NOALLOC_BYTES, about 4.3 MB) until the process exits;
//  * the first call on a device looks up the array's device address there
//    (cudaGetSymbolAddress, with that device current) and caches it; make that
//    first call before any stream capture;
//  * the cached address belongs to the device's current context: after
//    cudaDeviceReset on a device, do not call this entry point there again
//    in the same process;
//  * all calls share the array, which keeps the last call's contents; calls
//    that overlap on the GPU (other streams, other threads) race on it, so
//    serialise them.  Nothing in the array has to start at zero: every
//    intermediate is fully written before it is read;
//  * a kernel launch that fails inside goes through nfft_die (and its die
//    hook) like every launch of this library; an error left in the CUDA
//    context after the launches is returned as -2.
#include <cstring>
#include <mutex>

#include "../../include/nfft_gb300.h"
#include "gb_internal.h"

#define NOALLOC_MAX_NODES (1 << 18)
// keys, values and their ping-pong copies (4 x M u32) + radix histograms and
// scan blocks for M nodes (2 x 256 x M/4096 u32 + scan levels) with margin
#define NOALLOC_BYTES (4u * 4u * NOALLOC_MAX_NODES + 256u * 1024u)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64];  // device address of the scratch array, per device

void *scratch_for_current_device()
{
  int dev = 0;
  const cudaError_t ge = cudaGetDevice(&dev);
  if (ge != cudaSuccess) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: cudaGetDevice failed: %s", cudaGetErrorString(ge));
    return nullptr;
  }
  if (dev < 0 || dev >= 64) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: device %d is beyond the 64 devices it serves", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      gb::record_error("nfft_gb_sort_nodes_noalloc: cudaGetSymbolAddress failed: %s",
                       cudaGetErrorString(e));
      return nullptr;
    }
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

template <typename R>
int sort_noalloc(const R *x_dev, int d, const int *n, int m, int M, long long *index_x_dev,
                 cudaStream_t s)
{
  gb::Geom<R> g;
  memset(&g, 0, sizeof(g));
  g.d = d;
  g.m = m;
  g.w = 2 * m + 2;
  g.M = M;
  g.n_total = 1;
  for (int t = 0; t < GB_MAXD; ++t) {
    const int nt = t < d ? n[t] : 1;
    // keys are 32-bit: the product of the n_t must stay below 2^32 (checked
    // before each multiplication, so it cannot overflow)
    if (t < d && g.n_total > 0xffffffffLL / nt) {
      gb::record_error("nfft_gb_sort_nodes_noalloc: n_0 * ... * n_{d-1} must be below 2^32");
      return -1;
    }
    g.n[t] = nt;
    g.N[t] = nt;
    g.nR[t] = (R)nt;
    g.T[t] = nt;  // one tile: the tile keys are not used here
    g.ntile[t] = 1;
    g.ext[t] = 1;
    if (t < d) g.n_total *= nt;
  }
  g.cs = 1;
  g.csz = 1;
  g.sub = 1;
  unsigned char *base = (unsigned char *)scratch_for_current_device();
  if (!base) return -2;
  if (M == 0) return 0;
  const size_t Mz = (size_t)M;
  uint32_t *k1 = (uint32_t *)base;
  uint32_t *v1 = k1 + Mz;
  uint32_t *k2 = v1 + Mz;
  uint32_t *v2 = k2 + Mz;
  void *temp = (void *)(((uintptr_t)(v2 + Mz) + 255) & ~(uintptr_t)255);
  if ((unsigned char *)temp + gb::radix_temp_bytes(Mz) > base + NOALLOC_BYTES) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: scratch too small for M=%d", M);
    return -1;
  }
  // reference sort key into k1, node ids into v1 (the tile key goes to k2,
  // which the sort then uses as its ping-pong buffer)
  gb::launch_node_keys<R>(x_dev, g, k2, k1, v1, s);
  int bits = 0;
  while ((1LL << bits) < g.n_total) ++bits;
  gb::radix_sort_pairs(k1, v1, k2, v2, Mz, bits > 0 ? bits : 1, temp, s);
  gb::launch_ref_index_to_int64(k1, v1, M, index_x_dev, s);
  const cudaError_t le = cudaPeekAtLastError();
  if (le != cudaSuccess) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: CUDA error after the sort's launches: %s",
                     cudaGetErrorString(le));
    return -2;
  }
  return 0;
}

}  // namespace

extern "C" int nfft_gb_sort_nodes_noalloc(int single, const void *x_dev, int d, const int *n, int m,
                                          int M, long long *index_x_dev, void *stream)
{
  if (M > NOALLOC_MAX_NODES) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: M=%d exceeds the maximum of %d nodes", M,
                     NOALLOC_MAX_NODES);
    return -1;
  }
  if (d < 1 || d > GB_MAXD || m < 0 || M < 0 || !n || (M > 0 && (!x_dev || !index_x_dev))) {
    gb::record_error("nfft_gb_sort_nodes_noalloc: invalid arguments (d=%d, m=%d, M=%d)", d, m, M);
    return -1;
  }
  for (int t = 0; t < d; ++t)
    if (n[t] < 1) {
      gb::record_error("nfft_gb_sort_nodes_noalloc: n[%d]=%d must be positive", t, n[t]);
      return -1;
    }
  cudaStream_t s = (cudaStream_t)stream;
  return single ? sort_noalloc<float>((const float *)x_dev, d, n, m, M, index_x_dev, s)
                : sort_noalloc<double>((const double *)x_dev, d, n, m, M, index_x_dev, s);
}
