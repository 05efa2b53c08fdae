// gb_nnfft.cu -- NNFFT: nonequispaced nodes in space (x) and frequency (v),
// reference kernel/nnfft/nnfft.c (double precision, as the reference).
//
//   f_j = sum_k f_hat_k exp(-2 pi i sum_t v_kt x_jt N_t)     (trafo)
//   f_hat_k = sum_j f_j exp(+2 pi i sum_t v_kt x_jt N_t)     (adjoint)
//
// The fast transform follows the reference's factorisation (nnfft.c:291-343):
//  * B^T: every frequency node v_k is spread with the Kaiser-Bessel window of
//    grid length N1 (cut-off m, b = pi (2 - N/N1)) onto an aN1 equispaced
//    frequency grid, which is the f_hat of an inner NFFT of bandwidth aN1;
//  * the inner NFFT (this library's GPU plan) at the nodes x / sigma,
//    sigma = N1 / N;
//  * D: f_j times prod_t 1 / phi_hat_t(x_jt N_t) of the outer window.
// The adjoint runs the transposed steps in reverse.  Here B^T and B are GPU
// kernels over the frequency nodes (one thread per node and first-dimension
// tap, FP64 atomics for B^T), D is a GPU kernel, and the inner NFFT runs on
// device buffers; host arrays are only touched at the API boundary.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/nfft3.h"
#include "../../include/nfft_gb300.h"
#include "gb_common.cuh"

namespace gb {

struct NnGeom {
  int d, m;
  int N[GB_MAXD], N1[GB_MAXD], aN1[GB_MAXD];
  double b[GB_MAXD];
  long long Nt;  // frequency nodes
  long long M;   // space nodes
};

// the reference's window PHI(n, x, t) (include/infft.h:209-215) in double
__device__ __forceinline__ double nn_phi(double x, int n, int m, double b)
{
  const double xn2 = x * (double)n * x * (double)n;
  const double mm = (double)m * (double)m;
  if (mm - xn2 > 0.0) {
    const double s = sqrt(mm - xn2);
    return sinh(b * s) / (3.14159265358979323846 * s);
  }
  if (mm - xn2 < 0.0) {
    const double s = sqrt(xn2 - mm);
    return sin(b * s) / (3.14159265358979323846 * s);
  }
  return b / 3.14159265358979323846;
}

// first window index of frequency node v in one dimension (nnfft.c:86-103):
// u = trunc(v n), one lower when v n < 0, then minus m
__device__ __forceinline__ int nn_u(double v, int n, int m)
{
  const double c = v * (double)n;
  int u = (int)c;
  if (c < 0) u -= 1;
  return u - m;
}

// one thread per (frequency node k, tap i0 of the first dimension); the
// remaining dimensions' taps are looped.  adj == false: B^T (spread f_hat
// into F); adj == true: B (gather F into f_hat).
template <bool GATHER>
__global__ void k_nn_b(NnGeom g, const double *__restrict__ v, double2 *__restrict__ fhat, double2 *__restrict__ F)
{
  const int w = 2 * g.m + 2;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.Nt * w) return;
  const long long k = idx / w;
  const int i0 = (int)(idx - k * w);
  int u[GB_MAXD], lj[GB_MAXD];
  for (int t = 0; t < g.d; ++t) {
    u[t] = nn_u(v[k * g.d + t], g.N1[t], g.m);
    lj[t] = 0;
  }
  lj[0] = i0;
  long long taps = 1;
  for (int t = 1; t < g.d; ++t) taps *= w;
  double2 val = GATHER ? make_double2(0.0, 0.0) : fhat[k];
  double2 acc = make_double2(0.0, 0.0);
  for (long long q = 0; q < taps; ++q) {
    double phi = 1.0;
    long long li = 0;
    for (int t = 0; t < g.d; ++t) {
      const int l = u[t] + lj[t];
      phi *= nn_phi(-v[k * g.d + t] + (double)l / (double)g.N1[t], g.N1[t], g.m, g.b[t]);
      li = li * g.aN1[t] + (l + g.aN1[t] * 3 / 2) % g.aN1[t];
    }
    if (GATHER) {
      const double2 c = F[li];
      acc.x += phi * c.x;
      acc.y += phi * c.y;
    } else {
      atomicAdd(&F[li].x, phi * val.x);
      atomicAdd(&F[li].y, phi * val.y);
    }
    for (int t = g.d - 1; t >= 1; --t) {  // next tap of dimensions 1..d-1
      if (++lj[t] < w) break;
      lj[t] = 0;
    }
  }
  if (GATHER) {
    atomicAdd(&fhat[k].x, acc.x);
    atomicAdd(&fhat[k].y, acc.y);
  }
}

// c[j] = prod_t 1 / phi_hat(N1_t, x_jt N_t) (nnfft.c:347-362, include/infft.h:208)
__global__ void k_nn_cphi(NnGeom g, const double *__restrict__ x, double *__restrict__ c)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.M) return;
  double p = 1.0;
  for (int t = 0; t < g.d; ++t) {
    const double k = x[j * g.d + t] * (double)g.N[t];
    const double a = 2.0 * 3.14159265358979323846 * k / (double)g.N1[t];
    p *= 1.0 / cyl_bessel_i0((double)g.m * sqrt(g.b[t] * g.b[t] - a * a));
  }
  c[j] = p;
}

__global__ void k_nn_scale(long long M, const double *__restrict__ c, double2 *__restrict__ f)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < M) {
    f[j].x *= c[j];
    f[j].y *= c[j];
  }
}

// direct NNDFT (nnfft.c:40-84): one thread per output, FP64
template <bool ADJ>
__global__ void k_nndft(NnGeom g, const double *__restrict__ x, const double *__restrict__ v,
                        const double2 *__restrict__ in, double2 *__restrict__ out)
{
  const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nout = ADJ ? g.Nt : g.M, nin = ADJ ? g.M : g.Nt;
  if (o >= nout) return;
  const double sgn = ADJ ? 2.0 * 3.14159265358979323846 : -2.0 * 3.14159265358979323846;
  double re = 0.0, im = 0.0;
  for (long long q = 0; q < nin; ++q) {
    const long long j = ADJ ? q : o, k = ADJ ? o : q;
    double om = 0.0;
    for (int t = 0; t < g.d; ++t) om += v[k * g.d + t] * x[j * g.d + t] * (double)g.N[t];
    double s, c;
    sincos(sgn * om, &s, &c);
    const double2 a = in[q];
    re += a.x * c - a.y * s;
    im += a.x * s + a.y * c;
  }
  out[o] = make_double2(re, im);
}

}  // namespace gb

// ---------------------------------------------------------------- host side
namespace {

struct NnCtx {
  gb::NnGeom g;
  double *v_dev = nullptr, *x_dev = nullptr, *cphi_dev = nullptr;
  double2 *fhat_dev = nullptr, *f_dev = nullptr;  // for the direct transforms
  cudaStream_t s = nullptr;
  bool nodes_set = false;  // inner node set-up done by precompute_one_psi
  bool cphi_set = false;   // D factors from precompute_phi_hut
};

std::mutex g_nn_mu;
std::map<const nnfft_plan *, NnCtx *> g_nn;

NnCtx *ctx(const nnfft_plan *p)
{
  std::lock_guard<std::mutex> lk(g_nn_mu);
  auto it = g_nn.find(p);
  if (it == g_nn.end()) gb::fatal("nnfft: plan not initialised by this library");
  return it->second;
}

unsigned blocks(long long n, int th) { return (unsigned)((n + th - 1) / th); }

// the inner NFFT's nodes x / sigma (nnfft.c:296-300) on its device copy, then
// its node set-up
void inner_nodes(nnfft_plan *ths, NnCtx *c)
{
  const long long n = (long long)ths->M_total * ths->d;
  std::vector<double> xs((size_t)n);
  for (long long j = 0; j < ths->M_total; ++j)
    for (int t = 0; t < ths->d; ++t) xs[j * ths->d + t] = ths->x[j * ths->d + t] / ths->sigma[t];
  void *xd = nfft_gb_device_x(ths->direct_plan);
  GB_CUDA(cudaMemcpyAsync(xd, xs.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
  nfft_gb_precompute_device(ths->direct_plan);
}

// D factors from the host nodes (device and, with PRE_PHI_HUT, host copy)
void d_factors(nnfft_plan *ths, NnCtx *c)
{
  const long long M = ths->M_total;
  if (M == 0) return;
  GB_CUDA(cudaMemcpyAsync(c->x_dev, ths->x, (size_t)M * ths->d * sizeof(double), cudaMemcpyHostToDevice, c->s));
  gb::k_nn_cphi<<<blocks(M, 256), 256, 0, c->s>>>(c->g, c->x_dev, c->cphi_dev);
  GB_LAUNCHED("nn_cphi");
  if (ths->c_phi_inv)
    GB_CUDA(cudaMemcpyAsync(ths->c_phi_inv, c->cphi_dev, (size_t)M * sizeof(double), cudaMemcpyDeviceToHost, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void init_help(nnfft_plan *ths, int m2, unsigned nfft_flags, unsigned fftw_flags)
{
  const int d = ths->d;
  if (d < 1 || d > GB_MAXD) gb::fatal("nnfft: dimension %d not supported (1..%d)", d, GB_MAXD);
  ths->aN1 = (int *)nfft_malloc((size_t)d * sizeof(int));
  ths->a = (double *)nfft_malloc((size_t)d * sizeof(double));
  ths->sigma = (double *)nfft_malloc((size_t)d * sizeof(double));
  ths->b = (double *)nfft_malloc((size_t)d * sizeof(double));
  ths->n = ths->N1;
  ths->aN1_total = 1;
  std::vector<int> N2(d);
  for (int t = 0; t < d; ++t) {  // nnfft.c:504-519
    ths->a[t] = 1.0 + (2.0 * (double)ths->m) / (double)ths->N1[t];
    ths->aN1[t] = (int)(ths->a[t] * (double)ths->N1[t]);
    if (ths->aN1[t] % 2 != 0) ths->aN1[t] += 1;
    ths->aN1_total *= ths->aN1[t];
    ths->sigma[t] = (double)ths->N1[t] / (double)ths->N[t];
    N2[t] = (int)ceil(ths->sigma[t] * ths->aN1[t]);
    if (N2[t] % 2 != 0) N2[t] += 1;
    ths->b[t] = 3.1415926535897932384626433832795028841971693993751 * (2.0 - 1.0 / ths->sigma[t]);
  }
  if (ths->nnfft_flags & MALLOC_X) ths->x = (double *)nfft_malloc((size_t)d * ths->M_total * sizeof(double));
  if (ths->nnfft_flags & MALLOC_F) ths->f = (fftw_complex *)nfft_malloc((size_t)ths->M_total * sizeof(fftw_complex));
  if (ths->nnfft_flags & MALLOC_V) ths->v = (double *)nfft_malloc((size_t)d * ths->N_total * sizeof(double));
  if (ths->nnfft_flags & MALLOC_F_HAT)
    ths->f_hat = (fftw_complex *)nfft_malloc((size_t)ths->N_total * sizeof(fftw_complex));
  // the window is evaluated on the fly: no psi table (as the library's NFFT plans)
  ths->psi = nullptr;
  ths->psi_index_g = ths->psi_index_f = nullptr;
  ths->c_phi_inv = nullptr;
  ths->K = (ths->nnfft_flags & PRE_LIN_PSI) ? (int)((1U << 10) * (ths->m + 1)) : 0;
  ths->direct_plan = (nfft_plan *)nfft_malloc(sizeof(nfft_plan));
  nfft_init_guru(ths->direct_plan, d, ths->aN1, ths->M_total, N2.data(), m2, nfft_flags, fftw_flags);
  ths->direct_plan->x = ths->x;
  ths->direct_plan->f = ths->f;
  ths->F = ths->direct_plan->f_hat;
  ths->mv_trafo = (void (*)(void *))nnfft_trafo;
  ths->mv_adjoint = (void (*)(void *))nnfft_adjoint;

  NnCtx *c = new NnCtx();
  c->g.d = d;
  c->g.m = ths->m;
  for (int t = 0; t < d; ++t) {
    c->g.N[t] = ths->N[t];
    c->g.N1[t] = ths->N1[t];
    c->g.aN1[t] = ths->aN1[t];
    c->g.b[t] = ths->b[t];
  }
  c->g.Nt = ths->N_total;
  c->g.M = ths->M_total;
  c->s = (cudaStream_t)nfft_gb_get_stream(ths->direct_plan);
  const size_t Mz = (size_t)(ths->M_total > 0 ? ths->M_total : 1), Nz = (size_t)(ths->N_total > 0 ? ths->N_total : 1);
  GB_CUDA(cudaMalloc((void **)&c->v_dev, Nz * d * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->x_dev, Mz * d * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->cphi_dev, Mz * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->fhat_dev, Nz * sizeof(double2)));
  GB_CUDA(cudaMalloc((void **)&c->f_dev, Mz * sizeof(double2)));
  std::lock_guard<std::mutex> lk(g_nn_mu);
  g_nn[ths] = c;
}

void upload(NnCtx *c, void *dst, const void *src, size_t bytes)
{
  if (bytes) GB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->s));
}
void download(NnCtx *c, void *dst, const void *src, size_t bytes)
{
  if (bytes) GB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->s));
}

// inner nodes and D factors for a transform: from precompute_one_psi where it
// ran (PRE_PSI / PRE_FULL_PSI / PRE_PHI_HUT), else from the current x, as the
// reference evaluates them inside every call
void prepare(nnfft_plan *ths, NnCtx *c)
{
  if (!ths->x || !ths->v) gb::fatal("nnfft: x or v not set");
  if (!c->nodes_set) inner_nodes(ths, c);
  if (!c->cphi_set) d_factors(ths, c);
}

}  // namespace

extern "C" {

void nnfft_init_guru(nnfft_plan *ths, int d, int N_total, int M_total, int *N, int *N1, int m, unsigned nnfft_flags)
{
  // nnfft.c:577-611
  ths->d = d;
  ths->M_total = M_total;
  ths->N_total = N_total;
  ths->m = m;
  ths->nnfft_flags = nnfft_flags;
  const unsigned fftw_flags = FFTW_ESTIMATE | FFTW_DESTROY_INPUT;
  unsigned nfft_flags = PRE_PHI_HUT | MALLOC_F_HAT | FFTW_INIT | ((d == 1) ? FFT_OUT_OF_PLACE : 0U) |
                        NFFT_OMP_BLOCKWISE_ADJOINT;
  nfft_flags |= nnfft_flags & (PRE_PSI | PRE_FULL_PSI | PRE_LIN_PSI);
  ths->N = (int *)nfft_malloc((size_t)d * sizeof(int));
  ths->N1 = (int *)nfft_malloc((size_t)d * sizeof(int));
  for (int t = 0; t < d; ++t) {
    ths->N[t] = N[t];
    ths->N1[t] = N1[t];
  }
  init_help(ths, m, nfft_flags, fftw_flags);
}

void nnfft_init(nnfft_plan *ths, int d, int N_total, int M_total, int *N)
{
  // nnfft.c:613-650: m of the double-precision Kaiser-Bessel default, N1 = 1.5 N made even
  ths->d = d;
  ths->M_total = M_total;
  ths->N_total = N_total;
  ths->m = 8;
  ths->N = (int *)nfft_malloc((size_t)d * sizeof(int));
  ths->N1 = (int *)nfft_malloc((size_t)d * sizeof(int));
  for (int t = 0; t < d; ++t) {
    ths->N[t] = N[t];
    ths->N1[t] = (int)ceil(1.5 * N[t]);
    if (ths->N1[t] % 2 != 0) ths->N1[t] += 1;
  }
  ths->nnfft_flags = PRE_PSI | PRE_PHI_HUT | MALLOC_X | MALLOC_V | MALLOC_F_HAT | MALLOC_F;
  const unsigned nfft_flags = PRE_PSI | PRE_PHI_HUT | MALLOC_F_HAT | FFTW_INIT | ((d == 1) ? FFT_OUT_OF_PLACE : 0U) |
                              NFFT_OMP_BLOCKWISE_ADJOINT;
  init_help(ths, ths->m, nfft_flags, FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
}

void nnfft_init_1d(nnfft_plan *ths, int N1, int M_total) { nnfft_init(ths, 1, N1, M_total, &N1); }

void nnfft_precompute_phi_hut(nnfft_plan *ths)
{
  NnCtx *c = ctx(ths);
  if (!ths->c_phi_inv) ths->c_phi_inv = (double *)nfft_malloc((size_t)ths->M_total * sizeof(double));
  d_factors(ths, c);
  c->cphi_set = true;
}

// PRE_PSI / PRE_FULL_PSI: the inner NFFT's node set-up at the current x (the
// reference's psi tables for the outer window are evaluated on the fly here)
void nnfft_precompute_psi(nnfft_plan *ths)
{
  NnCtx *c = ctx(ths);
  inner_nodes(ths, c);
  c->nodes_set = true;
}
void nnfft_precompute_full_psi(nnfft_plan *ths) { nnfft_precompute_psi(ths); }
// PRE_LIN_PSI: the reference fills a lookup table of the outer window and the
// inner plan's; both are evaluated on the fly, and the nodes are read per call
void nnfft_precompute_lin_psi(nnfft_plan *ths) { (void)ctx(ths); }

void nnfft_precompute_one_psi(nnfft_plan *ths)
{
  // nnfft.c:481-492
  if (ths->nnfft_flags & PRE_PSI) nnfft_precompute_psi(ths);
  if (ths->nnfft_flags & PRE_FULL_PSI) nnfft_precompute_full_psi(ths);
  if (ths->nnfft_flags & PRE_LIN_PSI) nnfft_precompute_lin_psi(ths);
  if (ths->nnfft_flags & PRE_PHI_HUT) nnfft_precompute_phi_hut(ths);
}

void nnfft_trafo(nnfft_plan *ths)
{
  // nnfft.c:291-317: B^T, inner NFFT at x / sigma, D
  NnCtx *c = ctx(ths);
  prepare(ths, c);
  const int w = 2 * ths->m + 2;
  upload(c, c->v_dev, ths->v, (size_t)ths->N_total * ths->d * sizeof(double));
  upload(c, c->fhat_dev, ths->f_hat, (size_t)ths->N_total * sizeof(double2));
  double2 *F = (double2 *)nfft_gb_device_f_hat(ths->direct_plan);
  double2 *f = (double2 *)nfft_gb_device_f(ths->direct_plan);
  GB_CUDA(cudaMemsetAsync(F, 0, (size_t)ths->aN1_total * sizeof(double2), c->s));
  if (ths->N_total > 0) {
    gb::k_nn_b<false><<<blocks((long long)ths->N_total * w, 128), 128, 0, c->s>>>(c->g, c->v_dev, c->fhat_dev, F);
    GB_LAUNCHED("nn_bt");
  }
  nfft_gb_trafo_device(ths->direct_plan);
  if (ths->M_total > 0) {
    gb::k_nn_scale<<<blocks(ths->M_total, 256), 256, 0, c->s>>>(ths->M_total, c->cphi_dev, f);
    GB_LAUNCHED("nn_d");
  }
  download(c, ths->f, f, (size_t)ths->M_total * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void nnfft_adjoint(nnfft_plan *ths)
{
  // nnfft.c:319-343: D (in place on f, as the reference), inner adjoint, B
  NnCtx *c = ctx(ths);
  prepare(ths, c);
  const int w = 2 * ths->m + 2;
  double2 *F = (double2 *)nfft_gb_device_f_hat(ths->direct_plan);
  double2 *f = (double2 *)nfft_gb_device_f(ths->direct_plan);
  upload(c, f, ths->f, (size_t)ths->M_total * sizeof(double2));
  upload(c, c->v_dev, ths->v, (size_t)ths->N_total * ths->d * sizeof(double));
  if (ths->M_total > 0) {
    gb::k_nn_scale<<<blocks(ths->M_total, 256), 256, 0, c->s>>>(ths->M_total, c->cphi_dev, f);
    GB_LAUNCHED("nn_d");
  }
  download(c, ths->f, f, (size_t)ths->M_total * sizeof(double2));
  nfft_gb_adjoint_device(ths->direct_plan);
  GB_CUDA(cudaMemsetAsync(c->fhat_dev, 0, (size_t)ths->N_total * sizeof(double2), c->s));
  if (ths->N_total > 0) {
    gb::k_nn_b<true><<<blocks((long long)ths->N_total * w, 128), 128, 0, c->s>>>(c->g, c->v_dev, c->fhat_dev, F);
    GB_LAUNCHED("nn_b");
  }
  download(c, ths->f_hat, c->fhat_dev, (size_t)ths->N_total * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

static void nndft(nnfft_plan *ths, bool adj)
{
  NnCtx *c = ctx(ths);
  const size_t M = (size_t)ths->M_total, Nt = (size_t)ths->N_total;
  upload(c, c->x_dev, ths->x, M * ths->d * sizeof(double));
  upload(c, c->v_dev, ths->v, Nt * ths->d * sizeof(double));
  if (adj) {
    upload(c, c->f_dev, ths->f, M * sizeof(double2));
    if (Nt) gb::k_nndft<true><<<blocks((long long)Nt, 128), 128, 0, c->s>>>(c->g, c->x_dev, c->v_dev, c->f_dev, c->fhat_dev);
    download(c, ths->f_hat, c->fhat_dev, Nt * sizeof(double2));
  } else {
    upload(c, c->fhat_dev, ths->f_hat, Nt * sizeof(double2));
    if (M) gb::k_nndft<false><<<blocks((long long)M, 128), 128, 0, c->s>>>(c->g, c->x_dev, c->v_dev, c->fhat_dev, c->f_dev);
    download(c, ths->f, c->f_dev, M * sizeof(double2));
  }
  GB_LAUNCHED("nndft");
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void nnfft_trafo_direct(nnfft_plan *ths) { nndft(ths, false); }
void nnfft_adjoint_direct(nnfft_plan *ths) { nndft(ths, true); }

void nnfft_finalize(nnfft_plan *ths)
{
  // nnfft.c:657-693
  NnCtx *c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_nn_mu);
    auto it = g_nn.find(ths);
    if (it != g_nn.end()) {
      c = it->second;
      g_nn.erase(it);
    }
  }
  if (c) {
    cudaStreamSynchronize(c->s);
    cudaFree(c->v_dev);
    cudaFree(c->x_dev);
    cudaFree(c->cphi_dev);
    cudaFree(c->fhat_dev);
    cudaFree(c->f_dev);
    delete c;
  }
  nfft_finalize(ths->direct_plan);
  nfft_free(ths->direct_plan);
  nfft_free(ths->aN1);
  nfft_free(ths->a);
  nfft_free(ths->sigma);
  nfft_free(ths->b);
  nfft_free(ths->N);
  nfft_free(ths->N1);
  if (ths->c_phi_inv) nfft_free(ths->c_phi_inv);
  if (ths->nnfft_flags & MALLOC_F) nfft_free(ths->f);
  if (ths->nnfft_flags & MALLOC_F_HAT) nfft_free(ths->f_hat);
  if (ths->nnfft_flags & MALLOC_X) nfft_free(ths->x);
  if (ths->nnfft_flags & MALLOC_V) nfft_free(ths->v);
}

}  // extern "C"
