// gb_mri.cu -- MRI operators with a field inhomogeneity, reference
// kernel/mri/mri.c (double precision, as the reference).
//
// Samples of an image f_hat under an off-resonance map w (one value per
// pixel) at k-space nodes x_j read at times t_j:
//   f_j = sum_k f_hat_k exp(-2 pi i (k . x_j + w_k t_j N3))   (schematically)
// approximated, as in the reference, with the Kaiser-Bessel window of length
// N3 and oversampling sigma3 along the time / frequency axis:
//  * inh_2d1d: N3 + 1 two-dimensional NFFTs, one per time-window index l,
//    on f_hat_k exp(-2 pi i w_k l) / phi_hat(N3 w_k), whose results are
//    summed with the window phi(t_j - l / N3) (mri.c:57-102, adjoint 104-154);
//  * inh_3d: one three-dimensional NFFT whose third frequency axis holds
//    f_hat_k phi(w_k - l / N3), the results divided by phi_hat(N3 x_j3)
//    (mri.c:189-249).
// Here every elementwise step is a GPU kernel and the NFFTs run on the
// embedded plan's device buffers (the library's GPU NFFT); host arrays are
// read and written only at entry and exit.  Pointers stay put: where the
// reference swaps in freshly allocated f / f_hat arrays, the results are
// written into the caller's current arrays instead.
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <mutex>

#include "../../include/nfft3.h"
#include "../../include/nfft_gb300.h"
#include "gb_common.cuh"

namespace gb {

struct MriWin {
  int n, m;  // window length N3, cut-off m of the embedded plan
  double b;  // pi (2 - 1 / sigma3)
};

// the reference's PHI(n, x, 0) and PHI_HUT(n, k, 0) for the time window
__device__ __forceinline__ double mri_phi(double x, const MriWin &w)
{
  const double xn2 = x * (double)w.n * x * (double)w.n, mm = (double)w.m * (double)w.m;
  if (mm - xn2 > 0.0) {
    const double s = sqrt(mm - xn2);
    return sinh(w.b * s) / (3.14159265358979323846 * s);
  }
  if (mm - xn2 < 0.0) {
    const double s = sqrt(xn2 - mm);
    return sin(w.b * s) / (3.14159265358979323846 * s);
  }
  return w.b / 3.14159265358979323846;
}
__device__ __forceinline__ double mri_phi_hut(double k, const MriWin &w)
{
  const double a = 2.0 * 3.14159265358979323846 * k / (double)w.n;
  return cyl_bessel_i0((double)w.m * sqrt(w.b * w.b - a * a));
}
// the reference's support test |x| < m / n (strict)
__device__ __forceinline__ bool mri_in(double x, const MriWin &w) { return fabs(x) < w.m / (double)w.n; }

// 2d1d trafo, step l: g_k = f_hat_k exp(-2 pi i w_k l) / phi_hat(n w_k)
__global__ void k_mri_phase(long long N, int l, MriWin win, const double *__restrict__ w,
                            const double2 *__restrict__ fh, double2 *__restrict__ g)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  double s, c;
  sincospi(-2.0 * w[k] * (double)l, &s, &c);
  const double q = 1.0 / mri_phi_hut((double)win.n * w[k], win);
  const double2 a = fh[k];
  g[k] = make_double2((a.x * c - a.y * s) * q, (a.x * s + a.y * c) * q);
}

// 2d1d trafo, step l: acc_j += f_j phi(t_j - l / n) inside the window's support
__global__ void k_mri_tacc(long long M, int l, MriWin win, const double *__restrict__ t,
                           const double2 *__restrict__ f, double2 *__restrict__ acc)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const double x = t[j] - (double)l / (double)win.n;
  if (!mri_in(x, win)) return;
  const double p = mri_phi(x, win);
  acc[j].x += f[j].x * p;
  acc[j].y += f[j].y * p;
}

// 2d1d adjoint, step l: g_j = f_j phi(t_j - l / n) inside the support, else 0
__global__ void k_mri_twin(long long M, int l, MriWin win, const double *__restrict__ t,
                           const double2 *__restrict__ f, double2 *__restrict__ g)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const double x = t[j] - (double)l / (double)win.n;
  const double p = mri_in(x, win) ? mri_phi(x, win) : 0.0;
  g[j] = make_double2(f[j].x * p, f[j].y * p);
}

// 2d1d adjoint, step l: acc_k += h_k exp(+2 pi i w_k l); last: acc_k /= phi_hat(n w_k)
__global__ void k_mri_pacc(long long N, int l, bool last, MriWin win, const double *__restrict__ w,
                           const double2 *__restrict__ h, double2 *__restrict__ acc)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  double s, c;
  sincospi(2.0 * w[k] * (double)l, &s, &c);
  const double2 a = h[k];
  double2 r = acc[k];
  r.x += a.x * c - a.y * s;
  r.y += a.x * s + a.y * c;
  if (last) {
    const double q = 1.0 / mri_phi_hut((double)win.n * w[k], win);
    r.x *= q;
    r.y *= q;
  }
  acc[k] = r;
}

// 3d trafo: G[k n + l + n/2] = f_hat_k phi(w_k - l / n) inside the support, l in [-n/2, n/2)
__global__ void k_mri_fill3(long long N, MriWin win, const double *__restrict__ w, const double2 *__restrict__ fh,
                            double2 *__restrict__ G)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * win.n) return;
  const long long k = i / win.n;
  const int l = (int)(i - k * win.n) - win.n / 2;
  const double x = w[k] - (double)l / (double)win.n;
  const double p = mri_in(x, win) ? mri_phi(x, win) : 0.0;
  G[i] = make_double2(fh[k].x * p, fh[k].y * p);
}

// 3d: f_j /= phi_hat(n x_j3)
__global__ void k_mri_div3(long long M, MriWin win, const double *__restrict__ x, double2 *__restrict__ f)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const double q = 1.0 / mri_phi_hut((double)win.n * x[3 * j + 2], win);
  f[j].x *= q;
  f[j].y *= q;
}

// 3d adjoint: f_hat_k = sum_l G[k n + l + n/2] phi(w_k - l / n) inside the support
__global__ void k_mri_gather3(long long N, MriWin win, const double *__restrict__ w, const double2 *__restrict__ G,
                              double2 *__restrict__ fh)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  double2 r = make_double2(0.0, 0.0);
  for (int l = -win.n / 2; l < win.n / 2; ++l) {
    const double x = w[k] - (double)l / (double)win.n;
    if (!mri_in(x, win)) continue;
    const double p = mri_phi(x, win);
    const double2 a = G[k * win.n + l + win.n / 2];
    r.x += a.x * p;
    r.y += a.y * p;
  }
  fh[k] = r;
}

}  // namespace gb

// ---------------------------------------------------------------- host side
namespace {

struct MriCtx {
  gb::MriWin win;
  double *w_dev = nullptr, *t_dev = nullptr, *x_dev = nullptr;
  double2 *fh_dev = nullptr, *f_dev = nullptr, *acc_dev = nullptr;
  cudaStream_t s = nullptr;
  bool nodes_once = false;
};

std::mutex g_mri_mu;
std::map<const void *, MriCtx *> g_mri;

MriCtx *mctx(const void *p)
{
  std::lock_guard<std::mutex> lk(g_mri_mu);
  auto it = g_mri.find(p);
  if (it == g_mri.end()) gb::fatal("mri: plan not initialised by this library");
  return it->second;
}

unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

void new_ctx(const void *key, nfft_plan *plan, int N3, double sigma3, long long Nk, long long M, int d)
{
  MriCtx *c = new MriCtx();
  c->win.n = N3;
  c->win.m = (int)plan->m;
  c->win.b = 3.1415926535897932384626433832795028841971693993751 * (2.0 - 1.0 / sigma3);  // include/infft.h:216-222
  c->s = (cudaStream_t)nfft_gb_get_stream(plan);
  const size_t Mz = (size_t)(M > 0 ? M : 1), Nz = (size_t)(Nk > 0 ? Nk : 1);
  GB_CUDA(cudaMalloc((void **)&c->w_dev, Nz * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->t_dev, Mz * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->x_dev, Mz * d * sizeof(double)));
  GB_CUDA(cudaMalloc((void **)&c->fh_dev, Nz * sizeof(double2)));
  GB_CUDA(cudaMalloc((void **)&c->f_dev, Mz * sizeof(double2)));
  GB_CUDA(cudaMalloc((void **)&c->acc_dev, (Mz > Nz ? Mz : Nz) * sizeof(double2)));
  std::lock_guard<std::mutex> lk(g_mri_mu);
  g_mri[key] = c;
}

void free_ctx(const void *key)
{
  MriCtx *c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mri_mu);
    auto it = g_mri.find(key);
    if (it == g_mri.end()) return;
    c = it->second;
    g_mri.erase(it);
  }
  cudaStreamSynchronize(c->s);
  cudaFree(c->w_dev);
  cudaFree(c->t_dev);
  cudaFree(c->x_dev);
  cudaFree(c->fh_dev);
  cudaFree(c->f_dev);
  cudaFree(c->acc_dev);
  delete c;
}

// The embedded plan's node set-up on the device: once (the caller normally
// ran nfft_precompute_one_psi on it), or at every call when the plan has no
// precompute flag (the reference then reads the nodes inside every NFFT).
void plan_nodes(nfft_plan *plan, MriCtx *c)
{
  const bool pre = (plan->flags & (PRE_PSI | PRE_FULL_PSI | PRE_LIN_PSI | PRE_FG_PSI)) != 0;
  if (pre && c->nodes_once) return;
  if (!plan->x) gb::fatal("mri: nodes plan.x not set");
  const size_t bytes = (size_t)plan->M_total * plan->d * sizeof(double);
  if (bytes) GB_CUDA(cudaMemcpyAsync(nfft_gb_device_x(plan), plan->x, bytes, cudaMemcpyHostToDevice, c->s));
  GB_CUDA(cudaStreamSynchronize(c->s));
  nfft_gb_precompute_device(plan);
  c->nodes_once = true;
}

void h2d(MriCtx *c, void *d, const void *h, size_t n)
{
  if (n) GB_CUDA(cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, c->s));
}
void d2h(MriCtx *c, void *h, const void *d, size_t n)
{
  if (n) GB_CUDA(cudaMemcpyAsync(h, d, n, cudaMemcpyDeviceToHost, c->s));
}

}  // namespace

extern "C" {

void mri_inh_2d1d_init_guru(mri_inh_2d1d_plan *ths, int *N, int M, int *n, int m, double sigma, unsigned nfft_flags,
                            unsigned fftw_flags)
{
  // mri.c:156-172: a 2-D NFFT of N[0] x N[1], time window of length N[2]
  nfft_init_guru(&ths->plan, 2, N, M, n, m, nfft_flags, fftw_flags);
  ths->N3 = N[2];
  ths->sigma3 = sigma;
  ths->N_total = ths->plan.N_total;
  ths->M_total = ths->plan.M_total;
  ths->f = ths->plan.f;
  ths->f_hat = ths->plan.f_hat;
  ths->t = (double *)nfft_malloc((size_t)ths->M_total * sizeof(double));
  ths->w = (double *)nfft_malloc((size_t)ths->N_total * sizeof(double));
  ths->mv_trafo = (void (*)(void *))mri_inh_2d1d_trafo;
  ths->mv_adjoint = (void (*)(void *))mri_inh_2d1d_adjoint;
  new_ctx(ths, &ths->plan, ths->N3, sigma, ths->N_total, ths->M_total, 2);
}

void mri_inh_2d1d_trafo(mri_inh_2d1d_plan *ths)
{
  MriCtx *c = mctx(ths);
  nfft_plan *p = &ths->plan;
  plan_nodes(p, c);
  const long long N = ths->N_total, M = ths->M_total;
  h2d(c, c->w_dev, ths->w, (size_t)N * sizeof(double));
  h2d(c, c->t_dev, ths->t, (size_t)M * sizeof(double));
  h2d(c, c->fh_dev, ths->f_hat, (size_t)N * sizeof(double2));
  GB_CUDA(cudaMemsetAsync(c->acc_dev, 0, (size_t)M * sizeof(double2), c->s));
  double2 *pfh = (double2 *)nfft_gb_device_f_hat(p), *pf = (double2 *)nfft_gb_device_f(p);
  for (int l = -c->win.n / 2; l <= c->win.n / 2; ++l) {  // mri.c:74-90
    if (N) gb::k_mri_phase<<<nb(N), 256, 0, c->s>>>(N, l, c->win, c->w_dev, c->fh_dev, pfh);
    nfft_gb_trafo_device(p);
    if (M) gb::k_mri_tacc<<<nb(M), 256, 0, c->s>>>(M, l, c->win, c->t_dev, pf, c->acc_dev);
  }
  GB_LAUNCHED("mri_2d1d_trafo");
  d2h(c, ths->f, c->acc_dev, (size_t)M * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void mri_inh_2d1d_adjoint(mri_inh_2d1d_plan *ths)
{
  MriCtx *c = mctx(ths);
  nfft_plan *p = &ths->plan;
  plan_nodes(p, c);
  const long long N = ths->N_total, M = ths->M_total;
  h2d(c, c->w_dev, ths->w, (size_t)N * sizeof(double));
  h2d(c, c->t_dev, ths->t, (size_t)M * sizeof(double));
  h2d(c, c->f_dev, ths->f, (size_t)M * sizeof(double2));
  GB_CUDA(cudaMemsetAsync(c->acc_dev, 0, (size_t)N * sizeof(double2), c->s));
  double2 *pfh = (double2 *)nfft_gb_device_f_hat(p), *pf = (double2 *)nfft_gb_device_f(p);
  for (int l = -c->win.n / 2; l <= c->win.n / 2; ++l) {  // mri.c:122-144
    if (M) gb::k_mri_twin<<<nb(M), 256, 0, c->s>>>(M, l, c->win, c->t_dev, c->f_dev, pf);
    nfft_gb_adjoint_device(p);
    if (N) gb::k_mri_pacc<<<nb(N), 256, 0, c->s>>>(N, l, l == c->win.n / 2, c->win, c->w_dev, pfh, c->acc_dev);
  }
  GB_LAUNCHED("mri_2d1d_adjoint");
  d2h(c, ths->f_hat, c->acc_dev, (size_t)N * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void mri_inh_2d1d_finalize(mri_inh_2d1d_plan *ths)
{
  free_ctx(ths);
  nfft_free(ths->t);
  nfft_free(ths->w);
  ths->plan.f = ths->f;  // mri.c:174-181: the solver may have swapped them
  ths->plan.f_hat = ths->f_hat;
  nfft_finalize(&ths->plan);
}

void mri_inh_3d_init_guru(mri_inh_3d_plan *ths, int *N, int M, int *n, int m, double sigma, unsigned nfft_flags,
                          unsigned fftw_flags)
{
  // mri.c:251-264: a 3-D NFFT whose third axis (length N[2]) carries the field map
  ths->N3 = N[2];
  ths->sigma3 = sigma;
  nfft_init_guru(&ths->plan, 3, N, M, n, m, nfft_flags, fftw_flags);
  ths->N_total = (NFFT_INT)N[0] * N[1];
  ths->M_total = ths->plan.M_total;
  ths->f = ths->plan.f;
  ths->f_hat = (fftw_complex *)nfft_malloc((size_t)ths->N_total * sizeof(fftw_complex));
  ths->t = nullptr;
  ths->w = (double *)nfft_malloc((size_t)ths->N_total * sizeof(double));
  ths->mv_trafo = (void (*)(void *))mri_inh_3d_trafo;
  ths->mv_adjoint = (void (*)(void *))mri_inh_3d_adjoint;
  new_ctx(ths, &ths->plan, ths->N3, sigma, ths->N_total, ths->M_total, 3);
}

void mri_inh_3d_trafo(mri_inh_3d_plan *ths)
{
  MriCtx *c = mctx(ths);
  nfft_plan *p = &ths->plan;
  plan_nodes(p, c);
  const long long N = ths->N_total, M = ths->M_total;
  h2d(c, c->w_dev, ths->w, (size_t)N * sizeof(double));
  h2d(c, c->fh_dev, ths->f_hat, (size_t)N * sizeof(double2));
  h2d(c, c->x_dev, p->x, (size_t)M * 3 * sizeof(double));
  double2 *pfh = (double2 *)nfft_gb_device_f_hat(p), *pf = (double2 *)nfft_gb_device_f(p);
  if (N) gb::k_mri_fill3<<<nb(N * c->win.n), 256, 0, c->s>>>(N, c->win, c->w_dev, c->fh_dev, pfh);
  nfft_gb_trafo_device(p);
  if (M) gb::k_mri_div3<<<nb(M), 256, 0, c->s>>>(M, c->win, c->x_dev, pf);
  GB_LAUNCHED("mri_3d_trafo");
  d2h(c, ths->f, pf, (size_t)M * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void mri_inh_3d_adjoint(mri_inh_3d_plan *ths)
{
  MriCtx *c = mctx(ths);
  nfft_plan *p = &ths->plan;
  plan_nodes(p, c);
  const long long N = ths->N_total, M = ths->M_total;
  h2d(c, c->w_dev, ths->w, (size_t)N * sizeof(double));
  h2d(c, c->x_dev, p->x, (size_t)M * 3 * sizeof(double));
  double2 *pfh = (double2 *)nfft_gb_device_f_hat(p), *pf = (double2 *)nfft_gb_device_f(p);
  h2d(c, pf, ths->f, (size_t)M * sizeof(double2));
  if (M) gb::k_mri_div3<<<nb(M), 256, 0, c->s>>>(M, c->win, c->x_dev, pf);
  d2h(c, ths->f, pf, (size_t)M * sizeof(double2));  // mri.c:228-232 divides the caller's f in place
  nfft_gb_adjoint_device(p);
  if (N) gb::k_mri_gather3<<<nb(N), 256, 0, c->s>>>(N, c->win, c->w_dev, pfh, c->fh_dev);
  GB_LAUNCHED("mri_3d_adjoint");
  d2h(c, ths->f_hat, c->fh_dev, (size_t)N * sizeof(double2));
  GB_CUDA(cudaStreamSynchronize(c->s));
}

void mri_inh_3d_finalize(mri_inh_3d_plan *ths)
{
  free_ctx(ths);
  nfft_free(ths->w);
  nfft_free(ths->f_hat);
  nfft_finalize(&ths->plan);
}

}  // extern "C"
