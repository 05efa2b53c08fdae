// gb_solver.cu -- the inverse NFFT solver (solver_plan_complex) on the GPU.
//
// Reference: kernel/solver/solver.c -- init_advanced_complex (40-74),
// before_loop_complex (81-125), Landweber (128-178), steepest descent
// (181-229), CGNR (232-292), CGNE (295-344), loop_one_step (347-360),
// finalize (363-385); BLAS-1 helpers kernel/util/vector1.c:22-57,
// vector2.c:22-74, vector3.c:22-93.
//
// When the solver's mv plan is an nfft_plan of this library, the whole
// iteration stays in HBM: the transforms read and write the solver's device
// vectors directly in place of the reference's pointer swaps (solver.c:85-87,
// 106-108, ...), the step sizes alpha / beta are computed on the device from
// FP64 inner products (no host round trip inside an iteration), a step's
// launches replay as one CUDA graph, and only the scalars and the
// user-visible vectors are copied back at the end of each call.  Inner
// products accumulate in FP64 for both precisions.
//
// Any other mv plan (a user operator with its own mv_trafo / mv_adjoint)
// runs the same algorithm on the host through its function pointers.
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/nfft3.h"
#include "../../include/nfft_gb300.h"
#include "gb_internal.h"

namespace gb {

template <typename R> struct SApi;
template <> struct SApi<double> {
  typedef solver_plan_complex splan;
  typedef nfft_mv_plan_complex mvplan;
  typedef nfft_plan plan;
  static void *mal(size_t n) { return nfft_malloc(n); }
  static void fre(void *p) { nfft_free(p); }
  static bool ours(const mvplan *mv) { return mv->mv_trafo == (void (*)(void *))nfft_trafo; }
  static void *dev_fhat(plan *p) { return nfft_gb_device_f_hat(p); }
  static void *dev_f(plan *p) { return nfft_gb_device_f(p); }
  static void *stream(plan *p) { return nfft_gb_get_stream(p); }
  static void *dev_x(plan *p) { return nfft_gb_device_x(p); }
  static void trafo_dev(plan *p) { nfft_gb_trafo_device(p); }
  static void adjoint_dev(plan *p) { nfft_gb_adjoint_device(p); }
  static void trafo_ptr(plan *p, const void *fh, void *f) { nfft_gb_trafo_ptr(p, fh, f); }
  static void adjoint_ptr(plan *p, const void *f, void *fh) { nfft_gb_adjoint_ptr(p, f, fh); }
  static unsigned long long gen(plan *p) { return nfft_gb_generation(p); }
};
template <> struct SApi<float> {
  typedef solverf_plan_complex splan;
  typedef nfftf_mv_plan_complex mvplan;
  typedef nfftf_plan plan;
  static void *mal(size_t n) { return nfftf_malloc(n); }
  static void fre(void *p) { nfftf_free(p); }
  static bool ours(const mvplan *mv) { return mv->mv_trafo == (void (*)(void *))nfftf_trafo; }
  static void *dev_fhat(plan *p) { return nfftf_gb_device_f_hat(p); }
  static void *dev_f(plan *p) { return nfftf_gb_device_f(p); }
  static void *stream(plan *p) { return nfftf_gb_get_stream(p); }
  static void *dev_x(plan *p) { return nfftf_gb_device_x(p); }
  static void trafo_dev(plan *p) { nfftf_gb_trafo_device(p); }
  static void adjoint_dev(plan *p) { nfftf_gb_adjoint_device(p); }
  static void trafo_ptr(plan *p, const void *fh, void *f) { nfftf_gb_trafo_ptr(p, fh, f); }
  static void adjoint_ptr(plan *p, const void *f, void *fh) { nfftf_gb_adjoint_ptr(p, f, fh); }
  static unsigned long long gen(plan *p) { return nfftf_gb_generation(p); }
};


// device scalars (FP64): indices into SolverState::scal
enum { S_ALPHA = 0, S_BETA, S_DOT_R, S_DOT_R_OLD, S_DOT_Z, S_DOT_Z_OLD, S_DOT_P, S_DOT_V, S_COUNT };
// what a reduction finishes into
enum {
  F_DOT_V_ALPHA = 0,  // dot_v = s; alpha = dot_z / dot_v
  F_DOT_R,            // dot_r = s
  F_DOT_R_BETA,       // dot_r_old = dot_r; dot_r = s; beta = dot_r / dot_r_old
  F_DOT_Z,            // dot_z = s
  F_DOT_Z_BETA,       // dot_z_old = dot_z; dot_z = s; beta = dot_z / dot_z_old
  F_DOT_P,            // dot_p = s
  F_ALPHA_CGNE        // alpha = dot_r / dot_p (no reduction)
};

static constexpr int RED_BLOCKS = 152;  // one per SM: few partial sums for the finishing block
static constexpr int RED_THREADS = 256;

// ---------------------------------------------------------------- kernels
template <typename R>
__global__ void k_scale_copy(typename Cx<R>::T *__restrict__ dst, const typename Cx<R>::T *__restrict__ src,
                             const R *__restrict__ w, long long n)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    typename Cx<R>::T v = src[k];
    if (w) {
      v.x *= w[k];
      v.y *= w[k];
    }
    dst[k] = v;
  }
}

// x += sign * scal[idx] * w * y   (upd_xpay / upd_xpawy).  The vector
// updates of a single-precision solver run in single precision (the scalar
// rounded once to float, one FMA per component): FP64 stays with the inner
// products and norms, where it decides the iteration; GB300's FP64 rate is a
// small fraction of its FP32 rate.
template <typename R>
__global__ void k_upd(typename Cx<R>::T *__restrict__ x, const typename Cx<R>::T *__restrict__ y,
                      const R *__restrict__ w, long long n, const double *__restrict__ scal, int idx,
                      double sign)
{
  const double a = sign * scal[idx];
  const R ar = (R)a;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    typename Cx<R>::T v = x[k];
    const typename Cx<R>::T u = y[k];
    if constexpr (std::is_same<R, float>::value) {
      const float c = w ? ar * w[k] : ar;
      v.x = fmaf(c, u.x, v.x);
      v.y = fmaf(c, u.y, v.y);
    } else {
      const double c = w ? a * (double)w[k] : a;
      v.x = (R)((double)v.x + c * (double)u.x);
      v.y = (R)((double)v.y + c * (double)u.y);
    }
    x[k] = v;
  }
}

// x = a x + y with a = scal[idx] (idx >= 0) or a = -1 (idx < 0)   (upd_axpy)
template <typename R>
__global__ void k_axpy(typename Cx<R>::T *__restrict__ x, const typename Cx<R>::T *__restrict__ y, long long n,
                       const double *__restrict__ scal, int idx)
{
  const double a = idx >= 0 ? scal[idx] : -1.0;
  const R ar = (R)a;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    typename Cx<R>::T v = x[k];
    const typename Cx<R>::T u = y[k];
    if constexpr (std::is_same<R, float>::value) {
      v.x = fmaf(ar, v.x, u.x);
      v.y = fmaf(ar, v.y, u.y);
    } else {
      v.x = (R)(a * (double)v.x + (double)u.x);
      v.y = (R)(a * (double)v.y + (double)u.y);
    }
    x[k] = v;
  }
}

// The scalar update that ends a reduction (s = the reduced value).
__device__ __forceinline__ void finish_op(double s, double *__restrict__ scal, int op)
{
  switch (op) {
    case F_DOT_V_ALPHA:
      scal[S_DOT_V] = s;
      scal[S_ALPHA] = scal[S_DOT_Z] / s;
      break;
    case F_DOT_R:
      scal[S_DOT_R] = s;
      break;
    case F_DOT_R_BETA:
      scal[S_DOT_R_OLD] = scal[S_DOT_R];
      scal[S_DOT_R] = s;
      scal[S_BETA] = s / scal[S_DOT_R_OLD];
      break;
    case F_DOT_Z:
      scal[S_DOT_Z] = s;
      break;
    case F_DOT_Z_BETA:
      scal[S_DOT_Z_OLD] = scal[S_DOT_Z];
      scal[S_DOT_Z] = s;
      scal[S_BETA] = s / scal[S_DOT_Z_OLD];
      break;
    case F_DOT_P:
      scal[S_DOT_P] = s;
      break;
    case F_ALPHA_CGNE:
      scal[S_ALPHA] = scal[S_DOT_R] / scal[S_DOT_P];
      break;
  }
}

// one warp: lane l sums part[l], part[l + 32], ... and a butterfly adds the
// lanes (a fixed order, so the result does not vary between runs)
__device__ __forceinline__ double sum_parts(const volatile double *part, int nblk)
{
  double s = 0.0;
  for (int i = threadIdx.x & 31; i < nblk; i += 32) s += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

__global__ void k_finish(const double *__restrict__ part, int nblk, double *__restrict__ scal, int op)
{
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const double s = op != F_ALPHA_CGNE ? sum_parts(part, nblk) : 0.0;
  if (threadIdx.x == 0) finish_op(s, scal, op);
}

// Block sum of the threads' values v into part[blockIdx.x]; the block that
// finishes last (ticket) then adds the blocks' sums in a fixed order,
// applies the scalar update and resets the ticket for the next reduction.
__device__ __forceinline__ void reduce_and_finish(double v, double *__restrict__ part, unsigned *__restrict__ ticket,
                                                  double *__restrict__ scal, int op)
{
  __shared__ double sm[RED_THREADS / 32];
  __shared__ bool last;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < RED_THREADS / 32; ++i) t += sm[i];
    part[blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x < 32) {
    __threadfence();
    const double s = sum_parts(part, gridDim.x);
    if (threadIdx.x == 0) {
      finish_op(s, scal, op);
      *ticket = 0;
    }
  }
}

// sum of w |x|^2 (w == nullptr: |x|^2) and its scalar update, one launch
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_dot(const typename Cx<R>::T *__restrict__ x,
                                                     const R *__restrict__ w, long long n,
                                                     double *__restrict__ part, unsigned *__restrict__ ticket,
                                                     double *__restrict__ scal, int op)
{
  double s = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const typename Cx<R>::T v = x[k];
    const double a = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
    s += w ? (double)w[k] * a : a;
  }
  reduce_and_finish(s, part, ticket, scal, op);
}

// f_hat += alpha wh .* p (N values, skipped when p == nullptr) and
// r -= alpha v (M values), then the sum of w |r|^2 and its scalar update
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_upd_dot(typename Cx<R>::T *__restrict__ fh,
                                                         const typename Cx<R>::T *__restrict__ p,
                                                         const R *__restrict__ wh, long long N,
                                                         typename Cx<R>::T *__restrict__ r,
                                                         const typename Cx<R>::T *__restrict__ v,
                                                         const R *__restrict__ w, long long M,
                                                         double *__restrict__ part, unsigned *__restrict__ ticket,
                                                         double *__restrict__ scal, int op)
{
  const double a = scal[S_ALPHA];
  const R ar = (R)a;
  constexpr bool SP = std::is_same<R, float>::value;  // single precision: FP32 updates (see k_upd)
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long k0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p)
    for (long long k = k0; k < N; k += stride) {
      typename Cx<R>::T u = fh[k];
      const typename Cx<R>::T d = p[k];
      if constexpr (SP) {
        const float c = wh ? ar * wh[k] : ar;
        u.x = fmaf(c, d.x, u.x);
        u.y = fmaf(c, d.y, u.y);
      } else {
        const double c = wh ? a * (double)wh[k] : a;
        u.x = (R)((double)u.x + c * (double)d.x);
        u.y = (R)((double)u.y + c * (double)d.y);
      }
      fh[k] = u;
    }
  double s = 0.0;
  for (long long k = k0; k < M; k += stride) {
    typename Cx<R>::T u = r[k];
    const typename Cx<R>::T d = v[k];
    if constexpr (SP) {
      u.x = fmaf(-ar, d.x, u.x);
      u.y = fmaf(-ar, d.y, u.y);
    } else {
      u.x = (R)((double)u.x - a * (double)d.x);
      u.y = (R)((double)u.y - a * (double)d.y);
    }
    r[k] = u;
    const double q = (double)u.x * (double)u.x + (double)u.y * (double)u.y;
    s += w ? (double)w[k] * q : q;
  }
  reduce_and_finish(s, part, ticket, scal, op);
}

// FP64 residual refresh helpers: r = y - A f (A f in FP64), cast to plan precision
__global__ void k_f32_to_f64(const float2 *__restrict__ a, double2 *__restrict__ b, long long n)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    b[k] = make_double2((double)a[k].x, (double)a[k].y);
}
__global__ void k_x_to_f64(const float *__restrict__ a, double *__restrict__ b, long long n)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    b[k] = (double)a[k];
}
__global__ void k_residual_f64(const float2 *__restrict__ y, const double2 *__restrict__ af,
                               float2 *__restrict__ r, long long n)
{
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    r[k] = make_float2((float)((double)y[k].x - af[k].x), (float)((double)y[k].y - af[k].y));
}

// ---------------------------------------------------------------- state
template <typename R>
struct SolverState {
  typedef typename Cx<R>::T C;
  typename SApi<R>::plan *plan = nullptr;
  cudaStream_t s = nullptr;
  long long M = 0, N = 0;
  unsigned flags = 0;
  C *y = nullptr, *r = nullptr, *fh = nullptr, *p = nullptr, *z = nullptr, *v = nullptr;
  R *w = nullptr, *wh = nullptr;
  C *mv_f = nullptr, *mv_fh = nullptr;  // the plan's device f / f_hat
  double *scal = nullptr, *part = nullptr;
  unsigned *ticket = nullptr;  // blocks done in the current reduction (zero between launches)
  double *scal_host = nullptr;
  int sync_level = 2;
  // FP64 residual refresh (single-precision solvers)
  int refresh_every = 0;
  long long iter = 0;
  nfft_plan *plan64 = nullptr;
  cudaEvent_t refresh_ev = nullptr;  // orders the refresh's FP64 stream against the solver's
  double *hist = nullptr;  // dot_r of each step of a multi-step call
  int hist_cap = 0;
  // CUDA graph of one step's launches (steepest descent, CGNR, CGNE)
  bool use_graph = true;
  cudaGraphExec_t gexec = nullptr;
  unsigned long long gen = 0;  // the plan's node set-up it was captured against
};

static std::mutex g_solver_mu;
static std::map<const void *, void *> g_solver_state;

template <typename R>
static SolverState<R> *state_of(const typename SApi<R>::splan *ths)
{
  std::lock_guard<std::mutex> lk(g_solver_mu);
  auto it = g_solver_state.find(ths);
  return it == g_solver_state.end() ? nullptr : reinterpret_cast<SolverState<R> *>(it->second);
}

static unsigned grid_for(long long n)
{
  long long b = (n + 255) / 256;
  if (b > 4 * 152) b = 4 * 152;
  if (b < 1) b = 1;
  return (unsigned)b;
}

template <typename R>
static void dot_into(SolverState<R> *st, const typename Cx<R>::T *x, const R *w, long long n, int op)
{
  k_dot<R><<<RED_BLOCKS, RED_THREADS, 0, st->s>>>(x, w, n, st->part, st->ticket, st->scal, op);
  GB_LAUNCHED("dot");
}

// fh += alpha wh .* p (p == nullptr: no update), r -= alpha v, then the
// reduction of w |r|^2 into op
template <typename R>
static void upd_dot(SolverState<R> *st, typename Cx<R>::T *fh, const typename Cx<R>::T *p, const R *wh,
                    typename Cx<R>::T *r, const typename Cx<R>::T *v, const R *w, int op)
{
  k_upd_dot<R><<<RED_BLOCKS, RED_THREADS, 0, st->s>>>(fh, p, wh, st->N, r, v, w, st->M, st->part, st->ticket,
                                                      st->scal, op);
  GB_LAUNCHED("upd_dot");
}

template <typename R>
static void wcopy(SolverState<R> *st, typename Cx<R>::T *dst, const typename Cx<R>::T *src, const R *w,
                  long long n)
{
  k_scale_copy<R><<<grid_for(n), 256, 0, st->s>>>(dst, src, w, n);
  GB_LAUNCHED("scale_copy");
}

template <typename R>
static void upd(SolverState<R> *st, typename Cx<R>::T *x, const typename Cx<R>::T *y, const R *w,
                long long n, int idx, double sign)
{
  k_upd<R><<<grid_for(n), 256, 0, st->s>>>(x, y, w, n, st->scal, idx, sign);
  GB_LAUNCHED("upd");
}

template <typename R>
static void axpy(SolverState<R> *st, typename Cx<R>::T *x, const typename Cx<R>::T *y, long long n, int idx)
{
  k_axpy<R><<<grid_for(n), 256, 0, st->s>>>(x, y, n, st->scal, idx);
  GB_LAUNCHED("axpy");
}

template <typename R>
static void dcopy(SolverState<R> *st, void *dst, const void *src, size_t bytes, cudaMemcpyKind k)
{
  if (bytes) GB_CUDA(cudaMemcpyAsync(dst, src, bytes, k, st->s));
}

template <typename R>
static void refresh_residual(SolverState<R> *st);

template <>
void refresh_residual<double>(SolverState<double> *st)
{
  (void)st;  // a double solver already computes its residual in FP64
}

template <>
void refresh_residual<float>(SolverState<float> *st)
{
  // r = y - A f_hat_iter with an FP64 plan over the same nodes
  nfft_plan *q = st->plan64;
  double2 *qfh = (double2 *)nfft_gb_device_f_hat(q);
  double2 *qf = (double2 *)nfft_gb_device_f(q);
  cudaStream_t qs = (cudaStream_t)nfft_gb_get_stream(q);
  if (!st->refresh_ev) GB_CUDA(cudaEventCreateWithFlags(&st->refresh_ev, cudaEventDisableTiming));
  cudaEvent_t e = st->refresh_ev;
  GB_CUDA(cudaEventRecord(e, st->s));
  GB_CUDA(cudaStreamWaitEvent(qs, e, 0));
  k_f32_to_f64<<<grid_for(st->N), 256, 0, qs>>>(st->fh, qfh, st->N);
  GB_LAUNCHED("f32_to_f64");
  nfft_gb_trafo_device(q);
  k_residual_f64<<<grid_for(st->M), 256, 0, qs>>>(st->y, qf, st->r, st->M);
  GB_LAUNCHED("residual_f64");
  GB_CUDA(cudaEventRecord(e, qs));
  GB_CUDA(cudaStreamWaitEvent(st->s, e, 0));
}

template <typename R>
static void publish(typename SApi<R>::splan *ths, SolverState<R> *st, bool all_vectors)
{
  typedef typename Cx<R>::T C;
  dcopy<R>(st, st->scal_host, st->scal, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost);
  if (st->sync_level >= 1 || all_vectors) {
    dcopy<R>(st, ths->f_hat_iter, st->fh, st->N * sizeof(C), cudaMemcpyDeviceToHost);
    dcopy<R>(st, ths->r_iter, st->r, st->M * sizeof(C), cudaMemcpyDeviceToHost);
  }
  if (st->sync_level >= 2 || all_vectors) {
    dcopy<R>(st, ths->p_hat_iter, st->p, st->N * sizeof(C), cudaMemcpyDeviceToHost);
    if (ths->z_hat_iter != ths->p_hat_iter)
      dcopy<R>(st, ths->z_hat_iter, st->z, st->N * sizeof(C), cudaMemcpyDeviceToHost);
    if (ths->v_iter) dcopy<R>(st, ths->v_iter, st->v, st->M * sizeof(C), cudaMemcpyDeviceToHost);
  }
  GB_CUDA(cudaStreamSynchronize(st->s));
  const double *h = st->scal_host;
  ths->alpha_iter = (R)h[S_ALPHA];
  ths->beta_iter = (R)h[S_BETA];
  ths->dot_r_iter = (R)h[S_DOT_R];
  ths->dot_r_iter_old = (R)h[S_DOT_R_OLD];
  ths->dot_z_hat_iter = (R)h[S_DOT_Z];
  ths->dot_z_hat_iter_old = (R)h[S_DOT_Z_OLD];
  ths->dot_p_hat_iter = (R)h[S_DOT_P];
  ths->dot_v_iter = (R)h[S_DOT_V];
}

// ---------------------------------------------------------------- device path
template <typename R>
static void dev_before_loop(typename SApi<R>::splan *ths, SolverState<R> *st)
{
  typedef typename Cx<R>::T C;
  const long long M = st->M, N = st->N;
  const unsigned fl = st->flags;
  const R *w = (fl & PRECOMPUTE_WEIGHT) ? st->w : nullptr;
  const R *wh = (fl & PRECOMPUTE_DAMP) ? st->wh : nullptr;
  // user inputs: y, f_hat_iter, weights (and alpha for Landweber)
  dcopy<R>(st, st->y, ths->y, M * sizeof(C), cudaMemcpyHostToDevice);
  dcopy<R>(st, st->fh, ths->f_hat_iter, N * sizeof(C), cudaMemcpyHostToDevice);
  if (w) dcopy<R>(st, st->w, ths->w, M * sizeof(R), cudaMemcpyHostToDevice);
  if (wh) dcopy<R>(st, st->wh, ths->w_hat, N * sizeof(R), cudaMemcpyHostToDevice);
  GB_CUDA(cudaMemsetAsync(st->scal, 0, S_COUNT * sizeof(double), st->s));
  {
    double a = (double)ths->alpha_iter;  // Landweber step size is set by the caller
    GB_CUDA(cudaMemcpyAsync(st->scal + S_ALPHA, &a, sizeof(double), cudaMemcpyHostToDevice, st->s));
    GB_CUDA(cudaStreamSynchronize(st->s));
  }
  // r = y - A f_hat_iter (solver.c:83-89)
  wcopy<R>(st, st->mv_fh, st->fh, nullptr, N);
  SApi<R>::trafo_dev(st->plan);
  dcopy<R>(st, st->r, st->mv_f, M * sizeof(C), cudaMemcpyDeviceToDevice);
  axpy<R>(st, st->r, st->y, M, -1);
  if (st->refresh_every > 0) refresh_residual<R>(st);
  if (!(fl & LANDWEBER) || (fl & NORMS_FOR_LANDWEBER)) dot_into<R>(st, st->r, w, M, F_DOT_R);
  // z = A^H W r (solver.c:101-108)
  wcopy<R>(st, st->mv_f, st->r, w, M);
  SApi<R>::adjoint_dev(st->plan);
  dcopy<R>(st, st->z, st->mv_fh, N * sizeof(C), cudaMemcpyDeviceToDevice);
  if (!(fl & LANDWEBER) || (fl & NORMS_FOR_LANDWEBER)) dot_into<R>(st, st->z, wh, N, F_DOT_Z);
  if (fl & CGNE) {
    // dot_p = dot_z
    GB_CUDA(cudaMemcpyAsync(st->scal + S_DOT_P, st->scal + S_DOT_Z, sizeof(double), cudaMemcpyDeviceToDevice, st->s));
  }
  if (fl & CGNR) dcopy<R>(st, st->p, st->z, N * sizeof(C), cudaMemcpyDeviceToDevice);
  st->iter = 0;
  publish<R>(ths, st, true);
}

// One steepest-descent, CGNR or CGNE step (solver.c:181-344) on the
// solver's stream.  The transforms run straight on the solver's device
// vectors (the plan's own buffers only take the weighted copies), and every
// scalar stays on the device, so the sequence has no host dependency and can
// be captured as a graph.
template <typename R>
static void enqueue_step(SolverState<R> *st, bool refresh)
{
  typedef typename Cx<R>::T C;
  const long long M = st->M, N = st->N;
  const unsigned fl = st->flags;
  const R *w = (fl & PRECOMPUTE_WEIGHT) ? st->w : nullptr;
  const R *wh = (fl & PRECOMPUTE_DAMP) ? st->wh : nullptr;
  // out = A (wh .* in)
  auto trafo_w = [&](const C *in, C *out) {
    if (wh) {
      wcopy<R>(st, st->mv_fh, in, wh, N);
      in = st->mv_fh;
    }
    SApi<R>::trafo_ptr(st->plan, in, out);
  };
  // out = A^H (w .* in)
  auto adjoint_w = [&](const C *in, C *out) {
    if (w) {
      wcopy<R>(st, st->mv_f, in, w, M);
      in = st->mv_f;
    }
    SApi<R>::adjoint_ptr(st->plan, in, out);
  };
  if (fl & STEEPEST_DESCENT) {
    // solver.c:181-229
    trafo_w(st->z, st->v);
    dot_into<R>(st, st->v, w, M, F_DOT_V_ALPHA);
    if (refresh) {
      upd<R>(st, st->fh, st->z, wh, N, S_ALPHA, 1.0);
      upd<R>(st, st->r, st->v, nullptr, M, S_ALPHA, -1.0);
      refresh_residual<R>(st);
      dot_into<R>(st, st->r, w, M, F_DOT_R);
    } else {
      upd_dot<R>(st, st->fh, st->z, wh, st->r, st->v, w, F_DOT_R);
    }
    adjoint_w(st->r, st->z);
    dot_into<R>(st, st->z, wh, N, F_DOT_Z);
  } else if (fl & CGNR) {
    // solver.c:232-292
    trafo_w(st->p, st->v);
    dot_into<R>(st, st->v, w, M, F_DOT_V_ALPHA);
    if (refresh) {
      upd<R>(st, st->fh, st->p, wh, N, S_ALPHA, 1.0);
      upd<R>(st, st->r, st->v, nullptr, M, S_ALPHA, -1.0);
      refresh_residual<R>(st);
      dot_into<R>(st, st->r, w, M, F_DOT_R);
    } else {
      upd_dot<R>(st, st->fh, st->p, wh, st->r, st->v, w, F_DOT_R);
    }
    adjoint_w(st->r, st->z);
    dot_into<R>(st, st->z, wh, N, F_DOT_Z_BETA);
    axpy<R>(st, st->p, st->z, N, S_BETA);
  } else if (fl & CGNE) {
    // solver.c:295-344
    k_finish<<<1, 32, 0, st->s>>>(st->part, 0, st->scal, F_ALPHA_CGNE);
    GB_LAUNCHED("finish");
    upd<R>(st, st->fh, st->p, wh, N, S_ALPHA, 1.0);
    trafo_w(st->p, st->v);
    if (refresh) {
      upd<R>(st, st->r, st->v, nullptr, M, S_ALPHA, -1.0);
      refresh_residual<R>(st);
      dot_into<R>(st, st->r, w, M, F_DOT_R_BETA);
    } else {
      upd_dot<R>(st, st->fh, nullptr, wh, st->r, st->v, w, F_DOT_R_BETA);
    }
    adjoint_w(st->r, st->mv_fh);
    axpy<R>(st, st->p, st->mv_fh, N, S_BETA);
    dot_into<R>(st, st->p, wh, N, F_DOT_P);
  }
}

template <typename R>
static void dev_step_enqueue(typename SApi<R>::splan *ths, SolverState<R> *st)
{
  typedef typename Cx<R>::T C;
  const long long M = st->M, N = st->N;
  const unsigned fl = st->flags;
  const R *w = (fl & PRECOMPUTE_WEIGHT) ? st->w : nullptr;
  const R *wh = (fl & PRECOMPUTE_DAMP) ? st->wh : nullptr;
  ++st->iter;
  const bool refresh = st->refresh_every > 0 && (st->iter % st->refresh_every) == 0;
  if (fl & LANDWEBER) {
    // solver.c:128-178; the step size comes from the caller every step
    double a = (double)ths->alpha_iter;
    GB_CUDA(cudaMemcpyAsync(st->scal + S_ALPHA, &a, sizeof(double), cudaMemcpyHostToDevice, st->s));
    upd<R>(st, st->fh, st->z, wh, N, S_ALPHA, 1.0);
    wcopy<R>(st, st->mv_fh, st->fh, nullptr, N);
    SApi<R>::trafo_dev(st->plan);
    dcopy<R>(st, st->r, st->mv_f, M * sizeof(C), cudaMemcpyDeviceToDevice);
    axpy<R>(st, st->r, st->y, M, -1);
    if (refresh) refresh_residual<R>(st);
    if (fl & NORMS_FOR_LANDWEBER) dot_into<R>(st, st->r, w, M, F_DOT_R);
    wcopy<R>(st, st->mv_f, st->r, w, M);
    SApi<R>::adjoint_dev(st->plan);
    dcopy<R>(st, st->z, st->mv_fh, N * sizeof(C), cudaMemcpyDeviceToDevice);
    if (fl & NORMS_FOR_LANDWEBER) dot_into<R>(st, st->z, wh, N, F_DOT_Z);
  } else if (st->use_graph && !refresh) {
    const unsigned long long gen = SApi<R>::gen(st->plan);
    if (!st->gexec || st->gen != gen) {
      if (st->gexec) {
        GB_CUDA(cudaGraphExecDestroy(st->gexec));
        st->gexec = nullptr;
      }
      cudaGraph_t gph = nullptr;
      GB_CUDA(cudaStreamBeginCapture(st->s, cudaStreamCaptureModeRelaxed));
      enqueue_step<R>(st, false);
      GB_CUDA(cudaStreamEndCapture(st->s, &gph));
      GB_CUDA(cudaGraphInstantiate(&st->gexec, gph, 0));
      GB_CUDA(cudaGraphDestroy(gph));
      st->gen = gen;
    }
    GB_CUDA(cudaGraphLaunch(st->gexec, st->s));
  } else {
    enqueue_step<R>(st, refresh);
  }
}

template <typename R>
static void dev_step(typename SApi<R>::splan *ths, SolverState<R> *st)
{
  dev_step_enqueue<R>(ths, st);
  publish<R>(ths, st, false);
}

// k steps enqueued back to back (no host round trip between them), then one
// publish; dot_r of every step lands in dot_r_hist (host, k values) when
// given.  Landweber takes its step size from the host struct, which does not
// change in between.
template <typename R>
static int dev_steps(typename SApi<R>::splan *ths, SolverState<R> *st, int k, double *dot_r_hist)
{
  if (k <= 0) return 0;
  if (dot_r_hist && st->hist_cap < k) {
    if (st->hist) GB_CUDA(cudaFree(st->hist));
    GB_CUDA(cudaMalloc(&st->hist, (size_t)k * sizeof(double)));
    st->hist_cap = k;
  }
  for (int i = 0; i < k; ++i) {
    dev_step_enqueue<R>(ths, st);
    if (dot_r_hist)
      GB_CUDA(cudaMemcpyAsync(st->hist + i, st->scal + S_DOT_R, sizeof(double), cudaMemcpyDeviceToDevice, st->s));
  }
  if (dot_r_hist)
    GB_CUDA(cudaMemcpyAsync(dot_r_hist, st->hist, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, st->s));
  publish<R>(ths, st, false);
  return 0;
}

// ---------------------------------------------------------------- host path
// The same iteration for an arbitrary mv plan, through its function
// pointers and with the reference's vector swaps.
template <typename R>
struct HostOps {
  static double dot(const R *x, const R *w, long long n)
  {
    double s = 0;
    for (long long k = 0; k < n; ++k) {
      double a = (double)x[2 * k] * x[2 * k] + (double)x[2 * k + 1] * x[2 * k + 1];
      s += w ? w[k] * a : a;
    }
    return s;
  }
  static void wcp(R *x, const R *w, const R *y, long long n)
  {
    for (long long k = 0; k < n; ++k) {
      R c = w ? w[k] : (R)1;
      x[2 * k] = c * y[2 * k];
      x[2 * k + 1] = c * y[2 * k + 1];
    }
  }
  static void upd(R *x, double a, const R *w, const R *y, long long n)
  {
    for (long long k = 0; k < n; ++k) {
      double c = w ? a * w[k] : a;
      x[2 * k] = (R)(x[2 * k] + c * y[2 * k]);
      x[2 * k + 1] = (R)(x[2 * k + 1] + c * y[2 * k + 1]);
    }
  }
  static void axpy(R *x, double a, const R *y, long long n)
  {
    for (long long k = 0; k < 2 * n; ++k) x[k] = (R)(a * x[k] + y[k]);
  }
};

template <typename R>
static void host_before_loop(typename SApi<R>::splan *ths)
{
  typedef HostOps<R> H;
  typedef typename SApi<R>::mvplan MV;
  MV *mv = ths->mv;
  const long long M = mv->M_total, N = mv->N_total;
  const unsigned fl = ths->flags;
  const R *w = (fl & PRECOMPUTE_WEIGHT) ? ths->w : nullptr;
  const R *wh = (fl & PRECOMPUTE_DAMP) ? ths->w_hat : nullptr;
  if (!mv || !mv->mv_trafo || !mv->mv_adjoint) fatal("solver: mv plan without mv_trafo / mv_adjoint");
  H::wcp((R *)mv->f_hat, nullptr, (R *)ths->f_hat_iter, N);
  std::swap(ths->r_iter, mv->f);
  mv->mv_trafo(mv);
  std::swap(ths->r_iter, mv->f);
  H::axpy((R *)ths->r_iter, -1.0, (R *)ths->y, M);
  if (!(fl & LANDWEBER) || (fl & NORMS_FOR_LANDWEBER)) ths->dot_r_iter = (R)H::dot((R *)ths->r_iter, w, M);
  H::wcp((R *)mv->f, w, (R *)ths->r_iter, M);
  std::swap(ths->z_hat_iter, mv->f_hat);
  mv->mv_adjoint(mv);
  std::swap(ths->z_hat_iter, mv->f_hat);
  if (!(fl & LANDWEBER) || (fl & NORMS_FOR_LANDWEBER))
    ths->dot_z_hat_iter = (R)H::dot((R *)ths->z_hat_iter, wh, N);
  if (fl & CGNE) ths->dot_p_hat_iter = ths->dot_z_hat_iter;
  if (fl & CGNR) H::wcp((R *)ths->p_hat_iter, nullptr, (R *)ths->z_hat_iter, N);
}

template <typename R>
static void host_step(typename SApi<R>::splan *ths)
{
  typedef HostOps<R> H;
  typedef typename SApi<R>::mvplan MV;
  MV *mv = ths->mv;
  const long long M = mv->M_total, N = mv->N_total;
  const unsigned fl = ths->flags;
  const R *w = (fl & PRECOMPUTE_WEIGHT) ? ths->w : nullptr;
  const R *wh = (fl & PRECOMPUTE_DAMP) ? ths->w_hat : nullptr;
  R *fh = (R *)ths->f_hat_iter, *r = (R *)ths->r_iter;
  if (fl & LANDWEBER) {
    H::upd(fh, ths->alpha_iter, wh, (R *)ths->z_hat_iter, N);
    H::wcp((R *)mv->f_hat, nullptr, fh, N);
    std::swap(ths->r_iter, mv->f);
    mv->mv_trafo(mv);
    std::swap(ths->r_iter, mv->f);
    H::axpy((R *)ths->r_iter, -1.0, (R *)ths->y, M);
    if (fl & NORMS_FOR_LANDWEBER) ths->dot_r_iter = (R)H::dot((R *)ths->r_iter, w, M);
    H::wcp((R *)mv->f, w, (R *)ths->r_iter, M);
    std::swap(ths->z_hat_iter, mv->f_hat);
    mv->mv_adjoint(mv);
    std::swap(ths->z_hat_iter, mv->f_hat);
    if (fl & NORMS_FOR_LANDWEBER) ths->dot_z_hat_iter = (R)H::dot((R *)ths->z_hat_iter, wh, N);
  } else if (fl & (STEEPEST_DESCENT | CGNR)) {
    const bool cg = (fl & CGNR) != 0;
    R *dir = cg ? (R *)ths->p_hat_iter : (R *)ths->z_hat_iter;
    H::wcp((R *)mv->f_hat, wh, dir, N);
    std::swap(ths->v_iter, mv->f);
    mv->mv_trafo(mv);
    std::swap(ths->v_iter, mv->f);
    ths->dot_v_iter = (R)H::dot((R *)ths->v_iter, w, M);
    ths->alpha_iter = ths->dot_z_hat_iter / ths->dot_v_iter;
    H::upd(fh, ths->alpha_iter, wh, dir, N);
    H::upd(r, -ths->alpha_iter, nullptr, (R *)ths->v_iter, M);
    ths->dot_r_iter = (R)H::dot(r, w, M);
    H::wcp((R *)mv->f, w, r, M);
    std::swap(ths->z_hat_iter, mv->f_hat);
    mv->mv_adjoint(mv);
    std::swap(ths->z_hat_iter, mv->f_hat);
    ths->dot_z_hat_iter_old = ths->dot_z_hat_iter;
    ths->dot_z_hat_iter = (R)H::dot((R *)ths->z_hat_iter, wh, N);
    if (cg) {
      ths->beta_iter = ths->dot_z_hat_iter / ths->dot_z_hat_iter_old;
      H::axpy((R *)ths->p_hat_iter, ths->beta_iter, (R *)ths->z_hat_iter, N);
    }
  } else if (fl & CGNE) {
    ths->alpha_iter = ths->dot_r_iter / ths->dot_p_hat_iter;
    H::upd(fh, ths->alpha_iter, wh, (R *)ths->p_hat_iter, N);
    H::wcp((R *)mv->f_hat, wh, (R *)ths->p_hat_iter, N);
    mv->mv_trafo(mv);
    H::upd(r, -ths->alpha_iter, nullptr, (R *)mv->f, M);
    ths->dot_r_iter_old = ths->dot_r_iter;
    ths->dot_r_iter = (R)H::dot(r, w, M);
    ths->beta_iter = ths->dot_r_iter / ths->dot_r_iter_old;
    H::wcp((R *)mv->f, w, r, M);
    mv->mv_adjoint(mv);
    H::axpy((R *)ths->p_hat_iter, ths->beta_iter, (R *)mv->f_hat, N);
    ths->dot_p_hat_iter = (R)H::dot((R *)ths->p_hat_iter, wh, N);
  }
}

// ---------------------------------------------------------------- API
template <typename R>
static void init_advanced(typename SApi<R>::splan *ths, typename SApi<R>::mvplan *mv, unsigned flags)
{
  typedef typename Cx<R>::T C;
  memset(ths, 0, sizeof(*ths));
  ths->mv = mv;
  ths->flags = flags;
  const size_t M = (size_t)mv->M_total, N = (size_t)mv->N_total;
  // solver.c:40-74
  ths->y = (decltype(ths->y))SApi<R>::mal(M * sizeof(C));
  ths->r_iter = (decltype(ths->r_iter))SApi<R>::mal(M * sizeof(C));
  ths->f_hat_iter = (decltype(ths->f_hat_iter))SApi<R>::mal(N * sizeof(C));
  ths->p_hat_iter = (decltype(ths->p_hat_iter))SApi<R>::mal(N * sizeof(C));
  if (flags & LANDWEBER) ths->z_hat_iter = ths->p_hat_iter;
  if (flags & STEEPEST_DESCENT) {
    ths->z_hat_iter = ths->p_hat_iter;
    ths->v_iter = (decltype(ths->v_iter))SApi<R>::mal(M * sizeof(C));
  }
  if (flags & CGNR) {
    ths->z_hat_iter = (decltype(ths->z_hat_iter))SApi<R>::mal(N * sizeof(C));
    ths->v_iter = (decltype(ths->v_iter))SApi<R>::mal(M * sizeof(C));
  }
  if (flags & CGNE) ths->z_hat_iter = ths->p_hat_iter;
  if (flags & PRECOMPUTE_WEIGHT) ths->w = (R *)SApi<R>::mal(M * sizeof(R));
  if (flags & PRECOMPUTE_DAMP) ths->w_hat = (R *)SApi<R>::mal(N * sizeof(R));

  if (!SApi<R>::ours(mv)) return;  // host iteration over a foreign operator
  SolverState<R> *st = new SolverState<R>();
  st->plan = reinterpret_cast<typename SApi<R>::plan *>(mv);
  st->s = (cudaStream_t)SApi<R>::stream(st->plan);
  st->M = (long long)M;
  st->N = (long long)N;
  st->flags = flags;
  const size_t Mz = M ? M : 1, Nz = N ? N : 1;
  GB_CUDA(cudaMalloc(&st->y, Mz * sizeof(C)));
  GB_CUDA(cudaMalloc(&st->r, Mz * sizeof(C)));
  GB_CUDA(cudaMalloc(&st->v, Mz * sizeof(C)));
  GB_CUDA(cudaMalloc(&st->fh, Nz * sizeof(C)));
  GB_CUDA(cudaMalloc(&st->p, Nz * sizeof(C)));
  if (flags & (LANDWEBER | STEEPEST_DESCENT | CGNE)) st->z = st->p;
  else GB_CUDA(cudaMalloc(&st->z, Nz * sizeof(C)));
  GB_CUDA(cudaMalloc(&st->w, Mz * sizeof(R)));
  GB_CUDA(cudaMalloc(&st->wh, Nz * sizeof(R)));
  GB_CUDA(cudaMalloc(&st->scal, S_COUNT * sizeof(double)));
  GB_CUDA(cudaMalloc(&st->part, RED_BLOCKS * sizeof(double)));
  GB_CUDA(cudaMalloc(&st->ticket, sizeof(unsigned)));
  GB_CUDA(cudaMemset(st->ticket, 0, sizeof(unsigned)));
  GB_CUDA(cudaMallocHost(&st->scal_host, S_COUNT * sizeof(double)));
  st->mv_f = (C *)SApi<R>::dev_f(st->plan);
  st->mv_fh = (C *)SApi<R>::dev_fhat(st->plan);
  std::lock_guard<std::mutex> lk(g_solver_mu);
  g_solver_state[ths] = st;
}

template <typename R>
static void finalize_solver(typename SApi<R>::splan *ths)
{
  SolverState<R> *st = state_of<R>(ths);
  if (st) {
    cudaStreamSynchronize(st->s);
    if (st->gexec) cudaGraphExecDestroy(st->gexec);
    if (st->refresh_ev) cudaEventDestroy(st->refresh_ev);
    if (st->hist) cudaFree(st->hist);
    cudaFree(st->y);
    cudaFree(st->r);
    cudaFree(st->v);
    cudaFree(st->fh);
    if (st->z != st->p) cudaFree(st->z);
    cudaFree(st->p);
    cudaFree(st->w);
    cudaFree(st->wh);
    cudaFree(st->scal);
    cudaFree(st->part);
    cudaFree(st->ticket);
    cudaFreeHost(st->scal_host);
    if (st->plan64) {
      nfft_finalize(st->plan64);
      delete st->plan64;
    }
    delete st;
    std::lock_guard<std::mutex> lk(g_solver_mu);
    g_solver_state.erase(ths);
  }
  // solver.c:363-385
  const unsigned fl = ths->flags;
  if (fl & PRECOMPUTE_WEIGHT) SApi<R>::fre(ths->w);
  if (fl & PRECOMPUTE_DAMP) SApi<R>::fre(ths->w_hat);
  if (fl & CGNR) {
    SApi<R>::fre(ths->v_iter);
    SApi<R>::fre(ths->z_hat_iter);
  }
  if (fl & STEEPEST_DESCENT) SApi<R>::fre(ths->v_iter);
  SApi<R>::fre(ths->p_hat_iter);
  SApi<R>::fre(ths->f_hat_iter);
  SApi<R>::fre(ths->r_iter);
  SApi<R>::fre(ths->y);
}

template <typename R>
static void before_loop(typename SApi<R>::splan *ths)
{
  SolverState<R> *st = state_of<R>(ths);
  if (st) dev_before_loop<R>(ths, st);
  else host_before_loop<R>(ths);
}

template <typename R>
static void loop_one_step(typename SApi<R>::splan *ths)
{
  SolverState<R> *st = state_of<R>(ths);
  if (st) dev_step<R>(ths, st);
  else host_step<R>(ths);
}

}  // namespace gb

using namespace gb;

extern "C" {

#define GB_SOLVER_API(X, R)                                                                     \
  void X##init_advanced_complex(X##plan_complex *ths, SApi<R>::mvplan *mv, unsigned flags)      \
  {                                                                                             \
    init_advanced<R>(ths, mv, flags);                                                           \
  }                                                                                             \
  void X##init_complex(X##plan_complex *ths, SApi<R>::mvplan *mv)                               \
  {                                                                                             \
    init_advanced<R>(ths, mv, CGNR);                                                            \
  }                                                                                             \
  void X##before_loop_complex(X##plan_complex *ths) { before_loop<R>(ths); }                    \
  void X##loop_one_step_complex(X##plan_complex *ths) { loop_one_step<R>(ths); }                \
  void X##finalize_complex(X##plan_complex *ths) { finalize_solver<R>(ths); }                   \
  int X##gb_set_sync(X##plan_complex *ths, int level)                                           \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    if (!st) return -1;                                                                         \
    st->sync_level = level;                                                                     \
    return 0;                                                                                   \
  }                                                                                             \
  int X##gb_sync(X##plan_complex *ths)                                                          \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    if (!st) return -1;                                                                         \
    publish<R>(ths, st, true);                                                                  \
    return 0;                                                                                   \
  }                                                                                             \
  void *X##gb_device_f_hat_iter(X##plan_complex *ths)                                           \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    return st ? (void *)st->fh : nullptr;                                                       \
  }                                                                                             \
  void *X##gb_device_y(X##plan_complex *ths)                                                    \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    return st ? (void *)st->y : nullptr;                                                        \
  }                                                                                             \
  int X##gb_loop_steps(X##plan_complex *ths, int k, double *dot_r_hist)                          \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    if (!st) return -1;                                                                         \
    return dev_steps<R>(ths, st, k, dot_r_hist);                                                \
  }                                                                                             \
  int X##gb_set_graphs(X##plan_complex *ths, int on)                                            \
  {                                                                                             \
    SolverState<R> *st = state_of<R>(ths);                                                      \
    if (!st) return -1;                                                                         \
    st->use_graph = on != 0;                                                                    \
    return 0;                                                                                   \
  }

GB_SOLVER_API(solver_, double)
GB_SOLVER_API(solverf_, float)

// FP64 residual refresh every `every` iterations for a single-precision
// solver over an nfftf plan: r = y - A f_hat_iter is recomputed by an FP64
// plan over the same nodes (created here), then cast back to FP32.
int solverf_gb_set_refresh(solverf_plan_complex *ths, int every)
{
  SolverState<float> *st = state_of<float>(ths);
  if (!st) return -1;
  st->refresh_every = every;
  if (every > 0 && !st->plan64) {
    nfftf_plan *pf = st->plan;
    int d = (int)pf->d, N[GB_MAXD], n[GB_MAXD];
    for (int t = 0; t < d; ++t) {
      N[t] = (int)pf->N[t];
      n[t] = (int)pf->n[t];
    }
    nfft_plan *q = new nfft_plan();
    nfft_init_guru(q, d, N, (int)pf->M_total, n, (int)pf->m, PRE_PHI_HUT | PRE_PSI | FFTW_INIT,
                   FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
    // the FP64 plan reads the same nodes, widened on the device
    double *qx = (double *)nfft_gb_device_x(q);
    const float *fx = (const float *)nfftf_gb_device_x(pf);
    const long long nx = (long long)pf->M_total * d;
    cudaStream_t qs = (cudaStream_t)nfft_gb_get_stream(q);
    GB_CUDA(cudaStreamSynchronize(st->s));
    k_x_to_f64<<<grid_for(nx), 256, 0, qs>>>(fx, qx, nx);
    GB_LAUNCHED("x_to_f64");
    nfft_gb_precompute_device(q);
    GB_CUDA(cudaStreamSynchronize(qs));
    st->plan64 = q;
  }
  return 0;
}

int solver_gb_set_refresh(solver_plan_complex *ths, int every)
{
  SolverState<double> *st = state_of<double>(ths);
  if (!st) return -1;
  st->refresh_every = 0;  // already FP64
  (void)every;
  return 0;
}

}  // extern "C"
