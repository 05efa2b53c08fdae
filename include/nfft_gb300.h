/*
 * nfft_gb300.h -- GB300-specific extensions of the NFFT C API.
 *
 * These entry points have no counterpart in the reference NFFT; they expose
 * what a GPU caller needs beyond the host-array semantics of nfft3.h:
 * device-resident operands (inputs already in HBM), the CUDA stream a plan
 * runs on, per-stage timings, and the library's error state.  All take plain
 * pointers and sizes; CUDA handles are passed as void*.
 *
 * Each function exists for both precisions: nfft_gb_* (double plans) and
 * nfftf_gb_* (float plans).
 */
#ifndef NFFT_GB300_H
#define NFFT_GB300_H

#include "nfft3.h"

#ifdef __cplusplus
extern "C" {
#endif

#define NFFTGB_DEFINE_API(X) \
/* Run the plan on this cudaStream_t (NULL = the plan's own stream). */ \
int X(gb_set_stream)(X(plan) *ths, void *cuda_stream); \
void *X(gb_get_stream)(X(plan) *ths); \
/* Compensated adjoint of single-precision 2-D plans on the column kernels \
 * (no counterpart in the reference, whose double build needs none): the \
 * shared-memory subgrid keeps a second plane of rounding errors (error-free \
 * sums), the write-back adds them into the grid by error-free compare-and-swap \
 * with the remaining errors folded in before the FFT.  It roughly doubles \
 * the adjoint's B^T time and lowers the error only where very many nodes \
 * share cells.  mode 1 on, 0 or -1 off (the default).  Returns 0, or -1 \
 * (nothing changed) for a plan without such a kernel (double precision, \
 * d != 2, NDFT). */ \
int X(gb_set_compensated)(X(plan) *ths, int mode); \
/* Kernel of B (trafo) for single-precision 3-D plans with m = 4: mode 0 \
 * (the default) or 1 column segments, 2 sub-cell units (the column form is \
 * as fast or faster at every node density measured).  Both give the same \
 * result to rounding.  Returns 0, or -1 (nothing changed) for a plan without \
 * these kernels. */ \
int X(gb_set_b3_kernel)(X(plan) *ths, int mode); \
/* The B kernel such a plan runs now: 1 column segments, 2 sub-cell units; \
 * -1 for other plans. */ \
int X(gb_b3_kernel)(X(plan) *ths); \
/* Device buffers of the plan: f_hat (N_total complex), f (M_total complex), \
 * in the caller's natural orders, and x (M_total*d reals, node-major). */ \
void *X(gb_device_f_hat)(X(plan) *ths); \
void *X(gb_device_f)(X(plan) *ths); \
void *X(gb_device_x)(X(plan) *ths); \
/* Node set-up from a device copy of x (already in gb_device_x). */ \
void X(gb_precompute_device)(X(plan) *ths); \
/* Transforms on the device buffers, enqueued on the plan's stream; they do \
 * not synchronise and do not touch the host arrays. */ \
void X(gb_trafo_device)(X(plan) *ths); \
void X(gb_adjoint_device)(X(plan) *ths); \
/* The same on caller-owned device vectors: f_hat_dev (N_total complex) and \
 * f_dev (M_total complex) in the caller's natural orders. */ \
void X(gb_trafo_ptr)(X(plan) *ths, const void *f_hat_dev, void *f_dev); \
void X(gb_adjoint_ptr)(X(plan) *ths, const void *f_dev, void *f_hat_dev); \
/* Milliseconds of the last host-API transform per stage: \
 * [0] D or D^T, [1] FFT, [2] B or B^T kernel, [3] the rest (copies, the \
 * grid memset of B^T). */ \
void X(gb_stage_times)(X(plan) *ths, float *ms4); \
/* The same for the last device transform (waits for it to finish). */ \
void X(gb_device_stage_times)(X(plan) *ths, float *ms4); \
/* Kernel launches of the last transform (library kernels, not cuFFT). */ \
int X(gb_last_launch_count)(X(plan) *ths); \
/* Counter of node set-ups (precompute) of the plan: work captured against \
 * its node order (a CUDA graph) is stale once this changes. */ \
unsigned long long X(gb_generation)(X(plan) *ths); \
/* Time up to max_calls following device transforms with CUDA events on the \
 * plan's stream, without synchronising between them.  timing_end waits for \
 * them and returns the number of calls timed; sums7 (ms) = trafo D, trafo \
 * FFT, trafo B, adjoint grid memset, adjoint B^T, adjoint FFT, adjoint D^T; \
 * counts2 = trafo calls, adjoint calls. */ \
int X(gb_timing_begin)(X(plan) *ths, int max_calls); \
int X(gb_timing_end)(X(plan) *ths, float *sums7, int *counts2);

NFFTGB_DEFINE_API(NFFT_MANGLE_DOUBLE)
NFFTGB_DEFINE_API(NFFT_MANGLE_FLOAT)

/* Solver extensions (solver_gb_* for double, solverf_gb_* for float).  They
 * apply when the solver's mv plan is an nfft plan of this library, whose
 * iteration then runs in HBM; they return -1 for any other mv plan. */
#define NFFTGB_DEFINE_SOLVER_API(X) \
/* Which vectors each before_loop / loop_one_step call copies back to the \
 * host struct: 2 = all (default, the reference's visible state), \
 * 1 = f_hat_iter and r_iter, 0 = scalars only. */ \
int X(gb_set_sync)(X(plan_complex) *ths, int level); \
/* Copy every iterate vector back to the host struct now. */ \
int X(gb_sync)(X(plan_complex) *ths); \
/* Recompute r = y - A f_hat_iter with an FP64 transform every `every` \
 * iterations (single-precision solvers; 0 = off). */ \
int X(gb_set_refresh)(X(plan_complex) *ths, int every); \
/* Device copies of f_hat_iter (N_total complex) and y (M_total complex). */ \
void *X(gb_device_f_hat_iter)(X(plan_complex) *ths); \
void *X(gb_device_y)(X(plan_complex) *ths); \
/* 1 (default): steepest descent, CGNR and CGNE steps replay a CUDA graph of \
 * the step's launches, captured on first use and again after the plan's \
 * nodes change; 0: launch them one by one.  The results are the same. */ \
int X(gb_set_graphs)(X(plan_complex) *ths, int on); \
/* k calls of loop_one_step without a host round trip in between: the steps \
 * are enqueued back to back and the host struct is updated once at the end \
 * (as after the k-th call); dot_r_hist (host, k doubles, or NULL) receives \
 * dot_r_iter after each step. */ \
int X(gb_loop_steps)(X(plan_complex) *ths, int k, double *dot_r_hist);

NFFTGB_DEFINE_SOLVER_API(SOLVER_MANGLE_DOUBLE)
NFFTGB_DEFINE_SOLVER_API(SOLVER_MANGLE_FLOAT)

/* Last error message recorded by the library (empty string if none).  Fatal
 * errors also go through nfft_die / nfft_die_hook like the reference. */
const char *nfft_gb_last_error(void);
void nfft_gb_clear_error(void);

/* 1 when the library was built for and runs on an sm_103 device. */
int nfft_gb_device_ok(void);

/* Batched transforms of many independent 2-D single-precision plans (no
 * counterpart in the reference, which transforms one plan per call).  Plans
 * need m = 4 or 6 and their nodes set up; each plan keeps its own result:
 * trafo reads the plan's device f_hat (nfftf_gb_device_f_hat) and writes its
 * device f, adjoint reads the device f and writes the device f_hat.
 *  - create / destroy a batch over `count` plans (the plans must outlive it);
 *  - autotune: per class of plans (m, oversampling, node density) choose the
 *    tile edge (8, 16, 32) and threads per node (1, 4, 16), or the 2-D column
 *    kernels on 32^2 tiles (reported as T = 32, threads per node 0), by
 *    timing; the choice is remembered for the process;
 *  - run: what = 1 trafo, 2 adjoint, 3 both; mode 0 = stream launches, 1 = a
 *    CUDA graph of trafo + adjoint captured on first use (what must be 3);
 *    returns after the GPU has finished;
 *  - time: milliseconds per trafo + adjoint round over `reps` rounds. */
void *nfftf_gb_batch_create(nfftf_plan **plans, int count);
void nfftf_gb_batch_destroy(void *batch);
int nfftf_gb_batch_autotune(void *batch, int reps);
int nfftf_gb_batch_run(void *batch, int what, int mode);
float nfftf_gb_batch_time(void *batch, int reps, int mode);
long long nfftf_gb_batch_nodes(void *batch);
int nfftf_gb_batch_items(void *batch);
int nfftf_gb_batch_plan_config(void *batch, int k, int *T, int *tpn);
/* Set plan k's configuration by hand (T in {8, 16, 32} with threads per node
 * in {1, 4, 16}, or T = 32 with 0 for the column kernels); re-bins the plan's
 * nodes and rebuilds the batch tables.  Returns -1 for other values or a plan
 * the column kernels cannot take. */
int nfftf_gb_batch_set_config(void *batch, int k, int T, int tpn);

/* Density-compensation weights for the inverse NFFT (no counterpart in the
 * reference, whose solver takes the weights w from the caller):
 *  - nfftf_gb_dcf_fixed_point: w <- w / |A A^H w| `iters` times on the
 *    plan's nodes (w_dev: M_total reals on the device, in and out); from
 *    w = 1 one step gives the density estimate 1 / |A A^H 1|, which makes the
 *    weighted CGNR converge fastest: further steps amplify the negative
 *    sidelobes of the full-box point-spread function A A^H;
 *  - nfft_gb_dcf_features: 8 features per 2-D node (log(1 + neighbour count)
 *    within 1, 2, 4 cells of the n0 x n1 grid, 2|x|, cos/sin of the angle and
 *    of twice the angle), feat_dev = M x 8 floats, written in stream order
 *    (the call does not wait for them);
 *  - an MLP 8 -> 64 -> 64 -> 1 (GELU) on those features: parameter vector of
 *    nfft_gb_mlp_param_count() floats (W1[8][64], b1, W2[64][64], b2, W3, b3),
 *    forward, mean-squared-error gradient (grad and loss overwritten) and an
 *    Adam step; all operands are device pointers. */
int nfftf_gb_dcf_fixed_point(nfftf_plan *ths, float *w_dev, int iters);
int nfft_gb_dcf_features(const float *x_dev, int M, int n0, int n1, float *feat_dev, void *stream);
int nfft_gb_affine_columns(float *a, long long rows, int cols, const float *scale, const float *shift,
                           void *stream);
int nfft_gb_mlp_param_count(void);
int nfft_gb_mlp_forward(const float *params, const float *feat, int M, float *out, void *stream);
int nfft_gb_mlp_grad(const float *params, const float *feat, const float *target, int M, float *grad,
                     float *loss, void *stream);
int nfft_gb_mlp_adam(float *params, const float *grad, float *m1, float *m2, int step, float lr,
                     float beta1, float beta2, float eps, void *stream);

/* The polynomial form of the Kaiser-Bessel window that the single-precision
 * 3-D kernels evaluate on the fly in place of the PRE_PSI table (reference
 * window: include/infft.h:209-222).  For the window with cut-off m and shape
 * b, coef[l * 10 + k] (l < w = 2m + 2, k < 10, host memory) is the k-th
 * power coefficient of tap l as a polynomial in s = 2 frac(n x) - 1: the
 * degree-9 interpolant, in double precision at the ten Chebyshev points of
 * [-1, 1], of phi(n x - (u + l)) with u = floor(n x) - m.  Host only. */
void nfft_gb_kb_poly_fit(int m, double b, int w, float *coef);
/* The double-precision form of the 2-D double-precision kernels: coef[l * 17
 * + k] (k < 17), the degree-16 interpolant at the 17 Chebyshev points,
 * computed in extended precision and rounded to double.  Host only. */
void nfft_gb_kb_polyd_fit(int m, double b, int w, double *coef);

/* Bounded waits of the single-precision 3-D and 2-D transforms that gave up
 * since the last call (no counterpart in the reference).  Their B kernels
 * stage each tile of the oversampled grid with a TMA copy and wait for it at
 * most about a second; a copy that never arrives leaves that tile's samples
 * unwritten and is counted here instead of hanging the GPU.  The 3-D B^T
 * adds its column segments to a tile's subgrid under a lock whose spin is
 * bounded the same way (a segment that gives up is not added, and counted).
 * Reads and clears the count of the current device; 0 in every correct run. */
unsigned long long nfft_gb_tma_wait_timeouts(void);

/* The node sort of NFFT_SORT_NODES without any device allocation (no
 * counterpart in the reference).  For callers that cannot allocate device
 * memory where they sort nodes: their memory belongs to a caching allocator
 * or a fixed budget, or they cannot afford the device synchronisation that
 * cudaMalloc / cudaFree imply.  Writes into index_x_dev (2*M long long, device)
 * the same (key, node) pairs that nfft_precompute_one_psi puts in index_x for
 * nodes x_dev (M*d reals on the device, float if single != 0, else double)
 * and grid lengths n[0..d-1] with cut-off m, enqueued on `stream`.
 * Limits: M <= 262144 (else returns -1 without doing anything; the reason is
 * in nfft_gb_last_error); the n_t must multiply to less than 2^32.  All
 * intermediate buffers live in one static device array of about 4.3 MB that
 * every GPU loading the library keeps until exit; the first call on a device
 * looks up its address there (make that call before any stream capture);
 * calls share the array, so calls that overlap on the GPU race and must be
 * serialised by the caller.  After cudaDeviceReset on a device the cached
 * address is stale: do not call this there again in the same process.
 * Returns 0 on success, -1 on invalid input, -2 if the scratch array cannot
 * be reached on the current device or the CUDA context holds an error after
 * the launches (reason in nfft_gb_last_error); a launch that fails inside
 * goes through nfft_die and its hook, as every launch of this library. */
int nfft_gb_sort_nodes_noalloc(int single, const void *x_dev, int d, const int *n, int m, int M,
                               long long *index_x_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NFFT_GB300_H */
