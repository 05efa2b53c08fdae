/*
 * simple_calls.c -- a plain C caller of the drop-in ABI, compiled against
 * include/ only and linked with libnfft3_gb300.so (test program).
 *
 * It makes the calls the reference's example programs make, in their order:
 *  - examples/nfft/simple_test.c.in: init (init_1d, init_guru with
 *    PRE_FULL_PSI, init_3d in single precision), random nodes and
 *    coefficients from the library's vrand helpers, precompute_one_psi,
 *    check, trafo_direct, trafo, adjoint_direct, adjoint, finalize;
 *  - examples/solver/simple_test.c.in: solver_init_complex over the plan,
 *    a zero initial guess, the plan/solver pointer swap around a trafo of
 *    the iterate, before_loop, loop_one_step, finalize.
 * Every input and output array goes to a raw file in the directory given as
 * argv[1] (little-endian doubles / floats, interleaved complex), so that a
 * test can recompute each result with the oracle.
 *
 * Usage: simple_calls OUTDIR
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nfft3.h"

static const char *g_dir;

static void dump(const char *name, const void *p, size_t bytes)
{
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s.bin", g_dir, name);
  FILE *fh = fopen(path, "wb");
  if (!fh || fwrite(p, 1, bytes, fh) != bytes) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(2);
  }
  fclose(fh);
}

/* the four transforms of one double-precision plan, dumped under `tag` */
static int run_double(nfft_plan *p, const char *tag)
{
  char nm[256];
  const char *err;
  const size_t M = (size_t)p->M_total, N = (size_t)p->N_total;
  fftw_complex *f_direct = (fftw_complex *)nfft_malloc(M * sizeof(fftw_complex));
  fftw_complex *fh_direct = (fftw_complex *)nfft_malloc(N * sizeof(fftw_complex));

  nfft_vrand_shifted_unit_double(p->x, p->d * p->M_total);
  if (p->flags & PRE_ONE_PSI) nfft_precompute_one_psi(p);
  nfft_vrand_unit_complex(p->f_hat, p->N_total);
  err = nfft_check(p);
  if (err) {
    printf("Error in nfft module: %s\n", err);
    return 1;
  }
  snprintf(nm, sizeof nm, "%s_x", tag);
  dump(nm, p->x, M * (size_t)p->d * sizeof(double));
  snprintf(nm, sizeof nm, "%s_fhat", tag);
  dump(nm, p->f_hat, N * sizeof(fftw_complex));

  nfft_trafo_direct(p);
  memcpy(f_direct, p->f, M * sizeof(fftw_complex));
  nfft_trafo(p);
  snprintf(nm, sizeof nm, "%s_f_direct", tag);
  dump(nm, f_direct, M * sizeof(fftw_complex));
  snprintf(nm, sizeof nm, "%s_f", tag);
  dump(nm, p->f, M * sizeof(fftw_complex));
  printf("%s trafo vs ndft: %.3e\n", tag, (double)nfft_error_l_infty_complex(f_direct, p->f, p->M_total));

  /* the adjoints take the trafo's samples as input, as the example does */
  nfft_adjoint_direct(p);
  memcpy(fh_direct, p->f_hat, N * sizeof(fftw_complex));
  nfft_adjoint(p);
  snprintf(nm, sizeof nm, "%s_fhat_direct", tag);
  dump(nm, fh_direct, N * sizeof(fftw_complex));
  snprintf(nm, sizeof nm, "%s_fhat_adj", tag);
  dump(nm, p->f_hat, N * sizeof(fftw_complex));
  printf("%s adjoint vs adjoint ndft: %.3e\n", tag,
         (double)nfft_error_l_infty_complex(fh_direct, p->f_hat, p->N_total));
  nfft_free(f_direct);
  nfft_free(fh_direct);
  return 0;
}

static int test_1d(void)
{
  nfft_plan p;
  nfft_init_1d(&p, 14, 19);
  const int rc = run_double(&p, "d1");
  nfft_finalize(&p);
  return rc;
}

static int test_2d_full_psi(void)
{
  nfft_plan p;
  int N[2] = {32, 14}, n[2] = {64, 32};
  nfft_init_guru(&p, 2, N, N[0] * N[1], n, 7,
                 PRE_PHI_HUT | PRE_FULL_PSI | MALLOC_F_HAT | MALLOC_X | MALLOC_F | FFTW_INIT | FFT_OUT_OF_PLACE,
                 FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
  const int rc = run_double(&p, "d2");
  nfft_finalize(&p);
  return rc;
}

static int test_3d_single(void)
{
  nfftf_plan p;
  const int M = 3000;
  nfftf_init_3d(&p, 16, 16, 16, M);
  nfftf_vrand_shifted_unit_double(p.x, p.d * p.M_total);
  if (p.flags & PRE_ONE_PSI) nfftf_precompute_one_psi(&p);
  nfftf_vrand_unit_complex(p.f_hat, p.N_total);
  if (nfftf_check(&p)) return 1;
  dump("s3_x", p.x, (size_t)M * 3 * sizeof(float));
  dump("s3_fhat", p.f_hat, (size_t)p.N_total * sizeof(fftwf_complex));
  nfftf_trafo(&p);
  dump("s3_f", p.f, (size_t)M * sizeof(fftwf_complex));
  nfftf_adjoint(&p);
  dump("s3_fhat_adj", p.f_hat, (size_t)p.N_total * sizeof(fftwf_complex));
  nfftf_finalize(&p);
  return 0;
}

static int test_solver(void)
{
  nfft_plan p;
  solver_plan_complex ip;
  int N[2] = {32, 32}, n[2] = {64, 64};
  const int M = 1500, iters = 6;
  double res[16];
  nfft_init_guru(&p, 2, N, M, n, 6,
                 PRE_PHI_HUT | PRE_PSI | MALLOC_F_HAT | MALLOC_X | MALLOC_F | FFTW_INIT | FFT_OUT_OF_PLACE
                     | NFFT_SORT_NODES,
                 FFTW_ESTIMATE | FFTW_DESTROY_INPUT);
  nfft_vrand_shifted_unit_double(p.x, p.d * p.M_total);
  if (p.flags & PRE_ONE_PSI) nfft_precompute_one_psi(&p);
  solver_init_complex(&ip, (nfft_mv_plan_complex *)&p);
  nfft_vrand_unit_complex(ip.y, p.M_total);
  for (int k = 0; k < p.N_total; ++k) ip.f_hat_iter[k] = 0.0;
  if (nfft_check(&p)) return 1;
  dump("cg_x", p.x, (size_t)M * 2 * sizeof(double));
  dump("cg_y", ip.y, (size_t)M * sizeof(fftw_complex));

  /* the example's data fit: the plan and the solver swap f_hat pointers */
  fftw_complex *t = ip.f_hat_iter;
  ip.f_hat_iter = p.f_hat;
  p.f_hat = t;
  nfft_trafo(&p);
  t = ip.f_hat_iter;
  ip.f_hat_iter = p.f_hat;
  p.f_hat = t;

  solver_before_loop_complex(&ip);
  res[0] = ip.dot_r_iter;
  for (int l = 0; l < iters; ++l) {
    solver_loop_one_step_complex(&ip);
    res[l + 1] = ip.dot_r_iter;
    printf("iteration %d: residual %.6e\n", l, ip.dot_r_iter);
  }
  dump("cg_dot_r", res, (size_t)(iters + 1) * sizeof(double));
  dump("cg_fhat_iter", ip.f_hat_iter, (size_t)p.N_total * sizeof(fftw_complex));
  t = ip.f_hat_iter;
  ip.f_hat_iter = p.f_hat;
  p.f_hat = t;
  nfft_trafo(&p);
  dump("cg_fit", p.f, (size_t)M * sizeof(fftw_complex));
  t = ip.f_hat_iter;
  ip.f_hat_iter = p.f_hat;
  p.f_hat = t;
  solver_finalize_complex(&ip);
  nfft_finalize(&p);
  return 0;
}

int main(int argc, char **argv)
{
  if (argc < 2) {
    fprintf(stderr, "usage: %s OUTDIR\n", argv[0]);
    return 2;
  }
  g_dir = argv[1];
  nfft_srand48(7);
  if (test_1d() || test_2d_full_psi() || test_3d_single() || test_solver()) return 1;
  printf("all calls done\n");
  return 0;
}
