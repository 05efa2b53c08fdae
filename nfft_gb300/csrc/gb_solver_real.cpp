// gb_solver_real.cpp -- solver_*_double and solverf_*_double: the iterations
// of the inverse-problem solver (Landweber, steepest descent, CGNR, CGNE) over
// a real linear operator, reference kernel/solver/solver.c:392-736.
//
// The operator is an mv_plan_double (N_total, M_total, real f_hat and f,
// mv_trafo, mv_adjoint) that the caller supplies.  This library has no
// real-valued transform of its own, so the operator is always the caller's
// code: the iteration runs on the host around its function pointers, in the
// reference's order of steps and with its vector swaps (RSWAP), so an
// operator sees exactly the calls it would see under the reference solver.
// Inner products accumulate in double precision.
#include <cstring>
#include <utility>

#include "../../include/nfft3.h"
#include "gb_common.cuh"

namespace {

template <typename R>
struct RVec {
  static double dot(const R *x, const R *w, long long n)
  {
    double s = 0;
    for (long long k = 0; k < n; ++k) s += w ? (double)w[k] * x[k] * x[k] : (double)x[k] * x[k];
    return s;
  }
  // x = w .* y (w == nullptr: x = y)
  static void cp(R *x, const R *w, const R *y, long long n)
  {
    for (long long k = 0; k < n; ++k) x[k] = w ? w[k] * y[k] : y[k];
  }
  // x = x + a w .* y (w == nullptr: x = x + a y)
  static void xpawy(R *x, double a, const R *w, const R *y, long long n)
  {
    for (long long k = 0; k < n; ++k) x[k] = (R)(x[k] + (w ? a * w[k] : a) * y[k]);
  }
  // x = a x + y
  static void axpy(R *x, double a, const R *y, long long n)
  {
    for (long long k = 0; k < n; ++k) x[k] = (R)(a * x[k] + y[k]);
  }
};

template <typename R, typename SP, typename MV, void *(*MAL)(size_t), void (*FREE)(void *)>
struct RealSolver {
  typedef RVec<R> V;

  static void init_advanced(SP *ths, MV *mv, unsigned flags)
  {
    memset(ths, 0, sizeof(*ths));
    ths->mv = mv;
    ths->flags = flags;
    const size_t M = (size_t)mv->M_total, N = (size_t)mv->N_total;
    ths->y = (R *)MAL(M * sizeof(R));
    ths->r_iter = (R *)MAL(M * sizeof(R));
    ths->f_hat_iter = (R *)MAL(N * sizeof(R));
    ths->p_hat_iter = (R *)MAL(N * sizeof(R));
    if (flags & (LANDWEBER | STEEPEST_DESCENT | CGNE)) ths->z_hat_iter = ths->p_hat_iter;
    if (flags & STEEPEST_DESCENT) ths->v_iter = (R *)MAL(M * sizeof(R));
    if (flags & CGNR) {
      ths->z_hat_iter = (R *)MAL(N * sizeof(R));
      ths->v_iter = (R *)MAL(M * sizeof(R));
    }
    if (flags & PRECOMPUTE_WEIGHT) ths->w = (R *)MAL(M * sizeof(R));
    if (flags & PRECOMPUTE_DAMP) ths->w_hat = (R *)MAL(N * sizeof(R));
  }

  static const R *wt(const SP *ths) { return (ths->flags & PRECOMPUTE_WEIGHT) ? ths->w : nullptr; }
  static const R *dm(const SP *ths) { return (ths->flags & PRECOMPUTE_DAMP) ? ths->w_hat : nullptr; }

  // out = A in (in: N values, out: M values) through the operator's own f
  static void apply(SP *ths, R *&out)
  {
    std::swap(out, ths->mv->f);
    ths->mv->mv_trafo(ths->mv);
    std::swap(out, ths->mv->f);
  }
  // z = A^T (w .* r)
  static void apply_adjoint_weighted(SP *ths, const R *r)
  {
    MV *mv = ths->mv;
    V::cp(mv->f, wt(ths), r, mv->M_total);
    std::swap(ths->z_hat_iter, mv->f_hat);
    mv->mv_adjoint(mv);
    std::swap(ths->z_hat_iter, mv->f_hat);
  }

  static void before_loop(SP *ths)
  {
    MV *mv = ths->mv;
    if (!mv || !mv->mv_trafo || !mv->mv_adjoint) gb::fatal("solver: mv plan without mv_trafo / mv_adjoint");
    const long long M = mv->M_total, N = mv->N_total;
    const bool norms = !(ths->flags & LANDWEBER) || (ths->flags & NORMS_FOR_LANDWEBER);
    V::cp(mv->f_hat, nullptr, ths->f_hat_iter, N);
    apply(ths, ths->r_iter);
    V::axpy(ths->r_iter, -1.0, ths->y, M);  // r = y - A f
    if (norms) ths->dot_r_iter = (R)V::dot(ths->r_iter, wt(ths), M);
    apply_adjoint_weighted(ths, ths->r_iter);
    if (norms) ths->dot_z_hat_iter = (R)V::dot(ths->z_hat_iter, dm(ths), N);
    if (ths->flags & CGNE) ths->dot_p_hat_iter = ths->dot_z_hat_iter;
    if (ths->flags & CGNR) V::cp(ths->p_hat_iter, nullptr, ths->z_hat_iter, N);
  }

  static void step(SP *ths)
  {
    MV *mv = ths->mv;
    const long long M = mv->M_total, N = mv->N_total;
    const unsigned fl = ths->flags;
    if (fl & LANDWEBER) {  // solver.c:479-526
      V::xpawy(ths->f_hat_iter, ths->alpha_iter, dm(ths), ths->z_hat_iter, N);
      V::cp(mv->f_hat, nullptr, ths->f_hat_iter, N);
      apply(ths, ths->r_iter);
      V::axpy(ths->r_iter, -1.0, ths->y, M);
      if (fl & NORMS_FOR_LANDWEBER) ths->dot_r_iter = (R)V::dot(ths->r_iter, wt(ths), M);
      apply_adjoint_weighted(ths, ths->r_iter);
      if (fl & NORMS_FOR_LANDWEBER) ths->dot_z_hat_iter = (R)V::dot(ths->z_hat_iter, dm(ths), N);
    } else if (fl & (STEEPEST_DESCENT | CGNR)) {  // solver.c:528-644
      const bool cg = (fl & CGNR) != 0;
      R *dir = cg ? ths->p_hat_iter : ths->z_hat_iter;
      V::cp(mv->f_hat, dm(ths), dir, N);
      apply(ths, ths->v_iter);
      ths->dot_v_iter = (R)V::dot(ths->v_iter, wt(ths), M);
      ths->alpha_iter = ths->dot_z_hat_iter / ths->dot_v_iter;
      V::xpawy(ths->f_hat_iter, ths->alpha_iter, dm(ths), dir, N);
      V::xpawy(ths->r_iter, -ths->alpha_iter, nullptr, ths->v_iter, M);
      ths->dot_r_iter = (R)V::dot(ths->r_iter, wt(ths), M);
      apply_adjoint_weighted(ths, ths->r_iter);
      ths->dot_z_hat_iter_old = ths->dot_z_hat_iter;
      ths->dot_z_hat_iter = (R)V::dot(ths->z_hat_iter, dm(ths), N);
      if (cg) {
        ths->beta_iter = ths->dot_z_hat_iter / ths->dot_z_hat_iter_old;
        V::axpy(ths->p_hat_iter, ths->beta_iter, ths->z_hat_iter, N);
      }
    } else if (fl & CGNE) {  // solver.c:646-696
      ths->alpha_iter = ths->dot_r_iter / ths->dot_p_hat_iter;
      V::xpawy(ths->f_hat_iter, ths->alpha_iter, dm(ths), ths->p_hat_iter, N);
      V::cp(mv->f_hat, dm(ths), ths->p_hat_iter, N);
      mv->mv_trafo(mv);
      V::xpawy(ths->r_iter, -ths->alpha_iter, nullptr, mv->f, M);
      ths->dot_r_iter_old = ths->dot_r_iter;
      ths->dot_r_iter = (R)V::dot(ths->r_iter, wt(ths), M);
      ths->beta_iter = ths->dot_r_iter / ths->dot_r_iter_old;
      V::cp(mv->f, wt(ths), ths->r_iter, M);
      mv->mv_adjoint(mv);
      V::axpy(ths->p_hat_iter, ths->beta_iter, mv->f_hat, N);
      ths->dot_p_hat_iter = (R)V::dot(ths->p_hat_iter, dm(ths), N);
    }
  }

  static void finalize(SP *ths)
  {
    const unsigned fl = ths->flags;
    if (fl & PRECOMPUTE_WEIGHT) FREE(ths->w);
    if (fl & PRECOMPUTE_DAMP) FREE(ths->w_hat);
    if (fl & CGNR) {
      FREE(ths->v_iter);
      FREE(ths->z_hat_iter);
    }
    if (fl & STEEPEST_DESCENT) FREE(ths->v_iter);
    FREE(ths->p_hat_iter);
    FREE(ths->f_hat_iter);
    FREE(ths->r_iter);
    FREE(ths->y);
  }
};

typedef RealSolver<double, solver_plan_double, nfft_mv_plan_double, nfft_malloc, nfft_free> RS;
typedef RealSolver<float, solverf_plan_double, nfftf_mv_plan_double, nfftf_malloc, nfftf_free> RSF;

}  // namespace

extern "C" {

void solver_init_advanced_double(solver_plan_double *ths, nfft_mv_plan_double *mv, unsigned flags)
{
  RS::init_advanced(ths, mv, flags);
}
void solver_init_double(solver_plan_double *ths, nfft_mv_plan_double *mv) { RS::init_advanced(ths, mv, CGNR); }
void solver_before_loop_double(solver_plan_double *ths) { RS::before_loop(ths); }
void solver_loop_one_step_double(solver_plan_double *ths) { RS::step(ths); }
void solver_finalize_double(solver_plan_double *ths) { RS::finalize(ths); }

void solverf_init_advanced_double(solverf_plan_double *ths, nfftf_mv_plan_double *mv, unsigned flags)
{
  RSF::init_advanced(ths, mv, flags);
}
void solverf_init_double(solverf_plan_double *ths, nfftf_mv_plan_double *mv) { RSF::init_advanced(ths, mv, CGNR); }
void solverf_before_loop_double(solverf_plan_double *ths) { RSF::before_loop(ths); }
void solverf_loop_one_step_double(solverf_plan_double *ths) { RSF::step(ths); }
void solverf_finalize_double(solverf_plan_double *ths) { RSF::finalize(ths); }

}  // extern "C"
