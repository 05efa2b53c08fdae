/*
 * nfft3.h -- drop-in C API of the GB300 NFFT library (libnfft3_gb300.so).
 *
 * Declares the NFFT 3 entry points and structures that the transform path and
 * the inverse-NFFT solver use, with the same names, argument meanings and
 * structure layouts as the reference header (reference include/nfft3.h), so
 * that a program written against NFFT 3 recompiles -- or relinks -- against
 * this library unchanged.  Every declaration names the reference declaration
 * it replaces.
 *
 * Semantics that differ by design:
 *  - transforms run on the GPU (cuFFT for the oversampled FFT, hand-written
 *    sm_103a kernels for D, B and B^T) and return only when the result is in
 *    the host arrays, so callers may read f / f_hat right after the call;
 *  - the window is evaluated on the fly; PRE_PSI, PRE_FULL_PSI, PRE_LIN_PSI
 *    and PRE_FG_PSI are accepted and give the same results, but no psi table
 *    is allocated (psi, psi_index_g, psi_index_f stay NULL);
 *  - g, g_hat, g1 and g2 live in GPU memory and are NULL in the host struct;
 *  - my_fftw_plan1 holds the library's device context (opaque).
 */
#ifndef NFFT3_H_GB300
#define NFFT3_H_GB300

#include <stddef.h>
#include <fftw3.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NFFT_CONCAT(prefix, name) prefix ## name
#define NFFT_EXTERN extern

/* reference include/nfft3.h:51 */
typedef ptrdiff_t NFFT_INT;

/* reference include/nfft3.h:54-60 (members shared by all plans) */
#define MACRO_MV_PLAN(RC) \
  NFFT_INT N_total; \
  NFFT_INT M_total; \
  RC *f_hat; \
  RC *f; \
  void (*mv_trafo)(void*); \
  void (*mv_adjoint)(void*);

#define NFFT_MANGLE_DOUBLE(name) NFFT_CONCAT(nfft_, name)
#define NFFT_MANGLE_FLOAT(name) NFFT_CONCAT(nfftf_, name)

/* reference include/nfft3.h:70-85: allocation and exit hooks */
#define NFFT_DEFINE_MALLOC_API(X) \
NFFT_EXTERN void *X(malloc)(size_t n); \
NFFT_EXTERN void X(free)(void *p); \
NFFT_EXTERN void X(die)(const char *s); \
typedef void *(*X(malloc_type_function)) (size_t n); \
typedef void  (*X(free_type_function)) (void *p); \
typedef void  (*X(die_type_function)) (const char *errString); \
NFFT_EXTERN X(malloc_type_function) X(malloc_hook); \
NFFT_EXTERN X(free_type_function) X(free_hook); \
NFFT_EXTERN X(die_type_function) X(die_hook);

NFFT_DEFINE_MALLOC_API(NFFT_MANGLE_FLOAT)
NFFT_DEFINE_MALLOC_API(NFFT_MANGLE_DOUBLE)

/* reference include/nfft3.h:96-187: plan structures and transform API */
#define NFFT_DEFINE_API(X,Y,R,C) \
typedef struct { MACRO_MV_PLAN(C) } X(mv_plan_complex); \
typedef struct { MACRO_MV_PLAN(R) } X(mv_plan_double); \
typedef struct \
{ \
  MACRO_MV_PLAN(C) \
  NFFT_INT d; \
  NFFT_INT *N; \
  R *sigma; \
  NFFT_INT *n; \
  NFFT_INT n_total; \
  NFFT_INT m; \
  R *b; \
  NFFT_INT K; \
  unsigned flags; \
  unsigned fftw_flags; \
  R *x; \
  R MEASURE_TIME_t[3]; \
  Y(plan) my_fftw_plan1; \
  Y(plan) my_fftw_plan2; \
  R **c_phi_inv; \
  R *psi; \
  NFFT_INT *psi_index_g; \
  NFFT_INT *psi_index_f; \
  C *g; \
  C *g_hat; \
  C *g1; \
  C *g2; \
  R *spline_coeffs; \
  NFFT_INT *index_x; \
} X(plan); \
NFFT_EXTERN void X(trafo_direct)(const X(plan) *ths); \
NFFT_EXTERN void X(adjoint_direct)(const X(plan) *ths); \
NFFT_EXTERN void X(trafo)(X(plan) *ths); \
NFFT_EXTERN void X(trafo_1d)(X(plan) *ths); \
NFFT_EXTERN void X(trafo_2d)(X(plan) *ths); \
NFFT_EXTERN void X(trafo_3d)(X(plan) *ths); \
NFFT_EXTERN void X(adjoint)(X(plan) *ths); \
NFFT_EXTERN void X(adjoint_1d)(X(plan) *ths); \
NFFT_EXTERN void X(adjoint_2d)(X(plan) *ths); \
NFFT_EXTERN void X(adjoint_3d)(X(plan) *ths); \
NFFT_EXTERN void X(init_1d)(X(plan) *ths, int N1, int M); \
NFFT_EXTERN void X(init_2d)(X(plan) *ths, int N1, int N2, int M); \
NFFT_EXTERN void X(init_3d)(X(plan) *ths, int N1, int N2, int N3, int M); \
NFFT_EXTERN void X(init)(X(plan) *ths, int d, int *N, int M); \
NFFT_EXTERN void X(init_guru)(X(plan) *ths, int d, int *N, int M, int *n, \
  int m, unsigned flags, unsigned fftw_flags); \
NFFT_EXTERN void X(init_lin)(X(plan) *ths, int d, int *N, int M, int *n, \
  int m, int K, unsigned flags, unsigned fftw_flags); \
NFFT_EXTERN void X(precompute_one_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_full_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_fg_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_lin_psi)(X(plan) *ths); \
NFFT_EXTERN const char* X(check)(X(plan) *ths); \
NFFT_EXTERN void X(finalize)(X(plan) *ths);

NFFT_DEFINE_API(NFFT_MANGLE_FLOAT,FFTW_MANGLE_FLOAT,float,fftwf_complex)
NFFT_DEFINE_API(NFFT_MANGLE_DOUBLE,FFTW_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:195-209: plan flags */
#define PRE_PHI_HUT                (1U<<0)
#define FG_PSI                     (1U<<1)
#define PRE_LIN_PSI                (1U<<2)
#define PRE_FG_PSI                 (1U<<3)
#define PRE_PSI                    (1U<<4)
#define PRE_FULL_PSI               (1U<<5)
#define MALLOC_X                   (1U<<6)
#define MALLOC_F_HAT               (1U<<7)
#define MALLOC_F                   (1U<<8)
#define FFT_OUT_OF_PLACE           (1U<<9)
#define FFTW_INIT                  (1U<<10)
#define NFFT_SORT_NODES            (1U<<11)
#define NFFT_OMP_BLOCKWISE_ADJOINT (1U<<12)
#define PRE_ONE_PSI (PRE_LIN_PSI| PRE_FG_PSI| PRE_PSI| PRE_FULL_PSI)

/* reference include/nfft3.h:375-440: NNFFT, nonequispaced nodes in both space
 * and frequency (double precision, as the reference's kernel/nnfft/nnfft.c) */
#define NNFFT_MANGLE_DOUBLE(name) NFFT_CONCAT(nnfft_, name)

#define NNFFT_DEFINE_API(X,Z,R,C) \
typedef struct \
{ \
  MACRO_MV_PLAN(C) \
  int d; \
  R *sigma; \
  R *a; \
  int *N; \
  int *N1; \
  int *aN1; \
  int m; \
  R *b; \
  int K; \
  int aN1_total; \
  Z(plan) *direct_plan; \
  unsigned nnfft_flags; \
  int *n; \
  R *x; \
  R *v; \
  R *c_phi_inv; \
  R *psi; \
  int size_psi; \
  int *psi_index_g; \
  int *psi_index_f; \
  C *F; \
  R *spline_coeffs; \
} X(plan); \
NFFT_EXTERN void X(init)(X(plan) *ths_plan, int d, int N_total, int M_total, int *N); \
NFFT_EXTERN void X(init_1d)(X(plan) *ths_plan, int N, int M_total); \
NFFT_EXTERN void X(init_guru)(X(plan) *ths_plan, int d, int N_total, int M_total, \
  int *N, int *N1, int m, unsigned nnfft_flags); \
NFFT_EXTERN void X(trafo_direct)(X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint_direct)(X(plan) *ths_plan); \
NFFT_EXTERN void X(trafo)(X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint)(X(plan) *ths_plan); \
NFFT_EXTERN void X(precompute_lin_psi)(X(plan) *ths_plan); \
NFFT_EXTERN void X(precompute_psi)(X(plan) *ths_plan); \
NFFT_EXTERN void X(precompute_full_psi)(X(plan) *ths_plan); \
NFFT_EXTERN void X(precompute_phi_hut)(X(plan) *ths_plan); \
NFFT_EXTERN void X(precompute_one_psi)(X(plan) *ths); \
NFFT_EXTERN void X(finalize)(X(plan) *ths_plan);

NNFFT_DEFINE_API(NNFFT_MANGLE_DOUBLE,NFFT_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:439: additional NNFFT init flag */
#define MALLOC_V         (1U<< 11)

/* reference include/nfft3.h:210-288: NFCT, the nonequispaced fast cosine
 * transform, f_j = sum_{0 <= k < N} f_hat_k prod_t cos(2 pi k_t x_jt),
 * nodes x in [0, 1/2]^d */
#define NFCT_MANGLE_DOUBLE(name) NFFT_CONCAT(nfct_, name)
#define NFCT_MANGLE_FLOAT(name) NFFT_CONCAT(nfctf_, name)

#define NFCT_DEFINE_API(X,Y,R,C) \
typedef struct \
{ \
  MACRO_MV_PLAN(R) \
  NFFT_INT d; \
  NFFT_INT *N; \
  NFFT_INT *n; \
  NFFT_INT n_total; \
  R *sigma; \
  NFFT_INT m; \
  R *b; \
  NFFT_INT K; \
  unsigned flags; \
  unsigned fftw_flags; \
  R *x; \
  double MEASURE_TIME_t[3]; \
  Y(plan) my_fftw_r2r_plan; \
  Y(r2r_kind) *r2r_kind; \
  R **c_phi_inv; \
  R *psi; \
  NFFT_INT size_psi; \
  NFFT_INT *psi_index_g; \
  NFFT_INT *psi_index_f; \
  R *g; \
  R *g_hat; \
  R *g1; \
  R *g2; \
  R *spline_coeffs; \
} X(plan); \
NFFT_EXTERN void X(init_1d)(X(plan) *ths_plan, int N0, int M_total); \
NFFT_EXTERN void X(init_2d)(X(plan) *ths_plan, int N0, int N1, int M_total); \
NFFT_EXTERN void X(init_3d)(X(plan) *ths_plan, int N0, int N1, int N2, int M_total); \
NFFT_EXTERN void X(init)(X(plan) *ths_plan, int d, int *N, int M_total); \
NFFT_EXTERN void X(init_guru)(X(plan) *ths_plan, int d, int *N, int M_total, int *n, \
  int m, unsigned flags, unsigned fftw_flags); \
NFFT_EXTERN void X(precompute_one_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_full_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_fg_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_lin_psi)(X(plan) *ths); \
NFFT_EXTERN void X(trafo)(X(plan) *ths_plan); \
NFFT_EXTERN void X(trafo_direct)(const X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint)(X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint_direct)(const X(plan) *ths_plan); \
NFFT_EXTERN const char* X(check)(X(plan) *ths); \
NFFT_EXTERN void X(finalize)(X(plan) *ths_plan);

NFCT_DEFINE_API(NFCT_MANGLE_FLOAT,FFTW_MANGLE_FLOAT,float,fftwf_complex)
NFCT_DEFINE_API(NFCT_MANGLE_DOUBLE,FFTW_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:290-355: NFST, the nonequispaced fast sine
 * transform, f_j = sum_{1 <= k < N} f_hat_{k-1} prod_t sin(2 pi k_t x_jt),
 * nodes x in [0, 1/2]^d */
#define NFST_MANGLE_DOUBLE(name) NFFT_CONCAT(nfst_, name)
#define NFST_MANGLE_FLOAT(name) NFFT_CONCAT(nfstf_, name)

#define NFST_DEFINE_API(X,Y,R,C) \
typedef struct \
{ \
  MACRO_MV_PLAN(R) \
  NFFT_INT d; \
  NFFT_INT *N; \
  NFFT_INT *n; \
  NFFT_INT n_total; \
  R *sigma; \
  NFFT_INT m; \
  R *b; \
  NFFT_INT K; \
  unsigned flags; \
  unsigned fftw_flags; \
  R *x; \
  double MEASURE_TIME_t[3]; \
  Y(plan) my_fftw_r2r_plan; \
  Y(r2r_kind) *r2r_kind; \
  R **c_phi_inv; \
  R *psi; \
  NFFT_INT size_psi; \
  NFFT_INT *psi_index_g; \
  NFFT_INT *psi_index_f; \
  R *g; \
  R *g_hat; \
  R *g1; \
  R *g2; \
  R *spline_coeffs; \
  R X(full_psi_eps); \
} X(plan); \
NFFT_EXTERN void X(init_1d)(X(plan) *ths_plan, int N0, int M_total); \
NFFT_EXTERN void X(init_2d)(X(plan) *ths_plan, int N0, int N1, int M_total); \
NFFT_EXTERN void X(init_3d)(X(plan) *ths_plan, int N0, int N1, int N2, int M_total); \
NFFT_EXTERN void X(init)(X(plan) *ths_plan, int d, int *N, int M_total); \
NFFT_EXTERN void X(init_guru)(X(plan) *ths_plan, int d, int *N, int M_total, int *n, \
  int m, unsigned flags, unsigned fftw_flags); \
NFFT_EXTERN void X(precompute_one_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_full_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_fg_psi)(X(plan) *ths); \
NFFT_EXTERN void X(precompute_lin_psi)(X(plan) *ths); \
NFFT_EXTERN void X(trafo)(X(plan) *ths_plan); \
NFFT_EXTERN void X(trafo_direct)(const X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint)(X(plan) *ths_plan); \
NFFT_EXTERN void X(adjoint_direct)(const X(plan) *ths_plan); \
NFFT_EXTERN const char* X(check)(X(plan) *ths); \
NFFT_EXTERN void X(finalize)(X(plan) *ths_plan);

NFST_DEFINE_API(NFST_MANGLE_FLOAT,FFTW_MANGLE_FLOAT,float,fftwf_complex)
NFST_DEFINE_API(NFST_MANGLE_DOUBLE,FFTW_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:500-545: MRI operators with a field inhomogeneity
 * (double precision, as the reference's kernel/mri/mri.c) */
#define MRI_MANGLE_DOUBLE(name) NFFT_CONCAT(mri_, name)

#define MRI_DEFINE_API(X,Z,R,C) \
typedef struct \
{ \
  MACRO_MV_PLAN(C) \
  Z(plan) plan; \
  int N3; \
  R sigma3; \
  R *t; \
  R *w; \
} X(inh_2d1d_plan); \
typedef struct \
{ \
  MACRO_MV_PLAN(C) \
  Z(plan) plan; \
  int N3; \
  R sigma3; \
  R *t; \
  R *w; \
} X(inh_3d_plan); \
void X(inh_2d1d_trafo)(X(inh_2d1d_plan) *ths); \
void X(inh_2d1d_adjoint)(X(inh_2d1d_plan) *ths); \
void X(inh_2d1d_init_guru)(X(inh_2d1d_plan) *ths, int *N, int M, int *n, \
  int m, R sigma, unsigned nfft_flags, unsigned fftw_flags); \
void X(inh_2d1d_finalize)(X(inh_2d1d_plan) *ths); \
void X(inh_3d_trafo)(X(inh_3d_plan) *ths); \
void X(inh_3d_adjoint)(X(inh_3d_plan) *ths); \
void X(inh_3d_init_guru)(X(inh_3d_plan) *ths, int *N, int M, int *n, \
  int m, R sigma, unsigned nfft_flags, unsigned fftw_flags); \
void X(inh_3d_finalize)(X(inh_3d_plan) *ths);

MRI_DEFINE_API(MRI_MANGLE_DOUBLE,NFFT_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:747-815: inverse NFFT solver */
#define SOLVER_MANGLE_DOUBLE(name) NFFT_CONCAT(solver_, name)
#define SOLVER_MANGLE_FLOAT(name) NFFT_CONCAT(solverf_, name)

#define SOLVER_DEFINE_API(X,Y,R,C) \
typedef struct \
{ \
  Y(mv_plan_complex) *mv; \
  unsigned flags; \
  R *w; \
  R *w_hat; \
  C *y; \
  C *f_hat_iter; \
  C *r_iter; \
  C *z_hat_iter; \
  C *p_hat_iter; \
  C *v_iter; \
  R alpha_iter; \
  R beta_iter; \
  R dot_r_iter; \
  R dot_r_iter_old; \
  R dot_z_hat_iter; \
  R dot_z_hat_iter_old; \
  R dot_p_hat_iter; \
  R dot_v_iter; \
} X(plan_complex); \
NFFT_EXTERN void X(init_advanced_complex)(X(plan_complex)* ths, Y(mv_plan_complex) *mv, unsigned flags); \
NFFT_EXTERN void X(init_complex)(X(plan_complex)* ths, Y(mv_plan_complex) *mv); \
NFFT_EXTERN void X(before_loop_complex)(X(plan_complex)* ths); \
NFFT_EXTERN void X(loop_one_step_complex)(X(plan_complex) *ths); \
NFFT_EXTERN void X(finalize_complex)(X(plan_complex) *ths); \
/* reference include/nfft3.h:788-815: the same solver over a real operator */ \
typedef struct \
{ \
  Y(mv_plan_double) *mv; \
  unsigned flags; \
  R *w; \
  R *w_hat; \
  R *y; \
  R *f_hat_iter; \
  R *r_iter; \
  R *z_hat_iter; \
  R *p_hat_iter; \
  R *v_iter; \
  R alpha_iter; \
  R beta_iter; \
  R dot_r_iter; \
  R dot_r_iter_old; \
  R dot_z_hat_iter; \
  R dot_z_hat_iter_old; \
  R dot_p_hat_iter; \
  R dot_v_iter; \
} X(plan_double); \
NFFT_EXTERN void X(init_advanced_double)(X(plan_double)* ths, Y(mv_plan_double) *mv, unsigned flags); \
NFFT_EXTERN void X(init_double)(X(plan_double)* ths, Y(mv_plan_double) *mv); \
NFFT_EXTERN void X(before_loop_double)(X(plan_double)* ths); \
NFFT_EXTERN void X(loop_one_step_double)(X(plan_double) *ths); \
NFFT_EXTERN void X(finalize_double)(X(plan_double) *ths);

SOLVER_DEFINE_API(SOLVER_MANGLE_FLOAT,NFFT_MANGLE_FLOAT,float,fftwf_complex)
SOLVER_DEFINE_API(SOLVER_MANGLE_DOUBLE,NFFT_MANGLE_DOUBLE,double,fftw_complex)

/* reference include/nfft3.h:822-829: solver flags */
#define LANDWEBER             (1U<< 0)
#define STEEPEST_DESCENT      (1U<< 1)
#define CGNR                  (1U<< 2)
#define CGNE                  (1U<< 3)
#define NORMS_FOR_LANDWEBER   (1U<< 4)
#define PRECOMPUTE_WEIGHT     (1U<< 5)
#define PRECOMPUTE_DAMP       (1U<< 6)

/* reference include/nfft3.h:839-890: utilities used by callers and tests */
#define NFFT_DEFINE_UTIL_API(Y,R,C) \
R Y(drand48)(void); \
void Y(srand48)(long int seed); \
void Y(vrand_unit_complex)(C *x, const NFFT_INT n); \
void Y(vrand_shifted_unit_double)(R *x, const NFFT_INT n); \
void Y(vrand_real)(R *x, const NFFT_INT n, const R a, const R b); \
void Y(vpr_double)(R *x, const NFFT_INT n, const char *text); \
void Y(vpr_complex)(C *x, const NFFT_INT n, const char *text); \
NFFT_INT Y(get_num_threads)(void); \
void Y(set_num_threads)(NFFT_INT nthreads); \
NFFT_INT Y(has_threads_enabled)(void); \
R Y(clock_gettime_seconds)(void); \
R Y(error_l_infty_complex)(const C *x, const C *y, const NFFT_INT n); \
R Y(error_l_infty_1_complex)(const C *x, const C *y, const NFFT_INT n, \
  const C *z, const NFFT_INT m); \
NFFT_INT Y(exp2i)(const NFFT_INT a); \
NFFT_INT Y(next_power_of_2)(const NFFT_INT N); \
R Y(dot_complex)(C *x, NFFT_INT n); \
void Y(upd_axpy_complex)(C *x, R a, C *y, NFFT_INT n); \
void Y(fftshift_complex)(C *x, NFFT_INT d, NFFT_INT* N); \
void Y(fftshift_complex_int)(C *x, int d, int* N); \
void Y(get_version)(unsigned *major, unsigned *minor, unsigned *patch); \
const char *Y(get_window_name)(void); \
NFFT_INT Y(get_default_window_cut_off)(void);

NFFT_DEFINE_UTIL_API(NFFT_MANGLE_FLOAT,float,fftwf_complex)
NFFT_DEFINE_UTIL_API(NFFT_MANGLE_DOUBLE,double,fftw_complex)

#ifdef __cplusplus
}
#endif

#endif /* NFFT3_H_GB300 */
