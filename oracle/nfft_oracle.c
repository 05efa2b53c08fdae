/*
 * oracle/nfft_oracle.c -- CPU restatement of the NFFT transform path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the tests use it as the
 * checker for the GPU library, and the benchmark's CPU-baseline leg times it
 * on the host cores.  The product library never links, loads or calls it.
 *
 * It restates, in plain C + OpenMP, the algorithm of the reference NFFT 3.5.4
 * (Keiner, Kunis, Potts), for the Kaiser-Bessel window that the reference
 * selects by default.  Each function cites the reference file:line it follows
 * (paths relative to the reference project root).  Compiled twice: double
 * (prefix orc_) and -DORC_SINGLE float (prefix orcf_), mirroring the
 * reference's nfft_/nfftf_ precisions (include/infft.h:66-99).
 *
 * Complex vectors are interleaved (re, im) arrays of R.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORC_SINGLE
typedef float R;
#define P(name) orcf_##name
#define SQRT sqrtf
#define SINH sinhf
#define SIN sinf
#define FLOOR floorf
#define LRINT lrintf
#else
typedef double R;
#define P(name) orc_##name
#define SQRT sqrt
#define SINH sinh
#define SIN sin
#define FLOOR floor
#define LRINT lrint
#endif

#define ORC_PI 3.1415926535897932384626433832795028841971693993751
#define ORC_2PI 6.2831853071795864769252867665590057683943387987502
#define KPI ((R)ORC_PI)
#define K2PI ((R)ORC_2PI)

typedef ptrdiff_t INT;

void P(fft)(int d, const int *n, R *data, int sign);

/* Oracle plan flags. */
#define ORC_SORT 1u          /* compute the sorted node index (NFFT_SORT_NODES) */
#define ORC_BLOCKWISE 2u     /* OpenMP blockwise adjoint over dim-0 slabs */
#define ORC_PRE_PSI 4u       /* keep the M*d*(2m+2) window table (PRE_PSI) */

typedef struct {
  int d, m;
  int N[8], n[8];
  INT M, N_total, n_total;
  R sigma[8], b[8];
  unsigned flags;
  R *x;          /* M*d node coordinates, node-major (x[j*d+t]) */
  R *c_phi_inv;  /* concatenated per-dim tables, N_0 + ... + N_{d-1} */
  R *psi;        /* M*d*(2m+2) when ORC_PRE_PSI */
  INT *index_x;  /* 2*M: (key, node) pairs after the stable sort */
  R *g;          /* oversampled grid, n_total complex */
  double t_stage[3]; /* last call: D, FFT, B (seconds) */
} orc_plan;

static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------- */
/* Modified Bessel function I0.                                              */
/* The reference evaluates I0 with rational Chebyshev fits per precision      */
/* (kernel/util/bessel_i0.c:212-338).  Restated here from the defining power */
/* series I0(x) = sum_k ((x/2)^(2k)) / (k!)^2, summed in long double until   */
/* the terms stop contributing; for x > 700 the leading asymptotic term       */
/* e^x / sqrt(2 pi x) (1 + 1/(8x) + 9/(128x^2)) is used.                     */
/* ------------------------------------------------------------------------- */
double P(bessel_i0)(double x)
{
  long double ax = fabsl((long double)x), q, term, sum;
  int k;
  if (ax > 700.0L) {
    long double r = 1.0L / ax;
    return (double)(expl(ax) / sqrtl(2.0L * (long double)ORC_PI * ax) *
                    (1.0L + r / 8.0L + 9.0L * r * r / 128.0L));
  }
  q = ax * ax / 4.0L;
  term = 1.0L;
  sum = 1.0L;
  for (k = 1; k < 2000; k++) {
    term *= q / ((long double)k * (long double)k);
    sum += term;
    if (term < sum * 1e-21L) break;
  }
  return (double)sum;
}

/* Kaiser-Bessel window phi(x) for grid length n (include/infft.h:209-215).
 * The argument order of the products mirrors the macro so that the float
 * build rounds like the reference's nfftf build. */
R P(phi)(int n, int m, R b, R x)
{
  const R mm = (R)m * (R)m;
  const R arg = mm - x * (R)n * x * (R)n;
  if (arg > (R)0.0) {
    const R s = SQRT(arg);
    return SINH(b * s) / (KPI * s);
  } else if (arg < (R)0.0) {
    const R s = SQRT(x * (R)n * x * (R)n - mm);
    return SIN(b * s) / (KPI * s);
  }
  return b / KPI;
}

/* Fourier coefficient of the window, PHI_HUT (include/infft.h:208). */
static R phi_hut(const orc_plan *p, int n, INT k, int t)
{
  const R a = (R)2.0 * KPI * (R)k / (R)n;
  return (R)P(bessel_i0)((double)((R)p->m * SQRT(p->b[t] * p->b[t] - a * a)));
}

/* ------------------------------------------------------------------------- */
/* Plan set-up: init_help (kernel/nfft/nfft.c:5950-6046) and                 */
/* precompute_phi_hut (nfft.c:5754-5770).                                    */
/* ------------------------------------------------------------------------- */
orc_plan *P(plan_create)(int d, const int *N, const int *n, int m, long M,
                         unsigned flags)
{
  orc_plan *p = (orc_plan*)calloc(1, sizeof(orc_plan));
  int t;
  INT k, off;
  p->d = d; p->m = m; p->M = M; p->flags = flags;
  p->N_total = 1; p->n_total = 1;
  for (t = 0; t < d; t++) {
    p->N[t] = N[t]; p->n[t] = n[t];
    p->N_total *= N[t]; p->n_total *= n[t];
    p->sigma[t] = (R)n[t] / (R)N[t];
    /* b = pi (2 - 1/sigma), include/infft.h:216-222 */
    p->b[t] = KPI * ((R)2.0 - (R)1.0 / p->sigma[t]);
  }
  p->x = (R*)calloc((size_t)(M * d) + 1, sizeof(R));
  off = 0;
  for (t = 0; t < d; t++) off += N[t];
  p->c_phi_inv = (R*)malloc(sizeof(R) * (size_t)off);
  off = 0;
  for (t = 0; t < d; t++) {
    for (k = 0; k < N[t]; k++)
      p->c_phi_inv[off + k] = (R)1.0 / phi_hut(p, n[t], k - N[t] / 2, t);
    off += N[t];
  }
  p->g = (R*)malloc(sizeof(R) * 2 * (size_t)p->n_total);
  if (flags & (ORC_SORT | ORC_BLOCKWISE))
    p->index_x = (INT*)malloc(sizeof(INT) * 2 * (size_t)(M > 0 ? M : 1));
  return p;
}

void P(plan_destroy)(orc_plan *p)
{
  if (!p) return;
  free(p->x); free(p->c_phi_inv); free(p->psi); free(p->index_x); free(p->g);
  free(p);
}

void P(set_nodes)(orc_plan *p, const R *x)
{
  memcpy(p->x, x, sizeof(R) * (size_t)(p->M * p->d));
}

void P(get_c_phi_inv)(const orc_plan *p, double *out)
{
  INT off = 0, k;
  int t;
  for (t = 0; t < p->d; t++) off += p->N[t];
  for (k = 0; k < off; k++) out[k] = (double)p->c_phi_inv[k];
}

void P(get_index_x)(const orc_plan *p, int64_t *out)
{
  INT j;
  for (j = 0; j < 2 * p->M; j++) out[j] = (int64_t)p->index_x[j];
}

void P(stage_times)(const orc_plan *p, double *t3)
{
  t3[0] = p->t_stage[0]; t3[1] = p->t_stage[1]; t3[2] = p->t_stage[2];
}

/* ------------------------------------------------------------------------- */
/* Node sort: sort0 (nfft.c:75-109) computes per node the key               */
/*   sum_t u_t * prod_{s>t} n_s,  u_t = ((lrint(floor(n_t*x_t - m)) % n_t)   */
/*                                       + n_t) % n_t                       */
/* and sorts (key, j) pairs stably by key (kernel/util/sort.c:91-171 is an   */
/* LSD radix sort; any stable sort yields the same permutation).  Restated   */
/* here as an LSD radix sort with 8-bit digits.                              */
/* ------------------------------------------------------------------------- */
static void sort_nodes(orc_plan *p)
{
  const INT M = p->M;
  const int d = p->d;
  INT *ar = p->index_x, *tmp, j;
  int shift, t;
  INT nprod = p->n_total;
  int bits = 0;
  while (((INT)1 << bits) < nprod) bits++;
  for (j = 0; j < M; j++) {
    INT key = 0;
    for (t = 0; t < d; t++) {
      /* evaluated in plan precision without contraction: n*x rounded, then -m */
      volatile R nx = (R)p->n[t] * p->x[d * j + t];
      volatile R v = nx - (R)p->m;
      INT help = (INT)LRINT(FLOOR(v));
      INT u = (help % p->n[t] + p->n[t]) % p->n[t];
      key += u;
      if (t + 1 < d) key *= p->n[t + 1];
    }
    ar[2 * j] = key;
    ar[2 * j + 1] = j;
  }
  tmp = (INT*)malloc(sizeof(INT) * 2 * (size_t)(M > 0 ? M : 1));
  for (shift = 0; shift < bits; shift += 8) {
    INT cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (j = 0; j < M; j++) cnt[((ar[2 * j] >> shift) & 255) + 1]++;
    for (t = 0; t < 256; t++) cnt[t + 1] += cnt[t];
    for (j = 0; j < M; j++) {
      INT pos = cnt[(ar[2 * j] >> shift) & 255]++;
      tmp[2 * pos] = ar[2 * j];
      tmp[2 * pos + 1] = ar[2 * j + 1];
    }
    memcpy(ar, tmp, sizeof(INT) * 2 * (size_t)M);
  }
  free(tmp);
}

/* ------------------------------------------------------------------------- */
/* Window support and values: uo (nfft.c:324-332) gives u = floor(x n) - m,  */
/* the 2m+2 indices are u..u+2m+1 (wrapped mod n for memory, nfft.c:334-340) */
/* and the window values are phi(x - l/n) with the unwrapped l               */
/* (precompute_psi, nfft.c:5819-5844).                                       */
/* ------------------------------------------------------------------------- */
static inline INT node_u(const orc_plan *p, INT j, int t)
{
  const R xj = p->x[j * p->d + t];
  return (INT)LRINT(FLOOR(xj * (R)p->n[t])) - p->m;
}

static inline void node_psi(const orc_plan *p, INT j, int t, R *out)
{
  const int w = 2 * p->m + 2;
  const INT u = node_u(p, j, t);
  int l;
  for (l = 0; l < w; l++)
    out[l] = P(phi)(p->n[t], p->m, p->b[t],
                    p->x[j * p->d + t] - ((R)(u + l)) / (R)p->n[t]);
}

void P(precompute)(orc_plan *p)
{
  const int w = 2 * p->m + 2;
  if (p->index_x) sort_nodes(p);
  if (p->flags & ORC_PRE_PSI) {
    INT j;
    free(p->psi);
    p->psi = (R*)malloc(sizeof(R) * (size_t)(p->M * p->d * w + 1));
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (j = 0; j < p->M; j++) {
      int t;
      for (t = 0; t < p->d; t++) node_psi(p, j, t, p->psi + (j * p->d + t) * w);
    }
  }
}

static inline const R *psi_of(const orc_plan *p, INT j, int t, R *scratch)
{
  const int w = 2 * p->m + 2;
  if (p->psi) return p->psi + (j * p->d + t) * w;
  node_psi(p, j, t, scratch);
  return scratch;
}

/* ------------------------------------------------------------------------- */
/* NDFT: nfft_trafo_direct (nfft.c:145-205) and nfft_adjoint_direct          */
/* (nfft.c:207-297).  f_j = sum_k f^_k exp(-2 pi i k.x_j),                   */
/* f^_k = sum_j f_j exp(+2 pi i k.x_j), k in natural order -N/2..N/2-1 with  */
/* the last dimension fastest.  Evaluated here in long double with the phase */
/* reduced exactly for accuracy (it is the FP64 truth for the checks).       */
/* ------------------------------------------------------------------------- */
static void kvec(const orc_plan *p, INT kL, INT *k)
{
  int t;
  for (t = p->d - 1; t >= 0; t--) {
    k[t] = kL % p->N[t] - p->N[t] / 2;
    kL /= p->N[t];
  }
}

void P(trafo_direct)(const orc_plan *p, const R *fhat, R *f)
{
  INT j;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (j = 0; j < p->M; j++) {
    long double sr = 0.0L, si = 0.0L;
    INT kL, k[8];
    int t;
    for (kL = 0; kL < p->N_total; kL++) {
      long double ph = 0.0L, c, s;
      kvec(p, kL, k);
      for (t = 0; t < p->d; t++) ph += (long double)k[t] * (long double)p->x[j * p->d + t];
      ph -= floorl(ph);
      c = cosl(-2.0L * (long double)ORC_PI * ph);
      s = sinl(-2.0L * (long double)ORC_PI * ph);
      sr += fhat[2 * kL] * c - fhat[2 * kL + 1] * s;
      si += fhat[2 * kL] * s + fhat[2 * kL + 1] * c;
    }
    f[2 * j] = (R)sr; f[2 * j + 1] = (R)si;
  }
}

void P(adjoint_direct)(const orc_plan *p, const R *f, R *fhat)
{
  INT kL;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (kL = 0; kL < p->N_total; kL++) {
    long double sr = 0.0L, si = 0.0L;
    INT j, k[8];
    int t;
    kvec(p, kL, k);
    for (j = 0; j < p->M; j++) {
      long double ph = 0.0L, c, s;
      for (t = 0; t < p->d; t++) ph += (long double)k[t] * (long double)p->x[j * p->d + t];
      ph -= floorl(ph);
      c = cosl(2.0L * (long double)ORC_PI * ph);
      s = sinl(2.0L * (long double)ORC_PI * ph);
      sr += f[2 * j] * c - f[2 * j + 1] * s;
      si += f[2 * j] * s + f[2 * j + 1] * c;
    }
    fhat[2 * kL] = (R)sr; fhat[2 * kL + 1] = (R)si;
  }
}

/* ------------------------------------------------------------------------- */
/* D and D^T: zero-pad with roll-off correction into FFT order and crop back */
/* (trafo_2d D part nfft.c:3833-3897, adjoint_2d nfft.c:3941-3997; generic   */
/* D_openmp_A/T nfft.c:440-613).  Frequency k_t in -N_t/2..N_t/2-1 sits at   */
/* grid position k_t mod n_t.                                                */
/* ------------------------------------------------------------------------- */
static INT grid_pos_of_freq(const orc_plan *p, INT kL, R *c)
{
  INT k[8], pos = 0, off = 0;
  int t;
  kvec(p, kL, k);
  *c = (R)1.0;
  for (t = 0; t < p->d; t++) {
    INT kt = k[t] < 0 ? k[t] + p->n[t] : k[t];
    pos = pos * p->n[t] + kt;
    *c *= p->c_phi_inv[off + k[t] + p->N[t] / 2];
    off += p->N[t];
  }
  return pos;
}

static void D_A(orc_plan *p, const R *fhat)
{
  INT kL;
  memset(p->g, 0, sizeof(R) * 2 * (size_t)p->n_total);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (kL = 0; kL < p->N_total; kL++) {
    R c;
    INT pos = grid_pos_of_freq(p, kL, &c);
    p->g[2 * pos] = fhat[2 * kL] * c;
    p->g[2 * pos + 1] = fhat[2 * kL + 1] * c;
  }
}

static void D_T(orc_plan *p, R *fhat)
{
  INT kL;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (kL = 0; kL < p->N_total; kL++) {
    R c;
    INT pos = grid_pos_of_freq(p, kL, &c);
    fhat[2 * kL] = p->g[2 * pos] * c;
    fhat[2 * kL + 1] = p->g[2 * pos + 1] * c;
  }
}

/* ------------------------------------------------------------------------- */
/* B: f_j = sum_{l in [u,u+2m+1]^d} prod_t psi_t(l_t) g[l mod n]             */
/* (nfft_trafo_2d_compute nfft.c:2927-3004, 3-D nfft.c:4020-4265, generic    */
/* B_openmp_A nfft.c:1172-1278).  Nodes run in sorted order when the sort is */
/* on (nfft_trafo_2d_B nfft.c:3221-3410).                                    */
/* ------------------------------------------------------------------------- */
/* per node: window values ps[t] and wrapped grid indices idx[t][l] */
static void node_taps(const orc_plan *p, INT j, const R **ps, INT (*idx)[64], R *scratch)
{
  const int w = 2 * p->m + 2;
  int t, l;
  for (t = 0; t < p->d; t++) {
    const INT u = node_u(p, j, t), n = p->n[t];
    ps[t] = psi_of(p, j, t, scratch + 64 * t);
    for (l = 0; l < w; l++) idx[t][l] = (((u + l) % n) + n) % n;
  }
}

static void B_A(orc_plan *p, R *f)
{
  const int d = p->d, w = 2 * p->m + 2;
  INT jj;
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    R scratch[8 * 64];
    INT idx[8][64];
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (jj = 0; jj < p->M; jj++) {
      const INT j = p->index_x ? p->index_x[2 * jj + 1] : jj;
      const R *ps[8];
      R sr = 0, si = 0;
      int l0, l1, l2;
      node_taps(p, j, ps, idx, scratch);
      if (d == 1) {
        for (l0 = 0; l0 < w; l0++) {
          const R *gv = p->g + 2 * idx[0][l0];
          sr += ps[0][l0] * gv[0];
          si += ps[0][l0] * gv[1];
        }
      } else if (d == 2) {
        const INT n1 = p->n[1];
        for (l0 = 0; l0 < w; l0++) {
          const R *g0 = p->g + 2 * idx[0][l0] * n1;
          R tr = 0, ti = 0;
          for (l1 = 0; l1 < w; l1++) {
            const R *gv = g0 + 2 * idx[1][l1];
            tr += ps[1][l1] * gv[0];
            ti += ps[1][l1] * gv[1];
          }
          sr += ps[0][l0] * tr;
          si += ps[0][l0] * ti;
        }
      } else if (d == 3) {
        const INT n1 = p->n[1], n2 = p->n[2];
        for (l0 = 0; l0 < w; l0++) {
          const R *g0 = p->g + 2 * idx[0][l0] * n1 * n2;
          R ur = 0, ui = 0;
          for (l1 = 0; l1 < w; l1++) {
            const R *g01 = g0 + 2 * idx[1][l1] * n2;
            R tr = 0, ti = 0;
            for (l2 = 0; l2 < w; l2++) {
              const R *gv = g01 + 2 * idx[2][l2];
              tr += ps[2][l2] * gv[0];
              ti += ps[2][l2] * gv[1];
            }
            ur += ps[1][l1] * tr;
            ui += ps[1][l1] * ti;
          }
          sr += ps[0][l0] * ur;
          si += ps[0][l0] * ui;
        }
      } else {
        /* odometer over the w^d tensor product, last dim fastest */
        INT l[8];
        int t;
        for (t = 0; t < d; t++) l[t] = 0;
        for (;;) {
          INT pos = 0;
          R wgt = (R)1.0;
          for (t = 0; t < d; t++) {
            pos = pos * p->n[t] + idx[t][l[t]];
            wgt *= ps[t][l[t]];
          }
          sr += wgt * p->g[2 * pos];
          si += wgt * p->g[2 * pos + 1];
          for (t = d - 1; t >= 0; t--) {
            if (++l[t] < w) break;
            l[t] = 0;
          }
          if (t < 0) break;
        }
      }
      f[2 * j] = sr; f[2 * j + 1] = si;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* B^T: g[l mod n] += prod_t psi_t(l_t) f_j  (nfft_adjoint_2d_compute_serial */
/* nfft.c:3143-3218).  With ORC_BLOCKWISE the dim-0 rows are split into one  */
/* slab per OpenMP thread and every thread scans the nodes whose window can  */
/* touch its slab, writing only its own rows -- the reference's blockwise    */
/* adjoint (nfft_adjoint_B_omp_blockwise_init nfft.c:1345-1420,              */
/* nfft_adjoint_2d_compute_omp_blockwise nfft.c:3064-3139).                  */
/* ------------------------------------------------------------------------- */
static void spread_node(orc_plan *p, INT j, const R *f, INT row_lo, INT row_hi,
                        R *scratch)
{
  const int d = p->d, w = 2 * p->m + 2;
  const R *ps[8];
  INT idx[8][64];
  const R fr = f[2 * j], fi = f[2 * j + 1];
  int l0, l1, l2;
  node_taps(p, j, ps, idx, scratch);
  if (d == 1) {
    for (l0 = 0; l0 < w; l0++) {
      R *gv;
      if (idx[0][l0] < row_lo || idx[0][l0] >= row_hi) continue;
      gv = p->g + 2 * idx[0][l0];
      gv[0] += ps[0][l0] * fr;
      gv[1] += ps[0][l0] * fi;
    }
  } else if (d == 2) {
    const INT n1 = p->n[1];
    for (l0 = 0; l0 < w; l0++) {
      R *g0;
      R wr, wi;
      if (idx[0][l0] < row_lo || idx[0][l0] >= row_hi) continue;
      g0 = p->g + 2 * idx[0][l0] * n1;
      wr = ps[0][l0] * fr;
      wi = ps[0][l0] * fi;
      for (l1 = 0; l1 < w; l1++) {
        R *gv = g0 + 2 * idx[1][l1];
        gv[0] += ps[1][l1] * wr;
        gv[1] += ps[1][l1] * wi;
      }
    }
  } else if (d == 3) {
    const INT n1 = p->n[1], n2 = p->n[2];
    for (l0 = 0; l0 < w; l0++) {
      R *g0;
      if (idx[0][l0] < row_lo || idx[0][l0] >= row_hi) continue;
      g0 = p->g + 2 * idx[0][l0] * n1 * n2;
      for (l1 = 0; l1 < w; l1++) {
        R *g01 = g0 + 2 * idx[1][l1] * n2;
        const R w01 = ps[0][l0] * ps[1][l1];
        const R wr = w01 * fr, wi = w01 * fi;
        for (l2 = 0; l2 < w; l2++) {
          R *gv = g01 + 2 * idx[2][l2];
          gv[0] += ps[2][l2] * wr;
          gv[1] += ps[2][l2] * wi;
        }
      }
    }
  } else {
    INT l[8];
    int t;
    for (t = 0; t < d; t++) l[t] = 0;
    for (;;) {
      if (idx[0][l[0]] >= row_lo && idx[0][l[0]] < row_hi) {
        INT pos = 0;
        R wgt = (R)1.0;
        for (t = 0; t < d; t++) {
          pos = pos * p->n[t] + idx[t][l[t]];
          wgt *= ps[t][l[t]];
        }
        p->g[2 * pos] += wgt * fr;
        p->g[2 * pos + 1] += wgt * fi;
      }
      for (t = d - 1; t >= 0; t--) {
        if (++l[t] < w) break;
        l[t] = 0;
      }
      if (t < 0) break;
    }
  }
}

/* first sorted position whose key is >= key (index_x is sorted by key) */
static INT lower_bound_key(const INT *ar, INT M, INT key)
{
  INT lo = 0, hi = M;
  while (lo < hi) {
    INT mid = lo + (hi - lo) / 2;
    if (ar[2 * mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

static void B_T(orc_plan *p, const R *f)
{
  memset(p->g, 0, sizeof(R) * 2 * (size_t)p->n_total);
#ifdef _OPENMP
  if ((p->flags & ORC_BLOCKWISE) && p->index_x && omp_get_max_threads() > 1) {
#pragma omp parallel
    {
      const INT nth = omp_get_num_threads(), id = omp_get_thread_num();
      const INT n0 = p->n[0], rest = p->n_total / n0;
      const INT lo = n0 * id / nth, hi = n0 * (id + 1) / nth;
      R scratch[8 * 64];
      /* A node's window covers dim-0 rows u0..u0+2m+1 (mod n0).  Its sort
       * key's leading digit is the wrapped window start, which can differ
       * from u0 by one through rounding, so the candidate key rows are
       * [lo-2m-2, hi+1) taken mod n0; spread_node keeps only the rows of
       * this thread's slab [lo, hi). */
      INT r0 = lo - 2 * p->m - 2, r1 = hi + 1, r;
      if (r1 - r0 >= n0) { r0 = 0; r1 = n0; }
      for (r = r0; r < r1;) {
        INT rw = ((r % n0) + n0) % n0;
        INT run = r1 - r;
        INT a, b, jj;
        if (rw + run > n0) run = n0 - rw;
        a = lower_bound_key(p->index_x, p->M, rw * rest);
        b = lower_bound_key(p->index_x, p->M, (rw + run) * rest);
        for (jj = a; jj < b; jj++)
          spread_node(p, p->index_x[2 * jj + 1], f, lo, hi, scratch);
        r += run;
      }
    }
    return;
  }
#endif
  {
    INT jj;
    R scratch[8 * 64];
    for (jj = 0; jj < p->M; jj++) {
      const INT j = p->index_x ? p->index_x[2 * jj + 1] : jj;
      spread_node(p, j, f, 0, p->n[0], scratch);
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Transforms: nfft_trafo = D -> FFT(forward) -> B, nfft_adjoint =           */
/* B^T -> FFT(backward) -> D^T (nfft.c:5655-5749).  The reference switches to */
/* the NDFT when some N_t <= m or n_t <= 2m+2 (nfft.c:5658-5665).            */
/* ------------------------------------------------------------------------- */
static int use_direct(const orc_plan *p)
{
  int t;
  for (t = 0; t < p->d; t++)
    if (p->N[t] <= p->m || p->n[t] <= 2 * p->m + 2) return 1;
  return 0;
}

void P(trafo)(orc_plan *p, const R *fhat, R *f)
{
  double t0, t1, t2, t3;
  if (use_direct(p)) { P(trafo_direct)(p, fhat, f); return; }
  t0 = now_s();
  D_A(p, fhat);
  t1 = now_s();
  P(fft)(p->d, p->n, p->g, -1);
  t2 = now_s();
  B_A(p, f);
  t3 = now_s();
  p->t_stage[0] = t1 - t0; p->t_stage[1] = t2 - t1; p->t_stage[2] = t3 - t2;
}

void P(adjoint)(orc_plan *p, const R *f, R *fhat)
{
  double t0, t1, t2, t3;
  if (use_direct(p)) { P(adjoint_direct)(p, f, fhat); return; }
  t0 = now_s();
  B_T(p, f);
  t1 = now_s();
  P(fft)(p->d, p->n, p->g, +1);
  t2 = now_s();
  D_T(p, fhat);
  t3 = now_s();
  p->t_stage[2] = t1 - t0; p->t_stage[1] = t2 - t1; p->t_stage[0] = t3 - t2;
}

/* ------------------------------------------------------------------------- */
/* Inverse NFFT solver: CGNR and CGNE on the plan, restating                 */
/* kernel/solver/solver.c (init_advanced_complex 40-74, before_loop_complex  */
/* 81-125, CGNR step 232-292, CGNE step 295-344) with the BLAS-1 helpers of  */
/* kernel/util/vector1.c:22-57, vector2.c:22-74, vector3.c:22-93.  Dots are  */
/* accumulated in R like the reference.                                      */
/* ------------------------------------------------------------------------- */
#define ORC_CGNR 4u
#define ORC_CGNE 8u
#define ORC_PRECOMPUTE_WEIGHT 32u
#define ORC_PRECOMPUTE_DAMP 64u

typedef struct {
  orc_plan *p;
  unsigned flags;
  R *w, *w_hat, *y, *f_hat_iter, *r_iter, *z_hat_iter, *p_hat_iter, *v_iter;
  R *mv_f, *mv_f_hat; /* the plan's f and f_hat vectors */
  R alpha_iter, beta_iter, dot_r_iter, dot_r_iter_old, dot_z_hat_iter,
    dot_z_hat_iter_old, dot_p_hat_iter, dot_v_iter;
} orc_solver;

static R dot_c(const R *x, INT n)
{
  R s = 0; INT k;
  for (k = 0; k < n; k++) s += x[2 * k] * x[2 * k] + x[2 * k + 1] * x[2 * k + 1];
  return s;
}
static R dot_wc(const R *x, const R *w, INT n)
{
  R s = 0; INT k;
  for (k = 0; k < n; k++) s += w[k] * (x[2 * k] * x[2 * k] + x[2 * k + 1] * x[2 * k + 1]);
  return s;
}
static void cp_c(R *x, const R *y, INT n) { memcpy(x, y, sizeof(R) * 2 * (size_t)n); }
static void cp_wc(R *x, const R *w, const R *y, INT n)
{
  INT k;
  for (k = 0; k < n; k++) { x[2 * k] = w[k] * y[2 * k]; x[2 * k + 1] = w[k] * y[2 * k + 1]; }
}
/* x <- x + a y */
static void xpay(R *x, R a, const R *y, INT n)
{
  INT k;
  for (k = 0; k < 2 * n; k++) x[k] += a * y[k];
}
/* x <- x + a w y */
static void xpawy(R *x, R a, const R *w, const R *y, INT n)
{
  INT k;
  for (k = 0; k < n; k++) { x[2 * k] += a * w[k] * y[2 * k]; x[2 * k + 1] += a * w[k] * y[2 * k + 1]; }
}
/* x <- a x + y */
static void axpy(R *x, R a, const R *y, INT n)
{
  INT k;
  for (k = 0; k < 2 * n; k++) x[k] = a * x[k] + y[k];
}

orc_solver *P(solver_create)(orc_plan *p, unsigned flags)
{
  orc_solver *s = (orc_solver*)calloc(1, sizeof(orc_solver));
  const size_t M = (size_t)p->M, N = (size_t)p->N_total;
  s->p = p; s->flags = flags;
  s->y = (R*)calloc(2 * M, sizeof(R));
  s->r_iter = (R*)calloc(2 * M, sizeof(R));
  s->f_hat_iter = (R*)calloc(2 * N, sizeof(R));
  s->p_hat_iter = (R*)calloc(2 * N, sizeof(R));
  if (flags & ORC_CGNR) {
    s->z_hat_iter = (R*)calloc(2 * N, sizeof(R));
    s->v_iter = (R*)calloc(2 * M, sizeof(R));
  } else {
    s->z_hat_iter = s->p_hat_iter;
  }
  if (flags & ORC_PRECOMPUTE_WEIGHT) s->w = (R*)calloc(M, sizeof(R));
  if (flags & ORC_PRECOMPUTE_DAMP) s->w_hat = (R*)calloc(N, sizeof(R));
  s->mv_f = (R*)calloc(2 * M, sizeof(R));
  s->mv_f_hat = (R*)calloc(2 * N, sizeof(R));
  return s;
}

void P(solver_destroy)(orc_solver *s)
{
  if (!s) return;
  free(s->y); free(s->r_iter); free(s->f_hat_iter); free(s->p_hat_iter);
  if (s->flags & ORC_CGNR) { free(s->z_hat_iter); free(s->v_iter); }
  free(s->w); free(s->w_hat); free(s->mv_f); free(s->mv_f_hat);
  free(s);
}

void P(solver_set)(orc_solver *s, const R *y, const R *w, const R *w_hat,
                   const R *f_hat_iter)
{
  const size_t M = (size_t)s->p->M, N = (size_t)s->p->N_total;
  if (y) memcpy(s->y, y, sizeof(R) * 2 * M);
  if (w && s->w) memcpy(s->w, w, sizeof(R) * M);
  if (w_hat && s->w_hat) memcpy(s->w_hat, w_hat, sizeof(R) * N);
  if (f_hat_iter) memcpy(s->f_hat_iter, f_hat_iter, sizeof(R) * 2 * N);
}

void P(solver_before_loop)(orc_solver *s)
{
  orc_plan *p = s->p;
  const INT M = p->M, N = p->N_total;
  cp_c(s->mv_f_hat, s->f_hat_iter, N);
  P(trafo)(p, s->mv_f_hat, s->r_iter);          /* r = A f^ (swap into mv.f) */
  axpy(s->r_iter, (R)-1.0, s->y, M);            /* r = -r + y */
  s->dot_r_iter = (s->flags & ORC_PRECOMPUTE_WEIGHT) ? dot_wc(s->r_iter, s->w, M)
                                                     : dot_c(s->r_iter, M);
  if (s->flags & ORC_PRECOMPUTE_WEIGHT) cp_wc(s->mv_f, s->w, s->r_iter, M);
  else cp_c(s->mv_f, s->r_iter, M);
  P(adjoint)(p, s->mv_f, s->z_hat_iter);        /* z = A^H W r */
  s->dot_z_hat_iter = (s->flags & ORC_PRECOMPUTE_DAMP)
                          ? dot_wc(s->z_hat_iter, s->w_hat, N)
                          : dot_c(s->z_hat_iter, N);
  if (s->flags & ORC_CGNE) s->dot_p_hat_iter = s->dot_z_hat_iter;
  if (s->flags & ORC_CGNR) cp_c(s->p_hat_iter, s->z_hat_iter, N);
}

static void cgnr_step(orc_solver *s)
{
  orc_plan *p = s->p;
  const INT M = p->M, N = p->N_total;
  if (s->flags & ORC_PRECOMPUTE_DAMP) cp_wc(s->mv_f_hat, s->w_hat, s->p_hat_iter, N);
  else cp_c(s->mv_f_hat, s->p_hat_iter, N);
  P(trafo)(p, s->mv_f_hat, s->v_iter);
  s->dot_v_iter = (s->flags & ORC_PRECOMPUTE_WEIGHT) ? dot_wc(s->v_iter, s->w, M)
                                                     : dot_c(s->v_iter, M);
  s->alpha_iter = s->dot_z_hat_iter / s->dot_v_iter;
  if (s->flags & ORC_PRECOMPUTE_DAMP)
    xpawy(s->f_hat_iter, s->alpha_iter, s->w_hat, s->p_hat_iter, N);
  else
    xpay(s->f_hat_iter, s->alpha_iter, s->p_hat_iter, N);
  xpay(s->r_iter, -s->alpha_iter, s->v_iter, M);
  s->dot_r_iter = (s->flags & ORC_PRECOMPUTE_WEIGHT) ? dot_wc(s->r_iter, s->w, M)
                                                     : dot_c(s->r_iter, M);
  if (s->flags & ORC_PRECOMPUTE_WEIGHT) cp_wc(s->mv_f, s->w, s->r_iter, M);
  else cp_c(s->mv_f, s->r_iter, M);
  P(adjoint)(p, s->mv_f, s->z_hat_iter);
  s->dot_z_hat_iter_old = s->dot_z_hat_iter;
  s->dot_z_hat_iter = (s->flags & ORC_PRECOMPUTE_DAMP)
                          ? dot_wc(s->z_hat_iter, s->w_hat, N)
                          : dot_c(s->z_hat_iter, N);
  s->beta_iter = s->dot_z_hat_iter / s->dot_z_hat_iter_old;
  axpy(s->p_hat_iter, s->beta_iter, s->z_hat_iter, N);
}

static void cgne_step(orc_solver *s)
{
  orc_plan *p = s->p;
  const INT M = p->M, N = p->N_total;
  s->alpha_iter = s->dot_r_iter / s->dot_p_hat_iter;
  if (s->flags & ORC_PRECOMPUTE_DAMP)
    xpawy(s->f_hat_iter, s->alpha_iter, s->w_hat, s->p_hat_iter, N);
  else
    xpay(s->f_hat_iter, s->alpha_iter, s->p_hat_iter, N);
  if (s->flags & ORC_PRECOMPUTE_DAMP) cp_wc(s->mv_f_hat, s->w_hat, s->p_hat_iter, N);
  else cp_c(s->mv_f_hat, s->p_hat_iter, N);
  P(trafo)(p, s->mv_f_hat, s->mv_f);
  xpay(s->r_iter, -s->alpha_iter, s->mv_f, M);
  s->dot_r_iter_old = s->dot_r_iter;
  s->dot_r_iter = (s->flags & ORC_PRECOMPUTE_WEIGHT) ? dot_wc(s->r_iter, s->w, M)
                                                     : dot_c(s->r_iter, M);
  s->beta_iter = s->dot_r_iter / s->dot_r_iter_old;
  if (s->flags & ORC_PRECOMPUTE_WEIGHT) cp_wc(s->mv_f, s->w, s->r_iter, M);
  else cp_c(s->mv_f, s->r_iter, M);
  P(adjoint)(p, s->mv_f, s->mv_f_hat);
  axpy(s->p_hat_iter, s->beta_iter, s->mv_f_hat, N);
  s->dot_p_hat_iter = (s->flags & ORC_PRECOMPUTE_DAMP)
                          ? dot_wc(s->p_hat_iter, s->w_hat, N)
                          : dot_c(s->p_hat_iter, N);
}

void P(solver_step)(orc_solver *s)
{
  if (s->flags & ORC_CGNR) cgnr_step(s);
  if (s->flags & ORC_CGNE) cgne_step(s);
}

/* scalars: alpha, beta, dot_r, dot_r_old, dot_z, dot_z_old, dot_p, dot_v */
void P(solver_get)(const orc_solver *s, R *f_hat_iter, R *r_iter, double *sc)
{
  if (f_hat_iter) memcpy(f_hat_iter, s->f_hat_iter, sizeof(R) * 2 * (size_t)s->p->N_total);
  if (r_iter) memcpy(r_iter, s->r_iter, sizeof(R) * 2 * (size_t)s->p->M);
  if (sc) {
    sc[0] = s->alpha_iter; sc[1] = s->beta_iter; sc[2] = s->dot_r_iter;
    sc[3] = s->dot_r_iter_old; sc[4] = s->dot_z_hat_iter;
    sc[5] = s->dot_z_hat_iter_old; sc[6] = s->dot_p_hat_iter; sc[7] = s->dot_v_iter;
  }
}
