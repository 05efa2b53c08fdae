// gb_window.cpp -- per-tap polynomial form of the Kaiser-Bessel window for the
// single-precision 2-D / 3-D kernels and the double-precision 2-D kernels.
//
// The window (reference include/infft.h:209-215, with b = pi (2 - 1/sigma)
// from include/infft.h:216-222) is evaluated at t = n x - (u + l) for the W
// taps l of a node, where u = floor(n x) - m.  With s = 2 (n x - floor(n x)) - 1
// in [-1, 1) the argument of tap l is t = (s + 1)/2 + m - l, so each tap is a
// smooth function of s alone: phi_l(s) = phi((s + 1)/2 + m - l).  It is
// interpolated here, in double precision, at the KB_POLY_DP Chebyshev points
// of [-1, 1] by a polynomial of degree KB_POLY_DP - 1 in s; the kernels
// evaluate it by Horner's rule in single precision (KB_POLY_DP - 1 FMAs per
// tap, no transcendental functions).  Degree 9 keeps the interpolation error
// below 1e-9 of the window's peak for 2 <= m <= 8, far below single
// precision; the FP32 Horner evaluation itself is within 1e-7 of the peak.
#include <cmath>

#include "gb_common.cuh"

namespace gb {

static double kb_phi_host(double t, int m, double b)
{
  const double a = (double)m * m - t * t;
  if (a > 0) {
    const double s = std::sqrt(a);
    return std::sinh(b * s) / (M_PI * s);
  }
  if (a < 0) {
    const double s = std::sqrt(-a);
    return std::sin(b * s) / (M_PI * s);
  }
  return b / M_PI;
}

// Solves V c = y for the monomial coefficients c of the interpolant through
// (xk, yk) by Gaussian elimination with partial pivoting (n <= 16).
static void solve_vandermonde(const double *xk, const double *yk, int n, double *c)
{
  double A[16][17];
  for (int i = 0; i < n; ++i) {
    double p = 1.0;
    for (int j = 0; j < n; ++j) {
      A[i][j] = p;
      p *= xk[i];
    }
    A[i][n] = yk[i];
  }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
    if (piv != col)
      for (int j = 0; j <= n; ++j) std::swap(A[piv][j], A[col][j]);
    for (int r = col + 1; r < n; ++r) {
      const double f = A[r][col] / A[col][col];
      for (int j = col; j <= n; ++j) A[r][j] -= f * A[col][j];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = A[i][n];
    for (int j = i + 1; j < n; ++j) s -= A[i][j] * c[j];
    c[i] = s / A[i][i];
  }
}

void kb_poly_fit(int m, double b, int w, float *coef)
{
  const int n = KB_POLY_DP;
  double xk[KB_POLY_DP], yk[KB_POLY_DP], c[KB_POLY_DP];
  for (int k = 0; k < n; ++k) xk[k] = std::cos(M_PI * (k + 0.5) / n);
  for (int l = 0; l < w; ++l) {
    for (int k = 0; k < n; ++k) yk[k] = kb_phi_host(0.5 * (xk[k] + 1.0) + m - l, m, b);
    solve_vandermonde(xk, yk, n, c);
    for (int k = 0; k < n; ++k) coef[l * n + k] = (float)c[k];
  }
}

// Double-precision form: the tap functions are sampled in extended precision
// (long double) at the KB_POLYD_DP Chebyshev points of [-1, 1], their
// Chebyshev coefficients taken by the discrete cosine sums, converted to
// monomial coefficients by the three-term recurrence T_{k+1} = 2 s T_k -
// T_{k-1}, all in long double, and rounded to double once.
static long double kb_phi_ext(long double t, int m, long double b)
{
  const long double a = (long double)m * m - t * t;
  const long double pi = 3.141592653589793238462643383279502884L;
  if (a > 0) {
    const long double s = sqrtl(a);
    return sinhl(b * s) / (pi * s);
  }
  if (a < 0) {
    const long double s = sqrtl(-a);
    return sinl(b * s) / (pi * s);
  }
  return b / pi;
}

void kb_polyd_fit(int m, double b, int w, double *coef)
{
  const int n = KB_POLYD_DP;
  const long double pi = 3.141592653589793238462643383279502884L;
  long double xk[KB_POLYD_DP], yk[KB_POLYD_DP], ch[KB_POLYD_DP];
  long double tprev[KB_POLYD_DP], tcur[KB_POLYD_DP], tnext[KB_POLYD_DP], mono[KB_POLYD_DP];
  for (int k = 0; k < n; ++k) xk[k] = cosl(pi * (k + 0.5L) / n);
  for (int l = 0; l < w; ++l) {
    for (int k = 0; k < n; ++k) yk[k] = kb_phi_ext(0.5L * (xk[k] + 1.0L) + m - l, m, (long double)b);
    for (int j = 0; j < n; ++j) {
      long double s = 0;
      for (int k = 0; k < n; ++k) s += yk[k] * cosl(pi * j * (k + 0.5L) / n);
      ch[j] = s * (j == 0 ? 1.0L : 2.0L) / n;
    }
    for (int k = 0; k < n; ++k) tprev[k] = tcur[k] = mono[k] = 0;
    tprev[0] = 1;  // T_0
    tcur[1] = 1;   // T_1
    mono[0] = ch[0];
    for (int k = 0; k < n; ++k) mono[k] += ch[1] * tcur[k];
    for (int j = 2; j < n; ++j) {
      for (int k = 0; k < n; ++k) tnext[k] = (k > 0 ? 2 * tcur[k - 1] : 0) - tprev[k];
      for (int k = 0; k < n; ++k) {
        mono[k] += ch[j] * tnext[k];
        tprev[k] = tcur[k];
        tcur[k] = tnext[k];
      }
    }
    for (int k = 0; k < n; ++k) coef[l * n + k] = (double)mono[k];
  }
}

}  // namespace gb

extern "C" void nfft_gb_kb_poly_fit(int m, double b, int w, float *coef) { gb::kb_poly_fit(m, b, w, coef); }
extern "C" void nfft_gb_kb_polyd_fit(int m, double b, int w, double *coef) { gb::kb_polyd_fit(m, b, w, coef); }
