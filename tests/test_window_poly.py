"""The polynomial window of the single-precision 2-D and 3-D kernels, checked on the
CPU against the Kaiser-Bessel window of the reference (include/infft.h:209-222):
phi(t) = sinh(b sqrt(m^2 - t^2)) / (pi sqrt(m^2 - t^2)) inside the support,
sin(b sqrt(t^2 - m^2)) / (pi sqrt(t^2 - m^2)) outside, b / pi on its edge,
with t = n x - (u + l) and b = pi (2 - 1 / sigma)."""
import ctypes as C

import numpy as np
import pytest

import nfft_gb300


def kb_phi(t, m, b):
    t = np.asarray(t, dtype=np.float64)
    a = m * m - t * t
    out = np.full_like(t, b / np.pi)
    pos, neg = a > 0, a < 0
    s = np.sqrt(a[pos])
    out[pos] = np.sinh(b * s) / (np.pi * s)
    s = np.sqrt(-a[neg])
    out[neg] = np.sin(b * s) / (np.pi * s)
    return out


def horner_f32(c, s):
    """Single-precision Horner evaluation, one rounding per multiply-add as the
    kernels' fused multiply-adds (computed in double, rounded to float)."""
    s64 = s.astype(np.float32).astype(np.float64)
    v = np.full(s.shape, np.float32(c[-1]), dtype=np.float32)
    for k in range(len(c) - 2, -1, -1):
        v = (v.astype(np.float64) * s64 + np.float64(np.float32(c[k]))).astype(np.float32)
    return v.astype(np.float64)


@pytest.mark.parametrize("m,sigma", [(2, 2.0), (3, 2.0), (4, 2.0), (4, 1.5), (4, 1.25), (3, 1.25), (5, 2.0), (6, 2.0),
                                     (7, 2.0), (6, 1.5)])
def test_polynomial_window_matches_kaiser_bessel(m, sigma):
    lib = nfft_gb300.lib()
    fit = lib.nfft_gb_kb_poly_fit
    fit.restype = None
    fit.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_float)]
    w = 2 * m + 2
    b = float(np.float32(np.pi * (2.0 - 1.0 / sigma)))  # the plan keeps b in its precision
    coef = (C.c_float * (w * 10))()
    fit(m, b, w, coef)
    c = np.ctypeslib.as_array(coef).reshape(w, 10)
    rng = np.random.default_rng(m)
    frac = np.concatenate([rng.uniform(0, 1, 2000), [0.0, 0.5, 1.0 - 2.0 ** -24]])
    s = 2.0 * frac - 1.0
    peak = kb_phi(np.array([0.0]), m, b)[0]
    worst = 0.0
    for l in range(w):
        exact = kb_phi(frac + m - l, m, b)
        worst = max(worst, np.max(np.abs(horner_f32(c[l], s) - exact)) / peak)
    # single-precision rounding of the window's peak is 6e-8 of it
    assert worst < 2e-7, worst


def sym_f32(c, s):
    """The symmetric evaluation of the 3-D kernels (kb_poly_taps_sym): t = s^2
    rounded, E and O by single-precision Horner in t, then E + s O (tap l) and
    E - s O (tap w-1-l), each multiply-add rounded once."""
    f32 = np.float32
    s32 = s.astype(f32).astype(np.float64)
    t = (s32 * s32).astype(f32).astype(np.float64)
    e = np.full(s.shape, f32(c[8]), dtype=f32)
    o = np.full(s.shape, f32(c[9]), dtype=f32)
    for k in (6, 4, 2, 0):
        e = (e.astype(np.float64) * t + np.float64(f32(c[k]))).astype(f32)
        o = (o.astype(np.float64) * t + np.float64(f32(c[k + 1]))).astype(f32)
    lo = (s32 * o.astype(np.float64) + e.astype(np.float64)).astype(f32)
    hi = (-s32 * o.astype(np.float64) + e.astype(np.float64)).astype(f32)
    return lo.astype(np.float64), hi.astype(np.float64)


@pytest.mark.parametrize("m,sigma", [(2, 2.0), (3, 2.0), (4, 2.0), (4, 1.5), (5, 2.0), (6, 2.0), (7, 2.0)])
def test_symmetric_window_evaluation_matches_kaiser_bessel(m, sigma):
    """Taps l and w-1-l from tap l's even and odd parts at s and -s."""
    lib = nfft_gb300.lib()
    fit = lib.nfft_gb_kb_poly_fit
    fit.restype = None
    fit.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_float)]
    w = 2 * m + 2
    b = float(np.float32(np.pi * (2.0 - 1.0 / sigma)))
    coef = (C.c_float * (w * 10))()
    fit(m, b, w, coef)
    c = np.ctypeslib.as_array(coef).reshape(w, 10)
    rng = np.random.default_rng(10 + m)
    frac = np.concatenate([rng.uniform(0, 1, 2000), [0.0, 0.5, 1.0 - 2.0 ** -24]])
    s = 2.0 * frac - 1.0
    peak = kb_phi(np.array([0.0]), m, b)[0]
    worst = 0.0
    for l in range(w // 2):
        lo, hi = sym_f32(c[l], s)
        worst = max(worst, np.max(np.abs(lo - kb_phi(frac + m - l, m, b))) / peak)
        worst = max(worst, np.max(np.abs(hi - kb_phi(frac + m - (w - 1 - l), m, b))) / peak)
    assert worst < 2e-7, worst


@pytest.mark.parametrize("m,sigma", [(2, 2.0), (4, 2.0), (5, 1.5), (6, 2.0), (7, 2.0), (6, 1.25)])
def test_double_polynomial_window_matches_kaiser_bessel(m, sigma):
    """The degree-16 form of the double-precision 2-D kernels: Horner in
    double precision within 1e-14 of the window's peak (the kernels' taps
    then agree with the exact window to the last few digits)."""
    lib = nfft_gb300.lib()
    fit = lib.nfft_gb_kb_polyd_fit
    fit.restype = None
    fit.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double)]
    w = 2 * m + 2
    b = np.pi * (2.0 - 1.0 / sigma)
    coef = (C.c_double * (w * 17))()
    fit(m, b, w, coef)
    c = np.ctypeslib.as_array(coef).reshape(w, 17)
    rng = np.random.default_rng(m)
    frac = np.concatenate([rng.uniform(0, 1, 4000), [0.0, 0.5, 1.0 - 2.0 ** -52]])
    s = 2.0 * frac - 1.0
    peak = kb_phi(np.array([0.0]), m, b)[0]
    worst = 0.0
    for l in range(w):
        v = np.zeros_like(s)
        for a in c[l][::-1]:
            v = v * s + a
        worst = max(worst, np.max(np.abs(v - kb_phi(frac + m - l, m, b))) / peak)
    assert worst < 1e-14, worst
