"""Compensated single-precision 2-D adjoint (nfftf_gb_set_compensated).

Where many nodes crowd into few cells -- the centre of radial and spiral
k-space trajectories -- each cell of the oversampled grid sums thousands of
single-precision terms.  The compensated form keeps their rounding errors
(error-free sums) and folds them back in; its error against the FP64 NDFT
(nfft_adjoint_direct, reference nfft.c:207-297) must not exceed the plain
form's, and both must stay within the reference tests' bound
(tests/nfft.c:217-284).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import compare_adjoint, err_trafo_bound
from nfft_gb300 import abi
from nfft_gb300.plan import Plan

pytestmark = pytest.mark.gpu

FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.FFTW_INIT
         | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)


def _adjoint(lib, x, f, N, m, mode):
    p = Plan(lib, True, N, len(x), n=[2 * v for v in N], m=m, flags=FLAGS)
    fn = lib.nfftf_gb_set_compensated
    fn.argtypes = [C.c_void_p, C.c_int]
    fn.restype = C.c_int
    assert fn(C.addressof(p.p), mode) == 0
    p.x[:] = x
    p.precompute_one_psi()
    p.f[:] = f
    p.adjoint()
    out = p.f_hat.astype(np.complex128)
    p.finalize()
    return out


def _ndft_adjoint(lib, x, f, N, m):
    q = Plan(lib, False, N, len(x), n=[2 * v for v in N], m=m, flags=FLAGS)
    q.x[:] = x.astype(np.float64)
    q.f[:] = f.astype(np.complex128)
    q.adjoint_direct()
    out = q.f_hat.copy()
    q.finalize()
    return out


@pytest.mark.parametrize("m", [6, 7])
def test_compensated_adjoint_error_at_or_below_plain(gpulib, m):
    N, M = [64, 64], 200000
    rng = np.random.default_rng(11)
    # one dense blob: some 10^4 nodes per oversampled cell near its centre
    x = (0.01 * rng.standard_normal((M, 2))).astype(np.float32)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    ref = _ndft_adjoint(gpulib, x, f, N, m)
    plain = _adjoint(gpulib, x, f, N, m, 0)
    comp = _adjoint(gpulib, x, f, N, m, 1)
    e_plain = np.linalg.norm(plain - ref) / np.linalg.norm(ref)
    e_comp = np.linalg.norm(comp - ref) / np.linalg.norm(ref)
    print("m=%d: relative l2 vs FP64 NDFT, plain %.3e, compensated %.3e" % (m, e_plain, e_comp))
    assert e_comp <= e_plain, (e_comp, e_plain)
    bound = err_trafo_bound(m, True)
    assert compare_adjoint(comp, ref, f.astype(np.complex128)) < bound


def test_compensated_mode_only_where_it_applies(gpulib):
    fn = gpulib.nfftf_gb_set_compensated
    fn.argtypes = [C.c_void_p, C.c_int]
    fn.restype = C.c_int
    p = Plan(gpulib, True, [16, 16, 16], 100, n=[32, 32, 32], m=4, flags=FLAGS)
    assert fn(C.addressof(p.p), 1) == -1  # 3-D: no such kernel
    p.finalize()
    q = Plan(gpulib, True, [32, 32], 100, n=[64, 64], m=6, flags=FLAGS)
    assert fn(C.addressof(q.p), 2) == -1  # not a mode
    assert fn(C.addressof(q.p), -1) == 0
    q.finalize()
