"""Mixed-precision inverse NFFT (CGNR) on radial k-space, GPU.

FP32 transforms with FP64 inner products and an FP64 residual refresh must
reach 1e-5 relative distance to the converged FP64 CGNR solution of the same
normal equations (the FP64 solution is the reference; the reference library's
solver loop is kernel/solver/solver.c:232-292).
"""
import numpy as np
import pytest

from nfft_gb300 import infft, workloads
from nfft_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def _problem(lib, N=64, spokes=100, samples=128, m=6):
    x = workloads.radial_nodes(spokes, samples)
    f_true = workloads.ellipse_phantom(N, 20, seed=1)
    p = Plan(lib, False, [N, N], len(x), n=[2 * N, 2 * N], m=m, flags=infft.PLAN_FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = f_true
    p.trafo()
    y = workloads.add_noise(p.f.copy(), 40.0, np.random.default_rng(1))
    p.finalize()
    return [N, N], x, m, y, f_true


def test_mixed_precision_cgnr_tracks_fp64(gpulib):
    """After K iterations the FP32 solver with FP64 dots and an FP64 residual
    refresh stays close to the FP64 solver's iterate, and both approach the
    phantom (noisy data: the error against f_true stays at the noise level)."""
    N, x, m, y, f_true = _problem(gpulib)
    K = 40
    f64, _, d64 = infft.run_iterations(gpulib, False, N, x, m, y, K)
    f32, _, d32 = infft.run_iterations(gpulib, True, N, x, m, y, K, refresh=10)
    dist = np.linalg.norm(f32 - f64) / np.linalg.norm(f64)
    assert dist < 1e-2, dist
    e64 = np.linalg.norm(f64 - f_true) / np.linalg.norm(f_true)
    e32 = np.linalg.norm(f32 - f_true) / np.linalg.norm(f_true)
    assert abs(e32 - e64) < 1e-2 and e64 < 0.5, (e32, e64)
    assert d32[-1] < d32[0] and d64[-1] < d64[0]
