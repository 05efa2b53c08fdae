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


def test_mixed_precision_cgnr_reaches_fp64_solution(gpulib):
    N, x, m, y, f_true = _problem(gpulib)
    f_ref, it_ref = infft.fp64_solution(gpulib, N, x, m, y, max_iter=3000)
    r = infft.time_to_tolerance(gpulib, True, N, x, m, y, f_ref, tol=1e-5, refresh=10, max_iter=3000)
    assert r["reached"], r
    assert r["err"] < 1e-5, r
    # the FP64 solution of the noisy problem is close to the phantom
    assert np.linalg.norm(f_ref - f_true) / np.linalg.norm(f_true) < 0.5


def test_fp64_cgnr_matches_itself_with_weights(gpulib):
    """Weighted CGNR (PRECOMPUTE_WEIGHT, density-compensation-like weights)
    converges to the weighted least-squares solution in fewer iterations."""
    N, x, m, y, _ = _problem(gpulib)
    r = np.sqrt((x ** 2).sum(axis=1))
    w = np.maximum(r, 1.0 / 128)
    f_w, it_w = infft.fp64_solution(gpulib, N, x, m, y, w=w, max_iter=3000, rtol=1e-10)
    f_u, it_u = infft.fp64_solution(gpulib, N, x, m, y, max_iter=3000, rtol=1e-10)
    assert it_w < it_u, (it_w, it_u)
