"""The single-precision error at the 3-D benchmark shape (N = 128^3,
n = 256^3, m = 4) and at the 2-D radial inverse-NFFT shape, held to at most
twice the reference's own nfftf error on
the same problem: a 4096-node subset plan with seeded inputs, the reference's
nfftf_trafo / nfftf_adjoint outputs from tests/golden/cfg2_single_ref.npz
(tests/golden/make_cfg2_single_ref.py), the FP64 NDFT (nfft_trafo_direct /
nfft_adjoint_direct) computed here on the GPU, relative l2 errors over all
nodes (trafo) and over 4096 seeded frequencies (adjoint)."""
import os
import sys

import numpy as np
import pytest

from nfft_gb300.plan import Plan

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_cfg2_single_ref as G  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fp32_error_within_twice_the_reference_nfftf(gpulib):
    z = np.load(os.path.join(HERE, "golden", "cfg2_single_ref.npz"))
    x, fh, f, idx = G.inputs()
    assert np.array_equal(idx, z["idx"])
    p = Plan(gpulib, True, G.N, G.M, n=G.n, m=G.m, flags=G.FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = fh
    p.trafo()
    f_gpu = p.f.copy()
    p.f[:] = f
    p.adjoint()
    fhat_gpu = p.f_hat[idx].copy()
    p.finalize()
    q = Plan(gpulib, False, G.N, G.M, n=G.n, m=G.m, flags=G.FLAGS)
    q.x[:] = x.astype(np.float64)
    q.f_hat[:] = fh.astype(np.complex128)
    q.trafo_direct()
    f_ndft = q.f.copy()
    q.f[:] = f.astype(np.complex128)
    q.adjoint_direct()
    fhat_ndft = q.f_hat[idx].copy()
    q.finalize()
    e_ref_t, e_gpu_t = rel(z["f_ref"], f_ndft), rel(f_gpu, f_ndft)
    e_ref_a, e_gpu_a = rel(z["fhat_ref"], fhat_ndft), rel(fhat_gpu, fhat_ndft)
    print("trafo: reference nfftf %.2e, this library %.2e; adjoint: reference %.2e, this library %.2e"
          % (e_ref_t, e_gpu_t, e_ref_a, e_gpu_a))
    assert e_gpu_t <= 2 * e_ref_t, (e_gpu_t, e_ref_t)
    assert e_gpu_a <= 2 * e_ref_a, (e_gpu_a, e_ref_a)


def _subset_errors(lib, z, key, Nc, nc, mc, x, fh, f, idx):
    """Relative l2 errors of the reference's nfftf (fixture) and of this
    library's FP32 plan, both against the FP64 NDFT on the GPU."""
    assert np.array_equal(idx, z[key + "_idx"])
    f_gpu, fhat_gpu = G.run(lib, True, Nc, nc, mc, x, fh, f, idx)
    q = Plan(lib, False, Nc, len(x), n=nc, m=mc, flags=G.FLAGS)
    q.x[:] = x.astype(np.float64)
    q.f_hat[:] = fh.astype(np.complex128)
    q.trafo_direct()
    f_ndft = q.f.copy()
    q.f[:] = f.astype(np.complex128)
    q.adjoint_direct()
    fhat_ndft = q.f_hat[idx].copy()
    q.finalize()
    return (rel(z[key + "_f_ref"], f_ndft), rel(f_gpu, f_ndft),
            rel(z[key + "_fhat_ref"], fhat_ndft), rel(fhat_gpu, fhat_ndft))


def test_fp32_error_clustered_within_twice_the_reference_nfftf(gpulib):
    """The 3-D benchmark shape with clustered nodes (the second variant of the
    3-D workload: 32 Gaussians of std 0.02, which crowd many nodes into the
    same cells): 4096 such nodes, N = 128^3, n = 256^3, m = 4."""
    z = np.load(os.path.join(HERE, "golden", "cfg2_single_ref.npz"))
    x, fh, f, idx = G.inputs_clustered()
    e_ref_t, e_gpu_t, e_ref_a, e_gpu_a = _subset_errors(gpulib, z, "clustered", G.N, G.n, G.m, x, fh, f, idx)
    print("clustered 3-D trafo: reference nfftf %.2e, this library %.2e; adjoint: reference %.2e, "
          "this library %.2e" % (e_ref_t, e_gpu_t, e_ref_a, e_gpu_a))
    assert e_gpu_t <= 2 * e_ref_t, (e_gpu_t, e_ref_t)
    assert e_gpu_a <= 2 * e_ref_a, (e_gpu_a, e_ref_a)


def test_fp32_error_radial_2d_within_twice_the_reference_nfftf(gpulib):
    """The same at the 2-D radial shape of the inverse-NFFT workload (the
    column kernels): 4096 of its nodes, N = 256^2, n = 512^2, m = 6."""
    z = np.load(os.path.join(HERE, "golden", "cfg2_single_ref.npz"))
    x, fh, f, idx = G.inputs_radial()
    assert np.array_equal(idx, z["radial_idx"])
    f_gpu, fhat_gpu = G.run(gpulib, True, G.N2, G.n2, G.m2, x, fh, f, idx)
    q = Plan(gpulib, False, G.N2, len(x), n=G.n2, m=G.m2, flags=G.FLAGS)
    q.x[:] = x.astype(np.float64)
    q.f_hat[:] = fh.astype(np.complex128)
    q.trafo_direct()
    f_ndft = q.f.copy()
    q.f[:] = f.astype(np.complex128)
    q.adjoint_direct()
    fhat_ndft = q.f_hat[idx].copy()
    q.finalize()
    e_ref_t, e_gpu_t = rel(z["radial_f_ref"], f_ndft), rel(f_gpu, f_ndft)
    e_ref_a, e_gpu_a = rel(z["radial_fhat_ref"], fhat_ndft), rel(fhat_gpu, fhat_ndft)
    print("radial 2-D trafo: reference nfftf %.2e, this library %.2e; adjoint: reference %.2e, this library %.2e"
          % (e_ref_t, e_gpu_t, e_ref_a, e_gpu_a))
    assert e_gpu_t <= 2 * e_ref_t, (e_gpu_t, e_ref_t)
    assert e_gpu_a <= 2 * e_ref_a, (e_gpu_a, e_ref_a)
