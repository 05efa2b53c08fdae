"""Parity at the full sizes of the configurations the transform is quoted on.

* 2-D FP64, N = 256^2, n = 512^2, m = 6, M = 65536 uniform nodes (seed 0):
  trafo and adjoint within 1e-12 relative l2 of the reference's own
  nfft_trafo / nfft_adjoint compiled in place, and index_x identical to the
  reference's (tests/golden/cfg1_ref.npz, tests/golden/make_cfg1_ref.py);
* 3-D FP32, N = 128^3, n = 256^3, m = 4, M = 2^24 nodes, uniform and
  clustered (32 Gaussians, std 0.02): index_x bit for bit equal to the
  oracle's sort of the same nodes (the oracle's sort key and stable order
  are pinned to the reference: tests/test_oracle.py).
"""
import os
import sys

import numpy as np
import pytest

import oracle
from helpers import rel_l2
from nfft_gb300 import abi, workloads
from nfft_gb300.plan import Plan

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_cfg1_ref as G1  # noqa: E402

pytestmark = pytest.mark.gpu


def test_cfg1_full_shape_matches_reference(gpulib):
    z = np.load(os.path.join(HERE, "golden", "cfg1_ref.npz"))
    x, fh, y = G1.inputs()
    assert G1.sha(x, fh, y) == str(z["inputs_sha256"]), "seeded inputs differ from the fixture's"
    f, fhat, idx = G1.run(gpulib, x, fh, y)
    e_t, e_a = rel_l2(f, z["trafo"]), rel_l2(fhat, z["adjoint"])
    print("2-D FP64 256^2 / 65536 nodes: trafo %.2e, adjoint %.2e relative l2 to the reference" % (e_t, e_a))
    assert e_t <= 1e-12, e_t
    assert e_a <= 1e-12, e_a
    assert G1.sha(idx) == str(z["index_x_sha256"]), "index_x differs from the reference's"


@pytest.mark.parametrize("dist", ["uniform", "clustered"])
def test_sort_of_2e24_nodes_is_bit_exact(gpulib, dist):
    N, n, m, M = [128] * 3, [256] * 3, 4, 1 << 24
    x = workloads.cube_nodes(M, 3, dist, 0)
    flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)
    p = Plan(gpulib, True, N, M, n=n, m=m, flags=flags)
    p.x[:] = x
    p.precompute_one_psi()
    got = p.index_x.copy()
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m, single=True)
    o.set_nodes(x)
    o.precompute()
    want = o.index_x()
    o.close()
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, "first difference at %d of %d" % (bad[0], got.size)


@pytest.mark.parametrize("dist", ["uniform", "clustered"])
def test_full_3d_size_adjointness_and_linearity(gpulib, dist):
    """At the full 3-D single-precision size (N = 128^3, n = 256^3, m = 4,
    M = 2^24), properties that hold at any size: the adjoint is the adjoint,
    <A fh, f> = <fh, A^H f> (relative to |A fh| |f|), and the transform is
    linear, A(a u + b v) = a A u + b A v -- both to single-precision accuracy."""
    N, n, m, M = [128] * 3, [256] * 3, 4, 1 << 24
    NN = 128 ** 3
    x = workloads.cube_nodes(M, 3, dist, 0)
    flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)
    p = Plan(gpulib, True, N, M, n=n, m=m, flags=flags)
    p.x[:] = x
    p.precompute_one_psi()
    rng = np.random.default_rng(4)
    u = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    v = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    a, b = np.complex64(0.75 - 0.5j), np.complex64(-1.25 + 0.25j)
    p.f_hat[:] = u
    p.trafo()
    Au = p.f.astype(np.complex128)
    p.f_hat[:] = v
    p.trafo()
    Av = p.f.astype(np.complex128)
    p.f_hat[:] = a * u + b * v
    p.trafo()
    Aw = p.f.astype(np.complex128)
    p.f[:] = f
    p.adjoint()
    AHf = p.f_hat.astype(np.complex128)
    p.finalize()
    lhs = np.vdot(f.astype(np.complex128), Au)   # <A u, f> = f^H A u
    rhs = np.vdot(AHf, u.astype(np.complex128))  # <u, A^H f> = (A^H f)^H u
    adj = abs(lhs - rhs) / (np.linalg.norm(Au) * np.linalg.norm(f))
    lin = np.linalg.norm(Aw - (complex(a) * Au + complex(b) * Av)) / np.linalg.norm(Aw)
    print("%s 2^24 nodes: adjointness %.2e, linearity %.2e" % (dist, adj, lin))
    assert adj < 1e-5, adj
    assert lin < 1e-5, lin
