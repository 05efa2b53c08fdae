"""The reference's own single-precision error at the 3-D benchmark shape
(N = 128^3, n = 256^3, m = 4, Kaiser-Bessel; uniform nodes, and nodes
clustered as a mixture of 32 Gaussians of std 0.02), and at the 2-D radial shape of
the inverse-NFFT workload (N = 256^2, n = 512^2, m = 6): nfftf_trafo and nfftf_adjoint
of the reference compiled in place (oracle/ref/Makefile, single-precision
FFT stand-in) on a 4096-node subset plan with seeded inputs, stored as
tests/golden/cfg2_single_ref.npz: the trafo output at all 4096 nodes and the
adjoint output at 4096 seeded frequencies.  tests/test_gpu_single_error.py
regenerates the same inputs, computes the FP64 NDFT on the GPU and holds the
library's FP32 error to at most twice the reference's.

Usage: python tests/golden/make_cfg2_single_ref.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import Plan  # noqa: E402

N, n, m, M, SEED, NSAMP = [128, 128, 128], [256, 256, 256], 4, 4096, 2024, 4096
FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.FFTW_INIT
         | abi.FFT_OUT_OF_PLACE)
# the 2-D radial shape of the inverse-NFFT workload: every 50th node of the
# 402 x 512 radial lines (the first 4096), N = 256^2, n = 512^2, m = 6
N2, n2, m2 = [256, 256], [512, 512], 6


def inputs():
    """Nodes, coefficients, adjoint input and the sampled frequency indices
    (numpy's PCG64 stream: the same on every platform)."""
    rng = np.random.default_rng(SEED)
    x = rng.uniform(-0.5, 0.5, (M, 3)).astype(np.float32)
    NN = int(np.prod(N))
    fh = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    idx = np.sort(rng.choice(NN, NSAMP, replace=False))
    return x, fh, f, idx


def inputs_clustered():
    """The 3-D shape again, the 4096 nodes drawn from the clustered
    distribution of the benchmark's second variant (32 Gaussians, std 0.02,
    wrapped to the torus)."""
    from nfft_gb300 import workloads
    x = workloads.cube_nodes(M, 3, "clustered", SEED + 2)
    rng = np.random.default_rng(SEED + 3)
    NN = int(np.prod(N))
    fh = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    idx = np.sort(rng.choice(NN, NSAMP, replace=False))
    return x, fh, f, idx


def inputs_radial():
    """The same for the 2-D radial shape."""
    from nfft_gb300 import workloads
    x = workloads.radial_nodes(402, 512)[::50][:M].astype(np.float32)
    rng = np.random.default_rng(SEED + 1)
    NN = int(np.prod(N2))
    fh = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    idx = np.sort(rng.choice(NN, NSAMP, replace=False))
    return x, fh, f, idx


def run(lib, single, Nc, nc, mc, x, fh, f, idx):
    p = Plan(lib, single, Nc, len(x), n=nc, m=mc, flags=FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = fh
    p.trafo()
    out_f = p.f.copy()
    p.f[:] = f
    p.adjoint()
    out_fh = p.f_hat[idx].copy()
    p.finalize()
    return out_f, out_fh


def main():
    ref = oracle.load_reference(True)
    if ref is None:
        sys.exit("reference library not built (oracle.build_reference())")
    x2, fh2, f2, idx2 = inputs_radial()
    f_ref2, fhat_ref2 = run(ref, True, N2, n2, m2, x2, fh2, f2, idx2)
    x3, fh3, f3, idx3 = inputs_clustered()
    f_ref3, fhat_ref3 = run(ref, True, N, n, m, x3, fh3, f3, idx3)
    x, fh, f, idx = inputs()
    p = Plan(ref, True, N, M, n=n, m=m, flags=FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = fh
    p.trafo()
    f_ref = p.f.copy()
    p.f[:] = f
    p.adjoint()
    fhat_ref = p.f_hat[idx].copy()
    p.finalize()
    np.savez_compressed(os.path.join(HERE, "cfg2_single_ref.npz"), f_ref=f_ref, fhat_ref=fhat_ref, idx=idx,
                        radial_f_ref=f_ref2, radial_fhat_ref=fhat_ref2, radial_idx=idx2,
                        clustered_f_ref=f_ref3, clustered_fhat_ref=fhat_ref3, clustered_idx=idx3)
    print("cfg2_single_ref.npz written")


if __name__ == "__main__":
    main()
