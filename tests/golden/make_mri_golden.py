"""Generate tests/golden/mri_ref.npz: outputs of the reference's own MRI
operators with a field inhomogeneity (kernel/mri/mri.c, compiled in place
into oracle/_ref by oracle/ref/Makefile) on seeded inputs -- trafo, adjoint
and, for inh_3d, the input f as the adjoint leaves it (divided in place).
The GPU library's operators are compared with these (tests/test_gpu_mri.py).

Usage: python tests/golden/make_mri_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import MriPlan  # noqa: E402

FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.FFTW_INIT
         | abi.FFT_OUT_OF_PLACE)
# name, kind, N (N0, N1, N3), M, n, m, sigma
CASES = [
    ("2d1d_a", "2d1d", [16, 16, 8], 400, [32, 32], 6, 1.5),
    ("2d1d_b", "2d1d", [12, 20, 6], 300, [24, 40], 4, 2.0),
    ("3d_a", "3d", [12, 12, 8], 500, [24, 24, 16], 6, 2.0),
    ("3d_b", "3d", [16, 8, 10], 350, [32, 16, 20], 4, 2.0),
]


def case_inputs(kind, N, M, seed):
    rng = np.random.default_rng(seed)
    d = 2 if kind == "2d1d" else 3
    x = rng.uniform(-0.5, 0.5, size=(M, d))
    if d == 3:
        x[:, 2] = rng.uniform(-0.4, 0.4, M)
    NN = N[0] * N[1]
    w = rng.uniform(-0.25, 0.25, NN)
    t = rng.uniform(-0.4, 0.4, M)
    fh = rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, w, t, fh, f


def run(lib, kind, N, M, n, m, sigma, x, w, t, fh, f):
    p = MriPlan(lib, kind, N, M, n, m, sigma, FLAGS)
    p.x[:] = x.ravel()
    p.precompute()
    p.w[:] = w
    if kind == "2d1d":
        p.t[:] = t
    out = {}
    p.f_hat[:] = fh
    p.trafo()
    out["trafo"] = p.f.copy()
    p.f[:] = f
    p.adjoint()
    out["adjoint"] = p.f_hat.copy()
    out["f_after_adjoint"] = p.f.copy()
    p.finalize()
    return out


def main():
    ref = oracle.load_reference(False)
    if ref is None:
        sys.exit("reference library not built (oracle.build_reference())")
    arrays = {}
    for i, (name, kind, N, M, n, m, sigma) in enumerate(CASES):
        x, w, t, fh, f = case_inputs(kind, N, M, 200 + i)
        out = run(ref, kind, N, M, n, m, sigma, x, w, t, fh, f)
        for k, a in (("x", x), ("w", w), ("t", t), ("f_hat", fh), ("f", f)):
            arrays["%s/%s" % (name, k)] = a
        for k, a in out.items():
            arrays["%s/%s" % (name, k)] = a
    np.savez_compressed(os.path.join(HERE, "mri_ref.npz"), **arrays)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
