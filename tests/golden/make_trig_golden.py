"""Generate tests/golden/nfct_ref.npz: outputs of the reference's own NFCT and
NFST (kernel/nfct/nfct.c, kernel/nfst/nfst.c, compiled in place into oracle/_ref by
oracle/ref/Makefile) on seeded inputs -- trafo, adjoint and the direct
transforms -- in both precisions.  The GPU library's NFCT and NFST are compared with
these (tests/test_gpu_trig.py).

The reference built with OpenMP (as oracle/ref/Makefile builds it) takes, for
the multivariate NFST adjoint_direct, the branch at kernel/nfst/nfst.c:188-209,
which splits the flat frequency index with the bandwidths N_t instead of the
NFST's N_t - 1 frequencies per dimension, so for d >= 2 it sums the wrong
frequencies (nfst_d2_d differs from the fast adjoint by 1.4 in relative l2).
The serial branch (nfst.c:210-246) computes formula (1.2).  For those cases the
fixture keeps the reference's output as "adjoint_direct_openmp" and stores as
"adjoint_direct" the sum of formula (1.2) in double precision (nfst_direct
below, the serial branch restated with numpy), which the fast adjoint matches.

Usage: python tests/golden/make_trig_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import TrigPlan  # noqa: E402

FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.FFTW_INIT
         | abi.FFT_OUT_OF_PLACE)
# name, kind, single, N, M, n, m
CASES = [
    ("nfct_d1_d", "nfct", False, [64], 300, [130], 6),
    ("nfct_d2_d", "nfct", False, [24, 16], 400, [50, 34], 6),
    ("nfct_d3_d", "nfct", False, [12, 10, 8], 300, [26, 22, 18], 4),
    ("nfct_d1_s", "nfct", True, [64], 300, [130], 4),
    ("nfct_d2_s", "nfct", True, [24, 16], 400, [50, 34], 4),
    ("nfst_d1_d", "nfst", False, [64], 300, [129], 6),
    ("nfst_d2_d", "nfst", False, [24, 16], 400, [49, 33], 6),
    ("nfst_d3_d", "nfst", False, [12, 10, 8], 300, [25, 21, 17], 4),
    ("nfst_d2_s", "nfst", True, [24, 16], 400, [49, 33], 4),
]


def case_inputs(d, NN, M, seed, single):
    rng = np.random.default_rng(seed)
    dt = np.float32 if single else np.float64
    x = rng.uniform(0.0, 0.5, size=(M, d)).astype(dt)
    fh = rng.uniform(-1, 1, NN).astype(dt)
    f = rng.uniform(-1, 1, M).astype(dt)
    return x, fh, f


def nfst_direct_adjoint(N, x, f):
    """f_hat_k = sum_j f_j prod_t sin(2 pi k_t x_jt), k_t = 1 .. N_t - 1, in
    row-major order of k (kernel/nfst/nfst.c:210-246)."""
    d = len(N)
    k = np.indices([v - 1 for v in N]).reshape(d, -1).T + 1
    xx = np.asarray(x, np.float64).reshape(-1, d)
    A = np.prod(np.sin(2 * np.pi * k[None, :, :] * xx[:, None, :]), axis=2)
    return A.T @ np.asarray(f, np.float64)


def run(lib, kind, single, N, M, n, m, x, fh, f):
    p = TrigPlan(lib, kind, single, N, M, n, m, FLAGS)
    p.x[:] = x.ravel()
    p.precompute_one_psi()
    out = {}
    p.f_hat[:] = fh
    p.trafo()
    out["trafo"] = p.f.copy()
    p.trafo_direct()
    out["trafo_direct"] = p.f.copy()
    p.f[:] = f
    p.adjoint()
    out["adjoint"] = p.f_hat.copy()
    p.f[:] = f
    p.adjoint_direct()
    out["adjoint_direct"] = p.f_hat.copy()
    p.finalize()
    return out


def main():
    arrays = {}
    for i, (name, kind, single, N, M, n, m) in enumerate(CASES):
        ref = oracle.load_reference(single)
        if ref is None:
            sys.exit("reference library not built (oracle.build_reference())")
        NN = int(np.prod([v - (1 if kind == "nfst" else 0) for v in N]))
        x, fh, f = case_inputs(len(N), NN, M, 300 + i, single)
        out = run(ref, kind, single, N, M, n, m, x, fh, f)
        if kind == "nfst" and len(N) > 1:
            out["adjoint_direct_openmp"] = out["adjoint_direct"]
            out["adjoint_direct"] = nfst_direct_adjoint(N, x, f).astype(x.dtype)
        for k, a in (("x", x), ("f_hat", fh), ("f", f)):
            arrays["%s/%s" % (name, k)] = a
        for k, a in out.items():
            arrays["%s/%s" % (name, k)] = a
    np.savez_compressed(os.path.join(HERE, "nfct_ref.npz"), **arrays)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
