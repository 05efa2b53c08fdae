"""Generate tests/golden/nfct_ref.npz: outputs of the reference's own NFCT
(kernel/nfct/nfct.c, compiled in place into oracle/_ref by
oracle/ref/Makefile) on seeded inputs -- trafo, adjoint and the direct
transforms -- in both precisions.  The GPU library's NFCT is compared with
these (tests/test_gpu_trig.py).

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
]


def case_inputs(d, NN, M, seed, single):
    rng = np.random.default_rng(seed)
    dt = np.float32 if single else np.float64
    x = rng.uniform(0.0, 0.5, size=(M, d)).astype(dt)
    fh = rng.uniform(-1, 1, NN).astype(dt)
    f = rng.uniform(-1, 1, M).astype(dt)
    return x, fh, f


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
        for k, a in (("x", x), ("f_hat", fh), ("f", f)):
            arrays["%s/%s" % (name, k)] = a
        for k, a in out.items():
            arrays["%s/%s" % (name, k)] = a
    np.savez_compressed(os.path.join(HERE, "nfct_ref.npz"), **arrays)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
