"""Generate tests/golden/nnfft_ref.npz: outputs of the reference's own NNFFT
(kernel/nnfft/nnfft.c, compiled in place into oracle/_ref by
oracle/ref/Makefile) on seeded inputs -- trafo, adjoint (and the input f as
the adjoint leaves it: scaled in place by the D factors), and the direct
NNDFT -- for a few shapes and precompute flags.  The GPU library's NNFFT is
compared with these (tests/test_gpu_nnfft.py).

Usage: python tests/golden/make_nnfft_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import NnPlan  # noqa: E402

MALLOC = abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.MALLOC_V
# name, N, N1, N_total (frequency nodes), M (space nodes), m, flags
CASES = [
    ("d1_pre_psi", [32], [64], 200, 150, 6, abi.PRE_PSI | abi.PRE_PHI_HUT | MALLOC),
    ("d1_no_pre", [48], [72], 120, 90, 5, MALLOC),
    ("d2_pre_psi", [16, 12], [32, 24], 300, 250, 6, abi.PRE_PSI | abi.PRE_PHI_HUT | MALLOC),
    ("d2_full_psi", [12, 12], [24, 24], 150, 140, 4, abi.PRE_FULL_PSI | abi.PRE_PHI_HUT | MALLOC),
    ("d3_pre_psi", [8, 8, 8], [16, 16, 16], 200, 180, 4, abi.PRE_PSI | abi.PRE_PHI_HUT | MALLOC),
]


def case_inputs(d, N_total, M, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.5, 0.5, size=(M, d))
    v = rng.uniform(-0.5, 0.5, size=(N_total, d))
    fh = rng.uniform(-1, 1, N_total) + 1j * rng.uniform(-1, 1, N_total)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, v, fh, f


def run(lib, name, N, N1, Nt, M, m, flags, x, v, fh, f):
    p = NnPlan(lib, N, Nt, M, N1, m, flags)
    p.x[:] = x.ravel()
    p.v[:] = v.ravel()
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
    out["f_after_adjoint"] = p.f.copy()
    p.f[:] = f
    p.adjoint_direct()
    out["adjoint_direct"] = p.f_hat.copy()
    p.finalize()
    return out


def main():
    ref = oracle.load_reference(False)
    if ref is None:
        sys.exit("reference library not built (oracle.build_reference())")
    arrays = {}
    for i, (name, N, N1, Nt, M, m, flags) in enumerate(CASES):
        x, v, fh, f = case_inputs(len(N), Nt, M, 100 + i)
        out = run(ref, name, N, N1, Nt, M, m, flags, x, v, fh, f)
        for k, a in (("x", x), ("v", v), ("f_hat", fh), ("f", f)):
            arrays["%s/%s" % (name, k)] = a
        for k, a in out.items():
            arrays["%s/%s" % (name, k)] = a
    np.savez_compressed(os.path.join(HERE, "nnfft_ref.npz"), **arrays)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
