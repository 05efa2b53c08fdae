"""Generate the golden fixtures of the test suite (run where the reference exists).

1. reference_testdata.npz -- the reference's own golden files
   (tests/data/nfft_*.txt, written by tests/check_nfft.m at 64-digit precision:
   d, N, M, nodes, f_hat and f), converted to float64 arrays.  Parsed like the
   reference reader (tests/nfft.c:379-448).
2. refrun.npz -- outputs of the reference library itself, compiled in place
   from its sources (oracle/ref/Makefile), on seeded inputs: trafo, adjoint,
   sorted index_x and c_phi_inv per case, plus CGNR / CGNE iterations of its
   solver.  These pin the oracle and the GPU library to the reference.

Usage: python tests/golden/make_golden.py [--reference /path/to/nfft]
"""
import argparse
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import Plan, Solver  # noqa: E402

# seeded parity cases: (name, N, M, m, single)
CASES = [
    ("d1_n64_m300_d", [64], 300, 8, False),
    ("d2_n32x48_m500_d", [32, 48], 500, 8, False),
    ("d2_n64x64_m2000_m6_d", [64, 64], 2000, 6, False),
    ("d3_n16_m800_d", [16, 16, 16], 800, 8, False),
    ("d1_n128_m500_s", [128], 500, 4, True),
    ("d2_n32x32_m1000_s", [32, 32], 1000, 4, True),
    ("d2_n48x32_m700_m6_s", [48, 32], 700, 6, True),
    ("d3_n16x16x16_m2000_s", [16, 16, 16], 2000, 4, True),
    ("d3_n24x16x32_m1500_m6_s", [24, 16, 32], 1500, 6, True),
    ("d4_n8_m300_m3_d", [8, 8, 8, 8], 300, 3, False),
]

SOLVER_CASES = [
    # name, N, M, m, single, flags
    ("cgnr_d2_d", [16, 16], 400, 6, False, abi.CGNR),
    ("cgnr_w_damp_d2_d", [16, 16], 400, 6, False, abi.CGNR | abi.PRECOMPUTE_WEIGHT | abi.PRECOMPUTE_DAMP),
    ("cgne_d2_d", [16, 16], 200, 6, False, abi.CGNE),
    ("cgne_w_damp_d2_d", [16, 16], 200, 6, False, abi.CGNE | abi.PRECOMPUTE_WEIGHT | abi.PRECOMPUTE_DAMP),
    ("cgnr_d2_s", [16, 16], 400, 4, True, abi.CGNR | abi.PRECOMPUTE_WEIGHT),
]
SOLVER_ITERS = 6


def case_inputs(N, M, seed=0):
    rng = np.random.default_rng(seed)
    d = len(N)
    x = rng.uniform(-0.5, 0.5, size=(M, d))
    NN = int(np.prod(N))
    fh = rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, fh, f


def default_flags(d):
    fl = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
          | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)
    return fl


def next_pow2(v):
    return 1 << (int(v) - 1).bit_length() if v > 1 else v + 1


def convert_testdata(ref_root):
    out = {}
    files = sorted(glob.glob(os.path.join(ref_root, "tests", "data", "nfft_*.txt")))
    for fn in files:
        name = os.path.basename(fn)[:-4]
        with open(fn) as fh:
            g = oracle.parse_golden_text(fh.read())
        out[name + "/N"] = np.array(g["N"], dtype=np.int64)
        out[name + "/x"] = g["x"]
        out[name + "/f_hat"] = g["first"]
        out[name + "/f"] = g["second"]
    np.savez_compressed(os.path.join(HERE, "reference_testdata.npz"), **out)
    print("reference_testdata.npz: %d files" % len(files))


def run_reference():
    out = {}
    for name, N, M, m, single in CASES:
        lib = oracle.load_reference(single)
        x, fh, f = case_inputs(N, M)
        n = [2 * next_pow2(v) for v in N]
        p = Plan(lib, single, N, M, n=n, m=m, flags=default_flags(len(N)))
        p.x[:] = x
        p.precompute_one_psi()
        p.f_hat[:] = fh
        p.trafo()
        out[name + "/trafo"] = p.f.copy()
        p.f[:] = f
        p.adjoint()
        out[name + "/adjoint"] = p.f_hat.copy()
        out[name + "/index_x"] = p.index_x.copy()
        out[name + "/c_phi_inv"] = np.concatenate(p.c_phi_inv)
        out[name + "/meta"] = np.array([m, int(single)] + N, dtype=np.int64)
        p.finalize()
    for name, N, M, m, single, sflags in SOLVER_CASES:
        lib = oracle.load_reference(single)
        x, fh, f = case_inputs(N, M, seed=5)
        n = [2 * next_pow2(v) for v in N]
        p = Plan(lib, single, N, M, n=n, m=m, flags=default_flags(len(N)))
        p.x[:] = x
        p.precompute_one_psi()
        s = Solver(p, sflags)
        rng = np.random.default_rng(7)
        y = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
        s.y[:] = y
        w = rng.uniform(0.5, 1.5, M)
        wh = rng.uniform(0.5, 1.0, p.N_total)
        if sflags & abi.PRECOMPUTE_WEIGHT:
            s.w[:] = w
        if sflags & abi.PRECOMPUTE_DAMP:
            s.w_hat[:] = wh
        s.f_hat_iter[:] = 0
        s.before_loop()
        iters = [s.f_hat_iter.copy()]
        scal = [list(s.scalars().values())]
        for _ in range(SOLVER_ITERS):
            s.loop_one_step()
            iters.append(s.f_hat_iter.copy())
            scal.append(list(s.scalars().values()))
        out[name + "/y"] = y
        out[name + "/w"] = w
        out[name + "/w_hat"] = wh
        out[name + "/f_hat_iter"] = np.array(iters)
        out[name + "/scalars"] = np.array(scal)
        out[name + "/meta"] = np.array([m, int(single), sflags] + N, dtype=np.int64)
        s.finalize()
        p.finalize()
    np.savez_compressed(os.path.join(HERE, "refrun.npz"), **out)
    print("refrun.npz: %d cases, %d solver cases" % (len(CASES), len(SOLVER_CASES)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=oracle.REFERENCE_SRC)
    a = ap.parse_args()
    os.environ["NFFT_REFERENCE_SRC"] = a.reference
    oracle.REFERENCE_SRC = a.reference
    oracle.build()
    if not oracle.build_reference():
        raise SystemExit("reference sources not found at %s" % a.reference)
    convert_testdata(a.reference)
    run_reference()


if __name__ == "__main__":
    main()
