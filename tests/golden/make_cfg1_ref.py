"""The reference's own double-precision outputs at the full 2-D FP64 shape:
N = 256^2, sigma = 2 (n = 512^2), Kaiser-Bessel m = 6, M = 65536 nodes iid
uniform in [-1/2, 1/2)^2, f_hat and the adjoint input y with real and
imaginary parts iid U(-1, 1), seed 0 (drawn in that order: x, Re f_hat,
Im f_hat, Re y, Im y).

The reference compiled in place (oracle/ref/Makefile) runs nfft_init_guru with
PRE_PHI_HUT | PRE_PSI | NFFT_SORT_NODES (+ the MALLOC / FFTW flags),
nfft_precompute_one_psi, nfft_trafo and nfft_adjoint; stored in
tests/golden/cfg1_ref.npz are both outputs in full, the SHA-256 of its
index_x (2M int64, key / node pairs) and the SHA-256 of the inputs, so a test
that regenerates the inputs from the seed knows they are the same bytes.

Usage: python tests/golden/make_cfg1_ref.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nfft_gb300 import abi  # noqa: E402
from nfft_gb300.plan import Plan  # noqa: E402

N, n, m, M, SEED = [256, 256], [512, 512], 6, 65536, 0
FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F | abi.FFTW_INIT
         | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)


def inputs():
    rng = np.random.default_rng(SEED)
    x = rng.uniform(-0.5, 0.5, size=(M, 2))
    NN = int(np.prod(N))
    fh = rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)
    y = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, fh, y


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run(lib, x, fh, y):
    """trafo, adjoint and index_x of one plan of `lib` (either library)."""
    p = Plan(lib, False, N, M, n=n, m=m, flags=FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = fh
    p.trafo()
    f = p.f.copy()
    p.f[:] = y
    p.adjoint()
    fhat = p.f_hat.copy()
    idx = p.index_x.copy()
    p.finalize()
    return f, fhat, idx


def main():
    ref = oracle.load_reference(False)
    if ref is None:
        sys.exit("reference library not built (oracle.build_reference())")
    x, fh, y = inputs()
    f, fhat, idx = run(ref, x, fh, y)
    np.savez_compressed(os.path.join(HERE, "cfg1_ref.npz"), trafo=f, adjoint=fhat,
                        index_x_sha256=np.array(sha(idx)), inputs_sha256=np.array(sha(x, fh, y)))
    print("cfg1_ref.npz written")


if __name__ == "__main__":
    main()
