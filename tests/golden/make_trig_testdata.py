"""Convert the reference's NFCT / NFST golden files (tests/data/nfct_*.txt,
nfst_*.txt of the reference tree, read as tests/nfct.c and tests/nfst.c read
them: d, N_1..N_d, M, the M x d nodes, the real coefficients f_hat -- prod N_t
of them for the NFCT, prod (N_t - 1) for the NFST -- and the M real samples
f) into tests/golden/trig_testdata.npz.  Trafo files hold f = A f_hat, adjoint
files f_hat = A^T f, in the same positions.

Usage: python tests/golden/make_trig_testdata.py [reference root]
"""
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402  (the reference checkout's location)


def parse(text, sine):
    tok = text.split()
    pos = 0
    d = int(tok[pos]); pos += 1
    N = [int(tok[pos + i]) for i in range(d)]; pos += d
    M = int(tok[pos]); pos += 1
    x = np.array([float(v) for v in tok[pos:pos + M * d]]); pos += M * d
    NN = int(np.prod([v - 1 if sine else v for v in N]))
    fh = np.array([float(v) for v in tok[pos:pos + NN]]); pos += NN
    f = np.array([float(v) for v in tok[pos:pos + M]]); pos += M
    return N, x.reshape(M, d), fh, f


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else oracle.REFERENCE_SRC
    out = {}
    files = sorted(glob.glob(os.path.join(root, "tests", "data", "nfct_*.txt"))
                   + glob.glob(os.path.join(root, "tests", "data", "nfst_*.txt")))
    for fn in files:
        name = os.path.basename(fn)[:-4]
        with open(fn) as fh:
            N, x, fhat, f = parse(fh.read(), name.startswith("nfst"))
        out[name + "/N"] = np.array(N, dtype=np.int64)
        out[name + "/x"] = x
        out[name + "/f_hat"] = fhat
        out[name + "/f"] = f
    np.savez_compressed(os.path.join(HERE, "trig_testdata.npz"), **out)
    print("trig_testdata.npz: %d files" % len(files))


if __name__ == "__main__":
    main()
