"""Plans created and run from two host threads at once, in a fresh process.

Kernels that need more than 48 KB of dynamic shared memory get their limit
raised on first use, per device.  A process whose first plans of a kind come
from two threads at the same moment must see both transforms run with the
right limit (the reference's plans are independent objects too: each thread
may own one, include/nfft3.h:108-161).  The check runs in a child process so
that no earlier test has set any limit yet.
"""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r"""
    import sys, threading
    import numpy as np
    sys.path.insert(0, %(root)r)
    import nfft_gb300
    from nfft_gb300 import abi
    from nfft_gb300.plan import Plan

    lib = nfft_gb300.lib()
    FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)
    # (single, N, M, m): the 3-D column kernels, the 2-D column kernels in both
    # precisions and a 1-D tiled plan
    CASES = [(True, [32, 32, 32], 40000, 4), (True, [64, 64], 30000, 6),
             (False, [64, 64], 20000, 6), (True, [256], 5000, 4)]

    def run(case, seed):
        single, N, M, m = case
        rng = np.random.default_rng(seed)
        x = rng.uniform(-0.5, 0.5, (M, len(N)))
        fh = rng.uniform(-1, 1, int(np.prod(N))) + 1j * rng.uniform(-1, 1, int(np.prod(N)))
        f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
        p = Plan(lib, single, N, M, n=[2 * v for v in N], m=m, flags=FLAGS)
        p.x[:] = x
        p.precompute_one_psi()
        p.f_hat[:] = fh
        p.trafo()
        a = p.f.copy()
        p.f[:] = f
        p.adjoint()
        b = p.f_hat.copy()
        p.finalize()
        return a, b

    out = {}
    gate = threading.Barrier(2)

    def worker(k):
        gate.wait()
        out[k] = [run(c, 10 + i) for i, c in enumerate(CASES)]

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert sorted(out) == [0, 1], "a thread did not finish"
    again = [run(c, 10 + i) for i, c in enumerate(CASES)]  # one thread, afterwards
    for i, c in enumerate(CASES):
        tol = 1e-6 if c[0] else 1e-13
        for k in (0, 1):
            for got, want in zip(out[k][i], again[i]):
                e = np.linalg.norm(got - want) / np.linalg.norm(want)
                assert e < tol, (c, k, e)
    print("threads ok")
""")


def test_plans_from_two_threads_in_a_fresh_process():
    r = subprocess.run([sys.executable, "-c", CHILD % {"root": ROOT}], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "threads ok" in r.stdout
