"""NFCT and NFST (reference kernel/nfct/nfct.c, kernel/nfst/nfst.c) on the GPU
in both precisions, against
the reference's own outputs (tests/golden/nfct_ref.npz, written by
tests/golden/make_trig_golden.py from the reference compiled in place):
trafo, adjoint and the direct transforms; plus the reference's check strings."""
import os
import sys

import numpy as np
import pytest

from nfft_gb300.plan import TrigPlan

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
sys.path.insert(0, GOLD)
import make_trig_golden as mk  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("case", mk.CASES, ids=lambda c: c[0])
def test_trig_matches_reference(gpulib, case):
    name, kind, single, N, M, n, m = case
    z = np.load(os.path.join(GOLD, "nfct_ref.npz"))
    g = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
    tol = 2e-5 if single else 1e-10
    p = TrigPlan(gpulib, kind, single, N, M, n, m, mk.FLAGS)
    p.x[:] = g["x"].ravel()
    p.precompute_one_psi()
    assert p.check() is None
    for _ in range(2):  # repeated calls give the same result
        p.f_hat[:] = g["f_hat"]
        p.trafo()
        assert rel(p.f, g["trafo"]) < tol
    p.trafo_direct()
    assert rel(p.f, g["trafo_direct"]) < (2e-5 if single else 1e-11)
    p.f[:] = g["f"]
    p.adjoint()
    assert rel(p.f_hat, g["adjoint"]) < tol
    p.f[:] = g["f"]
    p.adjoint_direct()
    assert rel(p.f_hat, g["adjoint_direct"]) < (2e-5 if single else 1e-11)
    p.x[0] = 0.5
    assert p.check() == "ths->x out of range [0.0,0.5)"
    p.finalize()


def test_trig_fixture_pins_reference():
    """CPU: the fixture's fast transforms approximate its direct sums."""
    z = np.load(os.path.join(GOLD, "nfct_ref.npz"))
    for name, kind, single, *_ in mk.CASES:
        lim = 1e-5 if single else 1e-7
        assert rel(z[name + "/trafo"], z[name + "/trafo_direct"]) < lim
        assert rel(z[name + "/adjoint"], z[name + "/adjoint_direct"]) < lim


def test_nfst_openmp_direct_adjoint_quirk():
    """CPU: the reference's OpenMP multivariate NFST adjoint_direct
    (kernel/nfst/nfst.c:188-209) splits the flat index k_L by N_t rather than by
    the N_t - 1 sine frequencies; the fixture keeps its output, which this
    restatement of that split reproduces, and the GPU library follows formula
    (1.2) instead (the serial branch, nfst.c:210-246)."""
    z = np.load(os.path.join(GOLD, "nfct_ref.npz"))
    for name, kind, single, N, M, n, m in mk.CASES:
        if kind != "nfst" or len(N) == 1:
            continue
        x = z[name + "/x"].astype(np.float64).reshape(M, len(N))
        f = z[name + "/f"].astype(np.float64)
        NT = int(np.prod([v - 1 for v in N]))
        k = np.zeros((NT, len(N)), np.int64)
        rem = np.arange(NT)
        for t in range(len(N) - 1, -1, -1):
            k[:, t] = rem % N[t] + 1
            rem //= N[t]
        A = np.prod(np.sin(2 * np.pi * k[None, :, :] * x[:, None, :]), axis=2)
        assert rel(z[name + "/adjoint_direct_openmp"], A.T @ f) < (1e-5 if single else 1e-12)
        assert rel(z[name + "/adjoint_direct_openmp"], z[name + "/adjoint_direct"]) > 0.1
