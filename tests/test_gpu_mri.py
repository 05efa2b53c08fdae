"""MRI operators with a field inhomogeneity (mri_inh_2d1d, mri_inh_3d,
reference kernel/mri/mri.c) on the GPU, against the reference's own outputs
(tests/golden/mri_ref.npz, written by tests/golden/make_mri_golden.py from
the reference compiled in place): trafo, adjoint, and for inh_3d the input f
as the adjoint leaves it (divided in place, as in the reference)."""
import os
import sys

import numpy as np
import pytest

from nfft_gb300.plan import MriPlan

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
sys.path.insert(0, GOLD)
import make_mri_golden as mk  # noqa: E402


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _gold(name):
    z = np.load(os.path.join(GOLD, "mri_ref.npz"))
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


@pytest.mark.gpu
@pytest.mark.parametrize("case", mk.CASES, ids=lambda c: c[0])
def test_mri_matches_reference(gpulib, case):
    name, kind, N, M, n, m, sigma = case
    g = _gold(name)
    p = MriPlan(gpulib, kind, N, M, n, m, sigma, mk.FLAGS)
    p.x[:] = g["x"].ravel()
    p.precompute()
    p.w[:] = g["w"]
    if kind == "2d1d":
        p.t[:] = g["t"]
    for _ in range(2):  # repeated calls give the same result
        p.f_hat[:] = g["f_hat"]
        p.trafo()
        assert rel(p.f, g["trafo"]) < 1e-10
    p.f[:] = g["f"]
    p.adjoint()
    assert rel(p.f_hat, g["adjoint"]) < 1e-10
    assert rel(p.f, g["f_after_adjoint"]) < 1e-13
    p.finalize()


def test_mri_fixture_is_the_inhomogeneity_operator():
    """CPU: the fixture's trafo approximates the exact operator
    f_j = sum_k f_hat_k exp(-2 pi i k.x_j) exp(-2 pi i w_k t_j N3)
    (t_j = x_j3 for inh_3d) to the accuracy the time window allows here."""
    for name, kind, N, M, n, m, sigma in mk.CASES:
        g = _gold(name)
        ks = [np.arange(-v // 2, v // 2) for v in N[:2]]
        k = np.stack(np.meshgrid(*ks, indexing="ij"), -1).reshape(-1, 2)
        x = g["x"].reshape(M, -1)
        t = g["t"] if kind == "2d1d" else x[:, 2]
        ex = (np.exp(-2j * np.pi * (x[:, :2] @ k.T)) * np.exp(-2j * np.pi * np.outer(t, g["w"]) * N[2])) @ g["f_hat"]
        assert rel(g["trafo"], ex) < 0.35, name
