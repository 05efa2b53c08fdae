"""NNFFT (nonequispaced space and frequency nodes, reference
kernel/nnfft/nnfft.c) on the GPU, against the reference's own NNFFT outputs
(tests/golden/nnfft_ref.npz, written by tests/golden/make_nnfft_golden.py
from the reference compiled in place): trafo, adjoint, the input f as the
adjoint leaves it (scaled in place by the D factors, as in the reference),
and the FP64 direct NNDFT."""
import os

import numpy as np
import pytest

from nfft_gb300.plan import NnPlan

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _cases():
    import sys
    sys.path.insert(0, GOLD)
    import make_nnfft_golden as mk
    return mk.CASES


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_nnfft_matches_reference(gpulib, case):
    name, N, N1, Nt, M, m, flags = case
    z = np.load(os.path.join(GOLD, "nnfft_ref.npz"))
    g = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
    p = NnPlan(gpulib, N, Nt, M, N1, m, flags)
    p.x[:] = g["x"].ravel()
    p.v[:] = g["v"].ravel()
    p.precompute_one_psi()
    p.f_hat[:] = g["f_hat"]
    p.trafo()
    assert rel(p.f, g["trafo"]) < 1e-10
    p.trafo_direct()
    assert rel(p.f, g["trafo_direct"]) < 1e-12
    p.f[:] = g["f"]
    p.adjoint()
    assert rel(p.f_hat, g["adjoint"]) < 1e-10
    assert rel(p.f, g["f_after_adjoint"]) < 1e-13
    p.f[:] = g["f"]
    p.adjoint_direct()
    assert rel(p.f_hat, g["adjoint_direct"]) < 1e-12
    # repeated calls give the same result
    p.f_hat[:] = g["f_hat"]
    p.trafo()
    assert rel(p.f, g["trafo"]) < 1e-10
    p.finalize()


def test_nnfft_fixture_pins_reference():
    """The fixture's fast transforms approximate its direct NNDFT (CPU)."""
    z = np.load(os.path.join(GOLD, "nnfft_ref.npz"))
    for name, *_ in _cases():
        assert rel(z[name + "/trafo"], z[name + "/trafo_direct"]) < 1e-6
        assert rel(z[name + "/adjoint"], z[name + "/adjoint_direct"]) < 1e-6
