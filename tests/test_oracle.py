"""The oracle pinned to the reference (CPU only).

* against the reference's own 64-digit golden files (tests/data/nfft_*.txt,
  written by tests/check_nfft.m) with the reference's error measure and bound
  (tests/nfft.c:217-284, 739-781);
* against outputs of the reference library compiled in place from its sources
  (tests/golden/refrun.npz, made by tests/golden/make_golden.py): transforms,
  sorted index_x bit-exactly, D coefficients, and CGNR / CGNE iterates.
"""
import os

import numpy as np
import pytest

import oracle
from helpers import (compare_adjoint, compare_trafo, err_direct_bound, err_trafo_bound,
                     next_pow2, rel_l2, seeded_case)


def golden_names(testdata):
    return sorted({k.split("/")[0] for k in testdata})


def oracle_plan(N, M, m, single, x):
    n = [2 * next_pow2(v) for v in N]
    p = oracle.OraclePlan(N, M, n=n, m=m, single=single)
    p.set_nodes(np.asarray(x).reshape(M, len(N)))
    p.precompute()
    return p


@pytest.mark.parametrize("single", [False, True])
def test_oracle_vs_reference_golden_files(testdata, single):
    m = 4 if single else 8  # WINDOW_HELP_ESTIMATE_m of the Kaiser-Bessel window
    checked = 0
    for name in golden_names(testdata):
        N = [int(v) for v in testdata[name + "/N"]]
        x = testdata[name + "/x"]
        fh = testdata[name + "/f_hat"]
        f = testdata[name + "/f"]
        M = len(f)
        p = oracle_plan(N, M, m, single, x)
        if "adjoint" in name:
            got = p.adjoint(f)
            err = compare_adjoint(got, fh, f)
            got_d = p.adjoint_direct(f)
            err_d = compare_adjoint(got_d, fh, f)
        else:
            got = p.trafo(fh)
            err = compare_trafo(got, f, fh)
            got_d = p.trafo_direct(fh)
            err_d = compare_trafo(got_d, f, fh)
        assert err < err_trafo_bound(m, single), (name, err)
        assert err_d < err_direct_bound(single), (name, err_d)
        checked += 1
    assert checked == 66


def refrun_cases(refrun):
    return sorted({k.split("/")[0] for k in refrun if k.endswith("/trafo")})


def test_oracle_vs_reference_run(refrun):
    for name in refrun_cases(refrun):
        meta = refrun[name + "/meta"]
        m, single, N = int(meta[0]), bool(meta[1]), [int(v) for v in meta[2:]]
        M = len(refrun[name + "/trafo"])
        x, fh, f = seeded_case(N, M)
        p = oracle_plan(N, M, m, single, x)
        tol = 3e-6 if single else 1e-13
        assert rel_l2(p.trafo(fh), refrun[name + "/trafo"]) < tol, name
        assert rel_l2(p.adjoint(f), refrun[name + "/adjoint"]) < tol, name
        assert np.array_equal(p.index_x(), refrun[name + "/index_x"]), name
        assert rel_l2(p.c_phi_inv(), refrun[name + "/c_phi_inv"]) < (2e-7 if single else 4e-15), name


def test_oracle_solver_vs_reference_run(refrun):
    names = sorted({k.split("/")[0] for k in refrun if k.endswith("/f_hat_iter")})
    assert len(names) >= 4
    for name in names:
        meta = refrun[name + "/meta"]
        m, single, sflags, N = int(meta[0]), bool(meta[1]), int(meta[2]), [int(v) for v in meta[3:]]
        iters = refrun[name + "/f_hat_iter"]
        y = refrun[name + "/y"]
        M = len(y)
        x, _, _ = seeded_case(N, M, seed=5)
        p = oracle_plan(N, M, m, single, x)
        s = oracle.OracleSolver(p, sflags)
        s.set(y=y, w=refrun[name + "/w"], w_hat=refrun[name + "/w_hat"],
              f_hat_iter=np.zeros(p.N_total))
        s.before_loop()
        tol = 5e-5 if single else 1e-10
        for it in range(1, iters.shape[0]):
            s.step()
            fh, _, sc = s.get()
            assert rel_l2(fh, iters[it]) < tol * it, (name, it)
        s.close()


def test_oracle_vs_reference_run_full_2d_fp64_shape():
    """The oracle at the full 2-D FP64 shape (N = 256^2, n = 512^2, m = 6,
    M = 65536) against the reference run stored in tests/golden/cfg1_ref.npz."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_cfg1_ref as G1
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cfg1_ref.npz"))
    x, fh, y = G1.inputs()
    assert G1.sha(x, fh, y) == str(z["inputs_sha256"])
    o = oracle.OraclePlan(G1.N, G1.M, n=G1.n, m=G1.m)
    o.set_nodes(x)
    o.precompute()
    assert rel_l2(o.trafo(fh), z["trafo"]) < 1e-14
    assert rel_l2(o.adjoint(y), z["adjoint"]) < 1e-14
    assert G1.sha(o.index_x()) == str(z["index_x_sha256"])


def test_oracle_fft_matches_numpy():
    rng = np.random.default_rng(1)
    for shape in [(16,), (12,), (8, 32), (4, 8, 16), (6, 10)]:
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        fw = oracle.fft(a, -1)
        bw = oracle.fft(a, +1)
        assert rel_l2(fw, np.fft.fftn(a)) < 1e-14
        assert rel_l2(bw, np.fft.ifftn(a) * a.size) < 1e-14


def test_oracle_bessel_i0():
    scipy_special = pytest.importorskip("scipy.special")
    for x in [0.0, 1.0, 2.5, 10.0, 37.7, 60.0, 150.0]:
        ref = float(scipy_special.i0(x))
        assert abs(oracle.bessel_i0(x) - ref) <= 8 * np.finfo(float).eps * ref


def test_oracle_bessel_i0_reference_table():
    """The oracle's I0 against the reference's own table (tests/bessel.c:29-139,
    I0(j) at j = 0, 1, 2, ...) within the reference test's bound of 4 eps
    relative (tests/bessel.c:141-167)."""
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bessel_i0.npz"))
    assert len(z["i0"]) > 50
    bound = 4 * np.finfo(float).eps
    for x, ref in zip(z["x"], z["i0"]):
        assert abs(oracle.bessel_i0(float(x)) - ref) <= bound * ref, (x, oracle.bessel_i0(float(x)), ref)


def test_oracle_sort_is_stable_and_keyed():
    N, M = [16, 16], 3000
    x, _, _ = seeded_case(N, M, seed=3)
    x[:200] = x[200:400]  # duplicated nodes: ties must keep input order
    p = oracle_plan(N, M, 6, False, x)
    idx = p.index_x()
    keys, ids = idx[0::2], idx[1::2]
    assert np.all(np.diff(keys) >= 0)
    order = np.lexsort((np.arange(M), keys))
    assert np.array_equal(np.sort(ids), np.arange(M))
    # stable: equal keys appear with increasing node id
    same = np.diff(keys) == 0
    assert np.all(np.diff(ids)[same] > 0)
    assert len(order) == M


def test_oracle_blockwise_adjoint_matches_serial():
    N, M = [32, 32, 32], 4000
    x, _, f = seeded_case(N, M, seed=4)
    n = [64, 64, 64]
    a = oracle.OraclePlan(N, M, n=n, m=4, single=False, blockwise=True)
    a.set_nodes(x)
    a.precompute()
    b = oracle.OraclePlan(N, M, n=n, m=4, single=False, blockwise=False)
    b.set_nodes(x)
    b.precompute()
    assert rel_l2(a.adjoint(f), b.adjoint(f)) < 1e-13
