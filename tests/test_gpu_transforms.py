"""GPU parity of the transform path through the C ABI (nfft_* / nfftf_*).

Mirrors the reference's own test strategy (tests/nfft.c): golden files with
the reference's init variants and error bound, online cases against the NDFT,
plus bit-exact sorted index_x and element-wise agreement with the reference
library's outputs (tests/golden/refrun.npz) and with the oracle.

Tolerances: double plans agree with the reference to 1e-12 relative l2;
single plans stay within 2x of the reference nfftf error against the FP64
NDFT (plus 1e-7 absolute slack for rounding at tiny errors).
"""
import numpy as np
import pytest

import oracle
from helpers import (compare_adjoint, compare_trafo, default_guru_flags, err_direct_bound,
                     err_trafo_bound, next_pow2, rel_l2, seeded_case)
from nfft_gb300 import abi
from nfft_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def make_plan(lib, single, N, M, m=None, flags=None, init="guru", n=None):
    if init == "guru":
        if n is None:
            n = [2 * next_pow2(v) for v in N]
        if m is None:
            m = 4 if single else 8
        return Plan(lib, single, N, M, n=n, m=m,
                    flags=default_guru_flags() if flags is None else flags)
    return Plan(lib, single, N, M, init=init)


def run_both(p, x, fh, f):
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = fh
    p.trafo()
    out_f = p.f.copy()
    p.f[:] = f
    p.adjoint()
    return out_f, p.f_hat.copy()


def ndft(N, x, fh, f, m=8):
    o = oracle.OraclePlan(N, len(x), m=m, single=False)
    o.set_nodes(x)
    return o.trafo_direct(fh), o.adjoint_direct(f)


# ---------------------------------------------------------------- golden files
# tests/nfft.c:691-701 (its PRE_LIN_PSI variant is defined there and left out
# of the run lists at 812; its PRE_FG_PSI one exists only for the Gaussian
# window build).  This library evaluates the Kaiser-Bessel window exactly for
# every PRE_*PSI flag, so each variant is held to the window's bound.
INITS = ["dim", "default", "guru_pre_psi", "guru_pre_full_psi", "guru_pre_lin_psi", "guru_pre_fg_psi"]


@pytest.mark.parametrize("single", [False, True])
@pytest.mark.parametrize("init", INITS)
def test_golden_files(gpulib, testdata, single, init):
    """tests/nfft.c:691-708 init variants x trafo/adjoint on all 66 golden files."""
    names = sorted({k.split("/")[0] for k in testdata})
    for name in names:
        N = [int(v) for v in testdata[name + "/N"]]
        x = testdata[name + "/x"]
        fh = testdata[name + "/f_hat"]
        f = testdata[name + "/f"]
        M = len(f)
        d = len(N)
        if init == "dim":
            p = make_plan(gpulib, single, N, M, init="%dd" % d)
        elif init == "default":
            p = make_plan(gpulib, single, N, M, init="default")
        else:
            flags = default_guru_flags()
            if init == "guru_pre_full_psi":
                flags = (flags & ~abi.PRE_PSI) | abi.PRE_FULL_PSI
            elif init == "guru_pre_lin_psi":
                flags = (flags & ~abi.PRE_PSI) | abi.PRE_LIN_PSI
            elif init == "guru_pre_fg_psi":
                flags = (flags & ~abi.PRE_PSI) | abi.FG_PSI | abi.PRE_FG_PSI
            p = make_plan(gpulib, single, N, M, flags=flags)
        p.x[:] = x
        if p.check() is not None:
            # the reference counts a case its nfft_check rejects (odd N) as
            # passed without running it (tests/nfft.c:315-325)
            assert N[0] % 2 == 1, (name, p.check())
            p.finalize()
            continue
        p.precompute_one_psi()
        if "adjoint" in name:
            p.f[:] = f
            p.adjoint()
            err = compare_adjoint(p.f_hat.copy(), fh, f)
        else:
            p.f_hat[:] = fh
            p.trafo()
            err = compare_trafo(p.f.copy(), f, fh)
        bound = err_trafo_bound(p.m, single)
        p.finalize()
        assert err < bound, (name, init, err, bound)


@pytest.mark.parametrize("single", [False, True])
def test_golden_files_direct(gpulib, testdata, single):
    """trafo_direct / adjoint_direct on the golden files, bound 48 eps."""
    names = sorted({k.split("/")[0] for k in testdata})
    for name in names:
        N = [int(v) for v in testdata[name + "/N"]]
        x, fh, f = testdata[name + "/x"], testdata[name + "/f_hat"], testdata[name + "/f"]
        M = len(f)
        p = make_plan(gpulib, single, N, M, flags=default_guru_flags() & ~abi.PRE_PSI)
        p.x[:] = x
        if "adjoint" in name:
            p.f[:] = f
            p.adjoint_direct()
            err = compare_adjoint(p.f_hat.copy(), fh, f)
        else:
            p.f_hat[:] = fh
            p.trafo_direct()
            err = compare_trafo(p.f.copy(), f, fh)
        p.finalize()
        assert err < err_direct_bound(single), (name, err)


# ---------------------------------------------------------------- reference run
def test_reference_run_parity(gpulib, refrun):
    names = sorted({k.split("/")[0] for k in refrun if k.endswith("/trafo")})
    for name in names:
        meta = refrun[name + "/meta"]
        m, single, N = int(meta[0]), bool(meta[1]), [int(v) for v in meta[2:]]
        M = len(refrun[name + "/trafo"])
        x, fh, f = seeded_case(N, M)
        flags = default_guru_flags() | abi.NFFT_SORT_NODES
        p = make_plan(gpulib, single, N, M, m=m, flags=flags)
        gf, gfh = run_both(p, x, fh, f)
        idx = p.index_x
        cphi = np.concatenate(p.c_phi_inv)
        p.finalize()
        assert np.array_equal(idx, refrun[name + "/index_x"]), name
        rf, rfh = refrun[name + "/trafo"], refrun[name + "/adjoint"]
        if not single:
            assert rel_l2(gf, rf) < 1e-12, (name, rel_l2(gf, rf))
            assert rel_l2(gfh, rfh) < 1e-12, (name, rel_l2(gfh, rfh))
            assert rel_l2(cphi, refrun[name + "/c_phi_inv"]) < 1e-14
        else:
            tf, tfh = ndft(N, x.astype(np.float32).astype(np.float64), fh.astype(np.complex64),
                           f.astype(np.complex64))
            e_ref, e_gpu = rel_l2(rf, tf), rel_l2(gf, tf)
            assert e_gpu <= 2 * e_ref + 1e-7, (name, "trafo", e_gpu, e_ref)
            e_ref, e_gpu = rel_l2(rfh, tfh), rel_l2(gfh, tfh)
            assert e_gpu <= 2 * e_ref + 1e-7, (name, "adjoint", e_gpu, e_ref)


# ---------------------------------------------------------------- online vs oracle
CASES = [
    # N, M, m, single
    ([256], 3000, 8, False),
    ([100], 700, 5, False),
    ([64, 64], 5000, 6, False),
    ([40, 24], 900, 7, False),
    ([32, 32, 32], 6000, 4, False),
    ([16, 16, 16], 500, 9, False),  # no tiled kernel for m=9: generic path
    ([512], 20000, 4, True),
    ([128, 128], 40000, 6, True),
    ([64, 32], 3000, 3, True),
    ([64, 64, 64], 100000, 4, True),
    ([32, 48, 16], 20000, 6, True),
    ([8, 8, 8, 8], 500, 3, False),  # d = 4: generic kernels and split FFT
    ([6, 8, 4, 6, 4], 200, 2, True),  # d = 5
]


@pytest.mark.parametrize("N,M,m,single", CASES)
def test_online_vs_oracle(gpulib, N, M, m, single):
    x, fh, f = seeded_case(N, M, seed=11)
    flags = default_guru_flags() | abi.NFFT_SORT_NODES
    p = make_plan(gpulib, single, N, M, m=m, flags=flags)
    gf, gfh = run_both(p, x, fh, f)
    idx = p.index_x
    p.finalize()
    o = oracle.OraclePlan(N, M, n=[2 * next_pow2(v) for v in N], m=m, single=single)
    o.set_nodes(x.astype(np.float32) if single else x)
    o.precompute()
    assert np.array_equal(idx, o.index_x())
    od = oracle.OraclePlan(N, M, n=[2 * next_pow2(v) for v in N], m=m, single=False)
    od.set_nodes(x.astype(np.float32).astype(np.float64) if single else x)
    od.precompute()
    rf = od.trafo(fh.astype(np.complex64) if single else fh)
    rfh = od.adjoint(f.astype(np.complex64) if single else f)
    tol = 2e-5 if single else 1e-12
    assert rel_l2(gf, rf) < tol, rel_l2(gf, rf)
    assert rel_l2(gfh, rfh) < tol, rel_l2(gfh, rfh)


@pytest.mark.parametrize("N,n,m,single", [
    ([16, 16], [34, 34], 6, False),      # tile edge does not divide n; padded tile wraps twice
    ([30, 20], [40, 44], 4, True),
    ([6, 6, 6], [12, 12, 12], 4, True),  # 3-D sub-cell kernels on a grid smaller than tile + window
    ([10, 12, 8], [20, 26, 18], 4, True),
])
def test_non_power_of_two_grids(gpulib, N, n, m, single):
    M = 3000
    x, fh, f = seeded_case(N, M, seed=13)
    p = make_plan(gpulib, single, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    gf, gfh = run_both(p, x, fh, f)
    idx = p.index_x
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m, single=single)
    o.set_nodes(x.astype(np.float32) if single else x)
    o.precompute()
    assert np.array_equal(idx, o.index_x())
    od = oracle.OraclePlan(N, M, n=n, m=m, single=False)
    od.set_nodes(x.astype(np.float32).astype(np.float64) if single else x)
    od.precompute()
    tol = 2e-5 if single else 1e-12
    assert rel_l2(gf, od.trafo(fh.astype(np.complex64) if single else fh)) < tol
    assert rel_l2(gfh, od.adjoint(f.astype(np.complex64) if single else f)) < tol


def test_clustered_nodes_and_heavy_tiles(gpulib):
    """Nodes packed into a few tiles: many work items per tile, same results."""
    rng = np.random.default_rng(5)
    N, M, m = [32, 32, 32], 60000, 4
    centres = rng.uniform(-0.5, 0.5, (4, 3))
    x = centres[rng.integers(0, 4, M)] + 0.01 * rng.standard_normal((M, 3))
    x = ((x + 0.5) % 1.0) - 0.5
    fh = rng.uniform(-1, 1, 32 ** 3) + 1j * rng.uniform(-1, 1, 32 ** 3)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    p = make_plan(gpulib, True, N, M, m=m)
    gf, gfh = run_both(p, x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64))
    p.finalize()
    od = oracle.OraclePlan(N, M, n=[64] * 3, m=m, single=False)
    od.set_nodes(x.astype(np.float32).astype(np.float64))
    od.precompute()
    assert rel_l2(gf, od.trafo(fh.astype(np.complex64))) < 2e-5
    assert rel_l2(gfh, od.adjoint(f.astype(np.complex64))) < 2e-5


@pytest.mark.parametrize("density", [1, 3])
@pytest.mark.parametrize("m", [3, 4, 6])
def test_dense_3d_single(gpulib, density, m):
    """3-D single precision at >= 1 node per oversampled cell: sub-cell groups
    larger than one unit, the regime of the 3-D benchmark."""
    N = [16, 16, 16]
    M = density * 32 ** 3
    x, fh, f = seeded_case(N, M, seed=12)
    x32 = x.astype(np.float32)
    p = make_plan(gpulib, True, N, M, m=m)
    gf, gfh = run_both(p, x32, fh.astype(np.complex64), f.astype(np.complex64))
    p.finalize()
    od = oracle.OraclePlan(N, M, n=[32] * 3, m=m, single=False)
    od.set_nodes(x32.astype(np.float64))
    od.precompute()
    rf = od.trafo(fh.astype(np.complex64))
    rfh = od.adjoint(f.astype(np.complex64))
    assert rel_l2(gf, rf) < 2e-5, rel_l2(gf, rf)
    assert rel_l2(gfh, rfh) < 2e-5, rel_l2(gfh, rfh)


@pytest.mark.parametrize("m,single", [(2, True), (3, True), (4, True), (5, True), (6, True), (7, True),
                                      (4, False), (6, False)])
def test_radial_2d(gpulib, m, single):
    """2-D radial k-space lines: every spoke passes the centre (one node
    repeated per spoke there), so the central tiles hold hundreds of nodes
    per cell and split into many work items; every window width of the
    single-precision 2-D column kernels, and the double-precision column
    spreading."""
    N = [64, 64]
    spokes, samples = 96, 128
    ang = np.pi * np.arange(spokes) / spokes
    r = -0.5 + np.arange(samples) / samples
    x = np.stack([np.outer(np.cos(ang), r).ravel(), np.outer(np.sin(ang), r).ravel()], axis=1)
    x = (((x + 0.5) % 1.0) - 0.5).astype(np.float32 if single else np.float64)
    M = len(x)
    rng = np.random.default_rng(40 + m)
    ct = np.complex64 if single else np.complex128
    fh = (rng.uniform(-1, 1, 64 * 64) + 1j * rng.uniform(-1, 1, 64 * 64)).astype(ct)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(ct)
    p = make_plan(gpulib, single, N, M, m=m)
    gf, gfh = run_both(p, x, fh, f)
    p.finalize()
    od = oracle.OraclePlan(N, M, n=[128, 128], m=m, single=False)
    od.set_nodes(x.astype(np.float64))
    od.precompute()
    rf = od.trafo(fh)
    rfh = od.adjoint(f)
    tol = 2e-5 if single else 1e-12
    assert rel_l2(gf, rf) < tol, rel_l2(gf, rf)
    assert rel_l2(gfh, rfh) < tol, rel_l2(gfh, rfh)


def test_edge_nodes_and_small_m(gpulib):
    """Nodes on -1/2 and just below +1/2, window wrap-around on every side."""
    N, m = [32, 32], 6
    edge = np.array([-0.5, -0.5 + 1e-12, 0.5 - 1e-12, 0.0, -1e-17, 0.25])
    x = np.array(np.meshgrid(edge, edge)).reshape(2, -1).T.copy()
    M = len(x)
    rng = np.random.default_rng(2)
    fh = rng.uniform(-1, 1, 1024) + 1j * rng.uniform(-1, 1, 1024)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    for single in (False, True):
        xx = x.astype(np.float32) if single else x
        p = make_plan(gpulib, single, N, M, m=m, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
        gf, gfh = run_both(p, xx, fh, f)
        idx = p.index_x
        p.finalize()
        o = oracle.OraclePlan(N, M, n=[64, 64], m=m, single=single)
        o.set_nodes(xx)
        o.precompute()
        assert np.array_equal(idx, o.index_x())
        tf, tfh = ndft(N, xx.astype(np.float64), fh, f)
        bound = err_trafo_bound(m, single) * 10
        assert compare_trafo(gf, tf, fh) < bound
        assert compare_adjoint(gfh, tfh, f) < bound


def test_single_node_and_direct_fallback(gpulib):
    # M = 1, and N <= m forces the NDFT path (nfft.c:5658-5665)
    for N, M, m in (([16, 16], 1, 6), ([4, 6], 30, 8), ([2], 5, 4)):
        x, fh, f = seeded_case(N, M, seed=9)
        p = make_plan(gpulib, False, N, M, m=m)
        gf, gfh = run_both(p, x, fh, f)
        p.finalize()
        tf, tfh = ndft(N, x, fh, f)
        assert rel_l2(gf, tf) < 1e-9
        assert rel_l2(gfh, tfh) < 1e-9


@pytest.mark.parametrize("single", [False, True])
@pytest.mark.parametrize("N,m", [([16], 4), ([32, 32], 6), ([32, 32], 4), ([16, 16, 16], 4)])
def test_zero_nodes(gpulib, single, N, m):
    """A plan without nodes (M = 0): the reference's loops over j < M_total do
    nothing, so trafo writes no sample and adjoint returns f_hat = 0, on
    every call."""
    NN = int(np.prod(N))
    rng = np.random.default_rng(4)
    fh = rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)
    for flags in (default_guru_flags(), default_guru_flags() | abi.NFFT_SORT_NODES):
        p = make_plan(gpulib, single, N, 0, m=m, flags=flags)
        p.precompute_one_psi()
        for _ in range(2):
            p.f_hat[:] = fh
            p.trafo()
            assert len(p.f) == 0
            p.adjoint()
            assert np.array_equal(p.f_hat, np.zeros(NN))
        p.finalize()


def test_check_messages(gpulib):
    p = make_plan(gpulib, False, [16, 16], 10, m=4)
    p.x[:] = 0.1
    assert p.check() is None
    p.x[3, 1] = 0.5
    assert p.check() == "ths->x out of range [-0.5,0.5)"
    p.finalize()
    q = make_plan(gpulib, False, [15, 16], 10, m=4)
    q.x[:] = 0.0
    assert q.check() == "polynomial degree N has to be even"
    q.finalize()


def test_repeated_calls_and_no_precompute_flags(gpulib):
    """Without PRE_*PSI flags the node set-up follows x on every call."""
    N, M = [48, 48], 3000
    x, fh, f = seeded_case(N, M, seed=21)
    flags = abi.PRE_PHI_HUT | abi.MALLOC_X | abi.MALLOC_F | abi.MALLOC_F_HAT | abi.FFTW_INIT
    p = make_plan(gpulib, False, N, M, m=6, flags=flags)
    p.x[:] = x
    p.f_hat[:] = fh
    p.trafo()
    a = p.f.copy()
    p.trafo()
    assert np.array_equal(a, p.f)
    x2 = np.roll(x, 7, axis=0)
    p.x[:] = x2
    p.trafo()
    b = p.f.copy()
    p.finalize()
    tf, _ = ndft(N, x2, fh, f)
    assert rel_l2(b, tf) < 1e-9
    assert rel_l2(b, np.roll(a, 7)) < 1e-12


@pytest.mark.parametrize("N,n", [([16, 16, 16], [36, 40, 34]), ([16, 16, 16], [40, 36, 33]),
                                 ([8, 8, 8], [16, 16, 16]), ([12, 8, 20], [24, 16, 40])])
def test_3d_single_grids_with_and_without_tma_tiles(gpulib, N, n):
    """The 3-D single-precision kernels on grids where the TMA paths do not all
    apply: an odd last grid length (no tensor map: every tile staged and
    written back cell by cell), grids smaller than the padded tile (every tile
    wraps around the grid edge) and mixes of interior and edge tiles.  Both
    transforms against the oracle; no bounded TMA wait may have given up.
    (Oversampling stays at 2 or more: at n = N the window's Fourier
    coefficients nearly vanish at the band edge, and even the oracle's own
    single-precision path differs from its double-precision one by 2e3.)"""
    import ctypes as C
    M, m = 6000, 4
    x, fh, f = seeded_case(N, M, seed=31)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    got_f, got_fh = run_both(p, x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64))
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    e_t = rel_l2(got_f.astype(np.complex128), o.trafo(fh.astype(np.complex64).astype(np.complex128)))
    e_a = rel_l2(got_fh.astype(np.complex128), o.adjoint(f.astype(np.complex64).astype(np.complex128)))
    assert e_t < 1e-5 and e_a < 1e-5, (n, e_t, e_a)
    fn = gpulib.nfft_gb_tma_wait_timeouts
    fn.restype = C.c_ulonglong
    assert fn() == 0


@pytest.mark.parametrize("M", [6000, 300000])
def test_3d_single_b_kernels_against_oracle(gpulib, M):
    """Both kernels of the single-precision 3-D B (nfftf_gb_set_b3_kernel:
    column segments and sub-cell units) against the oracle on the same plan,
    at sparse (94 nodes per 8^3 tile) and dense (4688) nodes; the default is
    the column form at any density, and mode 0 returns to it."""
    import ctypes as C
    N, n, m = [16, 16, 16], [32, 32, 32], 4
    x, fh, _ = seeded_case(N, M, seed=41)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    p.x[:] = x.astype(np.float32)
    p.precompute_one_psi()
    pa = C.addressof(p.p)
    get = gpulib.nfftf_gb_b3_kernel
    get.restype, get.argtypes = C.c_int, [C.c_void_p]
    setk = gpulib.nfftf_gb_set_b3_kernel
    setk.restype, setk.argtypes = C.c_int, [C.c_void_p, C.c_int]
    assert get(pa) == 1
    o = oracle.OraclePlan(N, M, n=n, m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    want = o.trafo(fh.astype(np.complex64).astype(np.complex128))
    o.close()
    got = {}
    for mode in (1, 2):
        assert setk(pa, mode) == 0 and get(pa) == mode
        p.f_hat[:] = fh.astype(np.complex64)
        p.trafo()
        got[mode] = p.f.astype(np.complex128)
    assert setk(pa, 0) == 0 and get(pa) == 1
    p.finalize()
    e1, e2 = rel_l2(got[1], want), rel_l2(got[2], want)
    print("M=%d: column segments %.2e, sub-cell units %.2e relative l2 to the oracle" % (M, e1, e2))
    assert e1 < 1e-5 and e2 < 1e-5, (e1, e2)
    assert rel_l2(got[1], got[2]) < 1e-5
    fn = gpulib.nfft_gb_tma_wait_timeouts
    fn.restype = C.c_ulonglong
    assert fn() == 0


@pytest.mark.parametrize("N,n", [([32, 32], [64, 64]), ([32, 32], [96, 66]), ([32, 32], [64, 65]),
                                 ([16, 16], [40, 48])])
def test_2d_single_grids_with_and_without_tma_tiles(gpulib, N, n):
    """The 2-D single-precision column kernels on grids where B's TMA staging
    does not always apply: an odd last grid length (no tensor map: every tile
    staged cell by cell), grids smaller than the padded tile (every tile
    wraps around the grid edge) and mixes of interior and edge tiles.  Both
    transforms against the oracle; no bounded TMA wait may have given up."""
    import ctypes as C
    M, m = 3000, 6
    x, fh, f = seeded_case(N, M, seed=37)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    got_f, got_fh = run_both(p, x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64))
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    e_t = rel_l2(got_f.astype(np.complex128), o.trafo(fh.astype(np.complex64).astype(np.complex128)))
    e_a = rel_l2(got_fh.astype(np.complex128), o.adjoint(f.astype(np.complex64).astype(np.complex128)))
    o.close()
    assert e_t < 1e-5 and e_a < 1e-5, (n, e_t, e_a)
    fn = gpulib.nfft_gb_tma_wait_timeouts
    fn.restype = C.c_ulonglong
    assert fn() == 0


def _sweep_cases(count=10, seed=2024):
    """Seeded random single-precision 3-D plans for the column kernels (m = 4):
    N_t even in 8..40, n_t = sigma N_t with sigma in [1.5, 2.5] (odd n_t
    included), M in 200..60000, uniform or clustered nodes."""
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(count):
        N = [int(2 * rng.integers(4, 21)) for _ in range(3)]
        n = [max(int(np.ceil(rng.uniform(1.5, 2.5) * v)), 16) for v in N]
        M = int(rng.integers(200, 60001))
        dist = "clustered" if rng.random() < 0.3 else "uniform"
        cases.append((N, n, M, dist))
    return cases


@pytest.mark.parametrize("N,n,M,dist", _sweep_cases())
def test_3d_single_random_plans_both_b_kernels(gpulib, N, n, M, dist):
    """Random single-precision 3-D plans: trafo with either B kernel
    (column segments and sub-cell units) and the adjoint, against the oracle."""
    import ctypes as C
    from nfft_gb300 import workloads
    m = 4
    rng = np.random.default_rng(M)
    x = workloads.cube_nodes(M, 3, dist, int(M % 97)).astype(np.float64)
    NN = int(np.prod(N))
    fh = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    p.x[:] = x.astype(np.float32)
    p.precompute_one_psi()
    pa = C.addressof(p.p)
    setk = gpulib.nfftf_gb_set_b3_kernel
    setk.restype, setk.argtypes = C.c_int, [C.c_void_p, C.c_int]
    o = oracle.OraclePlan(N, M, n=n, m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    want_t = o.trafo(fh.astype(np.complex128))
    want_a = o.adjoint(f.astype(np.complex128))
    o.close()
    errs = []
    for mode in (1, 2):
        if setk(pa, mode) != 0:  # a plan without the 3-D column kernels: one B only
            continue
        p.f_hat[:] = fh
        p.trafo()
        errs.append(rel_l2(p.f.astype(np.complex128), want_t))
    p.f[:] = f
    p.adjoint()
    e_a = rel_l2(p.f_hat.astype(np.complex128), want_a)
    p.finalize()
    print(N, n, M, dist, "trafo", ["%.2e" % e for e in errs], "adjoint %.2e" % e_a)
    assert all(e < 1e-5 for e in errs), errs
    assert e_a < 1e-5, e_a
    fn = gpulib.nfft_gb_tma_wait_timeouts
    fn.restype = C.c_ulonglong
    assert fn() == 0


def _sweep_cases_2d(seed=2025):
    """Seeded random single-precision 2-D plans, one per column-kernel width
    (m = 2 ... 7, w = 2m + 2): N_t even in 32..96, n_t = sigma N_t with sigma
    in [1.5, 2.5] (odd n_t included), M in 500..40000."""
    rng = np.random.default_rng(seed)
    cases = []
    for m in range(2, 8):
        N = [int(2 * rng.integers(16, 49)) for _ in range(2)]
        n = [int(np.ceil(rng.uniform(1.5, 2.5) * v)) for v in N]
        cases.append((N, n, int(rng.integers(500, 40001)), m))
    return cases


@pytest.mark.parametrize("N,n,M,m", _sweep_cases_2d())
def test_2d_single_random_plans_every_width(gpulib, N, n, M, m):
    """Random single-precision 2-D plans, every window width of the column
    kernels: trafo and adjoint against the oracle."""
    import ctypes as C
    x, fh, f = seeded_case(N, M, seed=M)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    got_f, got_fh = run_both(p, x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64))
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    e_t = rel_l2(got_f.astype(np.complex128), o.trafo(fh.astype(np.complex64).astype(np.complex128)))
    e_a = rel_l2(got_fh.astype(np.complex128), o.adjoint(f.astype(np.complex64).astype(np.complex128)))
    o.close()
    print(N, n, M, m, "trafo %.2e adjoint %.2e" % (e_t, e_a))
    assert e_t < 1e-5 and e_a < 1e-5, (e_t, e_a)
    fn = gpulib.nfft_gb_tma_wait_timeouts
    fn.restype = C.c_ulonglong
    assert fn() == 0


def _sweep_cases_fp64(seed=2026):
    """Seeded random double-precision plans, four per dimension: N_t even and
    above m, n_t = sigma N_t with sigma in [1.5, 2.5] (odd n_t included, at
    least 2m + 3), m in 2..8, M in 100..20000, uniform nodes; every second
    plan sorts its nodes."""
    rng = np.random.default_rng(seed)
    cases = []
    lim = {1: (8, 129), 2: (4, 33), 3: (3, 11)}
    for d in (1, 2, 3):
        for k in range(4):
            m = int(rng.integers(2, 9))
            lo, hi = lim[d]
            N = [int(2 * rng.integers(max(lo, m // 2 + 1), hi)) for _ in range(d)]
            n = [max(int(np.ceil(rng.uniform(1.5, 2.5) * v)), 2 * m + 3) for v in N]
            cases.append((N, n, int(rng.integers(100, 20001)), m, k % 2 == 1))
    return cases


@pytest.mark.parametrize("N,n,M,m,sort", _sweep_cases_fp64())
def test_double_random_plans(gpulib, N, n, M, m, sort):
    """Random double-precision plans of every dimension: trafo and adjoint
    against the oracle to 1e-12, index_x bit for bit where the nodes are
    sorted."""
    x, fh, f = seeded_case(N, M, seed=M + 7)
    flags = default_guru_flags() | (abi.NFFT_SORT_NODES if sort else 0)
    p = make_plan(gpulib, False, N, M, m=m, n=n, flags=flags)
    gf, gfh = run_both(p, x, fh, f)
    idx = p.index_x if sort else None
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m, single=False)
    o.set_nodes(x)
    o.precompute()
    if sort:
        assert np.array_equal(idx, o.index_x())
    e_t, e_a = rel_l2(gf, o.trafo(fh)), rel_l2(gfh, o.adjoint(f))
    o.close()
    assert e_t < 1e-12 and e_a < 1e-12, (e_t, e_a)


def _sweep_cases_fp32_other(seed=2027):
    """Seeded random single-precision plans off the column kernels: 1-D
    (m in 2..8), 3-D with m in {2, 3, 5, 6} and 2-D with m = 8 (the tiled
    kernels); N_t even, n_t = sigma N_t with sigma in [1.5, 2.5] (odd n_t
    included), M in 100..20000."""
    rng = np.random.default_rng(seed)
    cases = []
    for d, ms, lo, hi in ((1, (2, 4, 6, 8), 8, 129), (3, (2, 3, 5, 6), 3, 11), (2, (8, 8), 8, 33)):
        for m in ms:
            N = [int(2 * rng.integers(max(lo, m // 2 + 1), hi)) for _ in range(d)]
            n = [max(int(np.ceil(rng.uniform(1.5, 2.5) * v)), 2 * m + 3) for v in N]
            cases.append((N, n, int(rng.integers(100, 20001)), m))
    return cases


@pytest.mark.parametrize("N,n,M,m", _sweep_cases_fp32_other())
def test_single_random_plans_tiled_paths(gpulib, N, n, M, m):
    """Random single-precision plans on the tiled kernels: trafo and adjoint
    against the oracle (FP64, on the single-precision inputs) to 2e-5, and
    index_x bit for bit."""
    x, fh, f = seeded_case(N, M, seed=M + 11)
    x32, fh32, f32 = x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64)
    p = make_plan(gpulib, True, N, M, m=m, n=n, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    gf, gfh = run_both(p, x32, fh32, f32)
    idx = p.index_x
    p.finalize()
    o = oracle.OraclePlan(N, M, n=n, m=m, single=True)
    o.set_nodes(x32)
    o.precompute()
    assert np.array_equal(idx, o.index_x())
    o.close()
    od = oracle.OraclePlan(N, M, n=n, m=m, single=False)
    od.set_nodes(x32.astype(np.float64))
    od.precompute()
    e_t = rel_l2(gf.astype(np.complex128), od.trafo(fh32.astype(np.complex128)))
    e_a = rel_l2(gfh.astype(np.complex128), od.adjoint(f32.astype(np.complex128)))
    od.close()
    assert e_t < 2e-5 and e_a < 2e-5, (e_t, e_a)
