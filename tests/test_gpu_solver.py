"""GPU parity of the inverse NFFT solver (solver_* / solverf_* over GPU plans).

The reference has no unit test for its solver; these tests pin the GPU
iteration to the reference library's own iterates (tests/golden/refrun.npz,
recorded from kernel/solver/solver.c compiled in place) and to the oracle.
"""
import numpy as np
import pytest

import oracle
from helpers import default_guru_flags, next_pow2, rel_l2, seeded_case
from nfft_gb300 import abi
from nfft_gb300.plan import Plan, Solver

pytestmark = pytest.mark.gpu


def gpu_plan(lib, single, N, M, m, x):
    n = [2 * next_pow2(v) for v in N]
    p = Plan(lib, single, N, M, n=n, m=m, flags=default_guru_flags() | abi.NFFT_SORT_NODES)
    p.x[:] = x
    p.precompute_one_psi()
    return p


def test_solver_matches_reference_iterates(gpulib, refrun):
    names = sorted({k.split("/")[0] for k in refrun if k.endswith("/f_hat_iter")})
    assert len(names) >= 4
    for name in names:
        meta = refrun[name + "/meta"]
        m, single, sflags, N = int(meta[0]), bool(meta[1]), int(meta[2]), [int(v) for v in meta[3:]]
        iters = refrun[name + "/f_hat_iter"]
        scal = refrun[name + "/scalars"]
        y = refrun[name + "/y"]
        M = len(y)
        x, _, _ = seeded_case(N, M, seed=5)
        p = gpu_plan(gpulib, single, N, M, m, x)
        s = Solver(p, sflags)
        s.y[:] = y
        if sflags & abi.PRECOMPUTE_WEIGHT:
            s.w[:] = refrun[name + "/w"]
        if sflags & abi.PRECOMPUTE_DAMP:
            s.w_hat[:] = refrun[name + "/w_hat"]
        s.f_hat_iter[:] = 0
        s.before_loop()
        tol = 2e-4 if single else 1e-10
        assert abs(s.scalars()["dot_r"] - scal[0][2]) <= tol * abs(scal[0][2])
        for it in range(1, iters.shape[0]):
            s.loop_one_step()
            assert rel_l2(s.f_hat_iter, iters[it]) < tol * it, (name, it, rel_l2(s.f_hat_iter, iters[it]))
            sc = s.scalars()
            for k, key in enumerate(("alpha", "beta", "dot_r")):
                ref = scal[it][k]
                assert abs(sc[key] - ref) <= 10 * tol * it * abs(ref) + 1e-30, (name, it, key, sc[key], ref)
        s.finalize()
        p.finalize()


def _oracle_landweber_sd(N, M, m, x, y, flags, alpha, iters):
    """Landweber / steepest descent restated on the oracle's transforms
    (kernel/solver/solver.c:128-229)."""
    o = oracle.OraclePlan(N, M, n=[2 * next_pow2(v) for v in N], m=m)
    o.set_nodes(x)
    o.precompute()
    fh = np.zeros(o.N_total, complex)
    r = y - o.trafo(fh)
    z = o.adjoint(r)
    out = []
    for _ in range(iters):
        if flags & abi.LANDWEBER:
            fh = fh + alpha * z
            r = y - o.trafo(fh)
            z = o.adjoint(r)
        else:
            v = o.trafo(z)
            a = np.vdot(z, z).real / np.vdot(v, v).real
            fh = fh + a * z
            r = r - a * v
            z = o.adjoint(r)
        out.append(fh.copy())
    return out


@pytest.mark.parametrize("flags", [abi.LANDWEBER | abi.NORMS_FOR_LANDWEBER, abi.STEEPEST_DESCENT])
def test_landweber_and_steepest_descent(gpulib, flags):
    N, M, m = [16, 16], 300, 6
    x, _, y = seeded_case(N, M, seed=8)
    p = gpu_plan(gpulib, False, N, M, m, x)
    s = Solver(p, flags)
    s.y[:] = y
    s.f_hat_iter[:] = 0
    alpha = 1e-4
    s.s.alpha_iter = alpha
    s.before_loop()
    ref = _oracle_landweber_sd(N, M, m, x, y, flags, alpha, 4)
    for it in range(4):
        s.s.alpha_iter = alpha if flags & abi.LANDWEBER else s.s.alpha_iter
        s.loop_one_step()
        assert rel_l2(s.f_hat_iter, ref[it]) < 1e-10, it
    s.finalize()
    p.finalize()


def test_single_precision_refresh_converges(gpulib):
    """FP32 CGNR with FP64 inner products and an FP64 residual refresh."""
    lib = gpulib
    N, M, m = [32, 32], 3000, 6
    rng = np.random.default_rng(3)
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f_true = rng.uniform(-1, 1, 1024) + 1j * rng.uniform(-1, 1, 1024)
    o = oracle.OraclePlan(N, M, n=[64, 64], m=m)
    o.set_nodes(x.astype(np.float32).astype(np.float64))
    o.precompute()
    y = o.trafo(f_true)
    p = gpu_plan(lib, True, N, M, m, x.astype(np.float32))
    s = Solver(p, abi.CGNR)
    import ctypes
    refresh = getattr(lib, "solverf_gb_set_refresh")
    refresh.argtypes = [ctypes.c_void_p, ctypes.c_int]
    refresh.restype = ctypes.c_int
    assert refresh(ctypes.addressof(s.s), 5) == 0
    s.y[:] = y
    s.f_hat_iter[:] = 0
    s.before_loop()
    for _ in range(40):
        s.loop_one_step()
    err = rel_l2(s.f_hat_iter.astype(np.complex128), f_true)
    s.finalize()
    p.finalize()
    assert err < 1e-3, err


def _set_graphs(lib, s, single, on):
    import ctypes
    fn = getattr(lib, ("solverf_" if single else "solver_") + "gb_set_graphs")
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
    fn.restype = ctypes.c_int
    assert fn(ctypes.addressof(s.s), int(on)) == 0


@pytest.mark.parametrize("single", [False, True])
@pytest.mark.parametrize("flags", [abi.CGNR | abi.PRECOMPUTE_WEIGHT | abi.PRECOMPUTE_DAMP, abi.CGNE,
                                   abi.STEEPEST_DESCENT | abi.PRECOMPUTE_WEIGHT])
def test_graph_steps_match_launched_steps(gpulib, single, flags):
    """Steps replayed from the captured CUDA graph give the iterates and
    scalars of the same steps launched one by one, also across a change of
    the nodes (precompute_one_psi again), which re-captures the graph.  The
    adjoint's atomic accumulation orders its additions differently from run
    to run, so two runs agree to rounding, not bit for bit."""
    N, M, m = [32, 32], 2500, 6
    x, _, y = seeded_case(N, M, seed=21)
    x2, _, _ = seeded_case(N, M, seed=22)
    rng = np.random.default_rng(4)
    w = rng.uniform(0.5, 1.5, M)
    wh = rng.uniform(0.5, 1.5, 1024)
    dt = np.float32 if single else np.float64
    runs = []
    for graphs in (True, False):
        p = gpu_plan(gpulib, single, N, M, m, x.astype(dt))
        s = Solver(p, flags)
        _set_graphs(gpulib, s, single, graphs)
        s.y[:] = y
        if flags & abi.PRECOMPUTE_WEIGHT:
            s.w[:] = w
        if flags & abi.PRECOMPUTE_DAMP:
            s.w_hat[:] = wh
        s.f_hat_iter[:] = 0
        s.before_loop()
        out = []
        for it in range(6):
            if it == 3:
                p.x[:] = x2.astype(dt)
                p.precompute_one_psi()
            s.loop_one_step()
            out.append((s.f_hat_iter.copy(), tuple(s.scalars().values())))
        s.finalize()
        p.finalize()
        runs.append(out)
    tol = 1e-4 if single else 1e-11
    for it, ((fa, sa), (fb, sb)) in enumerate(zip(*runs)):
        assert rel_l2(fa, fb) < tol, (it, rel_l2(fa, fb))
        for a, b in zip(sa, sb):
            assert abs(a - b) <= 10 * tol * abs(b) + 1e-30, (it, a, b)


@pytest.mark.parametrize("single", [False, True])
def test_multi_step_call_matches_single_steps(gpulib, single):
    """solver[f]_gb_loop_steps(k) leaves the iterate and scalars of k
    loop_one_step calls (to rounding: the adjoint's atomic accumulation) and
    reports dot_r of every step."""
    from nfft_gb300 import infft
    N, M, m = [32, 32], 2500, 6
    x, _, y = seeded_case(N, M, seed=23)
    dt = np.float32 if single else np.float64
    a = infft.CGNR(gpulib, single, N, x.astype(dt), m, y, refresh=3 if single else 0)
    a.set_sync(2)
    a.before_loop()
    dots = []
    for _ in range(7):
        a.step()
        dots.append(a.dot_r)
    fa = a.f_hat.copy()
    a.close()
    b = infft.CGNR(gpulib, single, N, x.astype(dt), m, y, refresh=3 if single else 0)
    b.set_sync(2)
    b.before_loop()
    hist = b.steps(7)
    fb = b.f_hat.copy()
    db = b.dot_r
    b.close()
    tol = 1e-4 if single else 1e-11
    assert rel_l2(fb, fa) < tol
    assert np.allclose(hist, dots, rtol=10 * tol)
    assert abs(db - dots[-1]) <= 10 * tol * abs(dots[-1])
