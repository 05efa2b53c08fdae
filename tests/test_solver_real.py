"""solver_*_double / solverf_*_double: the solver iterations over a real
operator (reference kernel/solver/solver.c:392-736), run here around a dense
random matrix given as an mv_plan_double with ctypes callbacks.  The
iterates (alpha, beta, the residual norms and f_hat_iter) are compared step by
step with the reference's own solver compiled in place (oracle/_ref), and
CGNR is checked to reach the least-squares solution."""
import ctypes as C

import numpy as np
import pytest

import nfft_gb300
import oracle
from nfft_gb300 import abi

FLAGS = [
    abi.CGNR,
    abi.CGNR | abi.PRECOMPUTE_WEIGHT | abi.PRECOMPUTE_DAMP,
    abi.CGNE,
    abi.CGNE | abi.PRECOMPUTE_WEIGHT | abi.PRECOMPUTE_DAMP,
    abi.LANDWEBER | abi.NORMS_FOR_LANDWEBER,
    abi.STEEPEST_DESCENT | abi.PRECOMPUTE_WEIGHT,
]
CB = C.CFUNCTYPE(None, C.c_void_p)


class RealRun:
    """One solver over the operator A through the solver_*_double entry points of lib."""

    def __init__(self, lib, single, A, flags, y, w, w_hat):
        self.R = C.c_float if single else C.c_double
        self.dt = np.float32 if single else np.float64
        mvt = abi.nfftf_mv_plan_double if single else abi.nfft_mv_plan_double
        spt = abi.solverf_plan_double if single else abi.solver_plan_double
        pfx = "solverf_" if single else "solver_"
        M, N = A.shape
        self.A = A.astype(self.dt)
        self.buf_fh = np.zeros(N, self.dt)
        self.buf_f = np.zeros(M, self.dt)
        self.mv = mvt()
        self.mv.N_total, self.mv.M_total = N, M
        self.mv.f_hat = self.buf_fh.ctypes.data_as(C.POINTER(self.R))
        self.mv.f = self.buf_f.ctypes.data_as(C.POINTER(self.R))

        def trafo(_):
            fh = np.ctypeslib.as_array(self.mv.f_hat, shape=(N,))
            f = np.ctypeslib.as_array(self.mv.f, shape=(M,))
            f[:] = (self.A.astype(np.float64) @ fh.astype(np.float64)).astype(self.dt)

        def adjoint(_):
            fh = np.ctypeslib.as_array(self.mv.f_hat, shape=(N,))
            f = np.ctypeslib.as_array(self.mv.f, shape=(M,))
            fh[:] = (self.A.astype(np.float64).T @ f.astype(np.float64)).astype(self.dt)

        self._cb = (CB(trafo), CB(adjoint))
        self.mv.mv_trafo = C.cast(self._cb[0], C.c_void_p)
        self.mv.mv_adjoint = C.cast(self._cb[1], C.c_void_p)
        self.sp = spt()
        self.fn = {k: getattr(lib, pfx + k) for k in
                   ("init_advanced_double", "before_loop_double", "loop_one_step_double", "finalize_double")}
        self.fn["init_advanced_double"](C.byref(self.sp), C.byref(self.mv), C.c_uint(flags))
        np.ctypeslib.as_array(self.sp.y, shape=(M,))[:] = y
        np.ctypeslib.as_array(self.sp.f_hat_iter, shape=(N,))[:] = 0
        if flags & abi.PRECOMPUTE_WEIGHT:
            np.ctypeslib.as_array(self.sp.w, shape=(M,))[:] = w
        if flags & abi.PRECOMPUTE_DAMP:
            np.ctypeslib.as_array(self.sp.w_hat, shape=(N,))[:] = w_hat
        self.N = N

    def state(self):
        sp = self.sp
        return (sp.alpha_iter, sp.beta_iter, sp.dot_r_iter, sp.dot_z_hat_iter,
                np.ctypeslib.as_array(sp.f_hat_iter, shape=(self.N,)).astype(np.float64).copy())

    def run(self, steps):
        self.fn["before_loop_double"](C.byref(self.sp))
        out = [self.state()]
        for _ in range(steps):
            self.fn["loop_one_step_double"](C.byref(self.sp))
            out.append(self.state())
        self.fn["finalize_double"](C.byref(self.sp))
        return out


def _problem(seed=3, M=60, N=24):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, N)) / np.sqrt(M)
    y = rng.standard_normal(M)
    w = rng.uniform(0.5, 1.5, M)
    w_hat = rng.uniform(0.5, 1.5, N)
    return A, y, w, w_hat


@pytest.mark.parametrize("single", [False, True])
@pytest.mark.parametrize("flags", FLAGS)
def test_real_solver_matches_reference(flags, single):
    ref = oracle.load_reference(single)
    if ref is None:
        pytest.skip("reference library not built here")
    A, y, w, w_hat = _problem()
    if flags & abi.LANDWEBER:
        A = A * 0.5  # Landweber with alpha = 1 needs ||A|| < sqrt(2)
    ours = RealRun(nfft_gb300.lib(), single, A, flags, y, w, w_hat)
    theirs = RealRun(ref, single, A, flags, y, w, w_hat)
    if flags & abi.LANDWEBER:
        ours.sp.alpha_iter = theirs.sp.alpha_iter = 1.0
    a, b = ours.run(6), theirs.run(6)
    rtol = 2e-4 if single else 1e-10
    for k, (sa, sb) in enumerate(zip(a, b)):
        for qa, qb in zip(sa[:4], sb[:4]):
            assert qa == pytest.approx(qb, rel=rtol, abs=1e-30), (k, sa[:4], sb[:4])
        assert np.allclose(sa[4], sb[4], rtol=rtol, atol=rtol * np.abs(sb[4]).max()), k


def test_real_cgnr_reaches_least_squares():
    A, y, _, _ = _problem(seed=5, M=80, N=20)
    run = RealRun(nfft_gb300.lib(), False, A, abi.CGNR, y, None, None)
    f = run.run(40)[-1][4]
    ls = np.linalg.lstsq(A, y, rcond=None)[0]
    assert np.linalg.norm(f - ls) / np.linalg.norm(ls) < 1e-10
