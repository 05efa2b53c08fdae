"""Inverse NFFT (CGNR) driver on the GPU library, for benchmarks and tests.

Runs the solver through the reference-facing C ABI (solver_* over nfft_*
plans, solverf_* over nfftf_* plans) with the library's extensions: timed
steps enqueued back to back (solver_gb_loop_steps), and an FP64 residual refresh for
single-precision solvers (r = y - A f recomputed by an FP64 transform every
`refresh` iterations, kernel/solver/solver.c:81-125 being the formula).
"""
import ctypes as C
import time

import numpy as np

from . import abi
from .plan import Plan, Solver

PLAN_FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
              | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE)


def _ext(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


def disk_damping(N):
    """Damping factors w_hat of the reference's MRI reconstruction
    (applications/mri/mri2d/reconstruct_data_2d.c: CGNR | PRECOMPUTE_DAMP):
    1 on the image's inscribed disk (pixel (j, k), j2 = j - N/2, k2 = k - N/2,
    sqrt(j2^2 + k2^2) <= N/2), 0 outside."""
    j = np.arange(N) - N // 2
    r = np.sqrt(j[:, None] ** 2 + j[None, :] ** 2)
    return (r <= N / 2).astype(np.float64).reshape(-1)


class CGNR:
    """CGNR on one plan; weights w (M) make it the weighted normal equations
    A^H W A f = A^H W y (PRECOMPUTE_WEIGHT); damping factors w_hat (N_total)
    enter as the reference's PRECOMPUTE_DAMP."""

    def __init__(self, lib, single, N, x, m, y, w=None, refresh=0, cgne=False, w_hat=None):
        self.lib = lib
        self.single = single
        M = len(x)
        n = [2 * (1 << (int(v) - 1).bit_length()) for v in N]
        self.plan = Plan(lib, single, N, M, n=n, m=m, flags=PLAN_FLAGS)
        self.plan.x[:] = x.astype(np.float32 if single else np.float64)
        self.plan.precompute_one_psi()
        flags = abi.CGNE if cgne else abi.CGNR
        if w is not None:
            flags |= abi.PRECOMPUTE_WEIGHT
        if w_hat is not None:
            flags |= abi.PRECOMPUTE_DAMP
        self.solver = Solver(self.plan, flags)
        self.solver.y[:] = y
        if w is not None:
            self.solver.w[:] = w
        if w_hat is not None:
            self.solver.w_hat[:] = w_hat
        self.solver.f_hat_iter[:] = 0
        pfx = "solverf_" if single else "solver_"
        self._set_sync = _ext(lib, pfx + "gb_set_sync", C.c_int, [C.c_void_p, C.c_int])
        self._sync = _ext(lib, pfx + "gb_sync", C.c_int, [C.c_void_p])
        self._refresh = _ext(lib, pfx + "gb_set_refresh", C.c_int, [C.c_void_p, C.c_int])
        self._steps = _ext(lib, pfx + "gb_loop_steps", C.c_int,
                           [C.c_void_p, C.c_int, C.POINTER(C.c_double)])
        self.addr = C.addressof(self.solver.s)
        if refresh:
            self._refresh(self.addr, int(refresh))

    def set_sync(self, level):
        self._set_sync(self.addr, int(level))

    def sync(self):
        self._sync(self.addr)

    def before_loop(self):
        self.solver.before_loop()

    def step(self):
        self.solver.loop_one_step()

    def steps(self, k):
        """k steps enqueued back to back (one host synchronisation at the
        end); returns dot_r after each step."""
        hist = np.zeros(k, dtype=np.float64)
        if k > 0:
            self._steps(self.addr, int(k), hist.ctypes.data_as(C.POINTER(C.c_double)))
        return hist

    @property
    def f_hat(self):
        return self.solver.f_hat_iter.astype(np.complex128)

    @property
    def dot_r(self):
        return float(self.solver.s.dot_r_iter)

    def close(self):
        self.solver.finalize()
        self.plan.finalize()


def fp64_solution(lib, N, x, m, y, w=None, max_iter=3000, rtol=1e-14, w_hat=None):
    """FP64 CGNR run to convergence (relative change of f below rtol)."""
    s = CGNR(lib, False, N, x, m, y, w=w, w_hat=w_hat)
    s.set_sync(1)
    s.before_loop()
    prev = s.f_hat.copy()
    it = 0
    for it in range(1, max_iter + 1):
        s.step()
        if it % 10 == 0:
            cur = s.f_hat
            ch = np.linalg.norm(cur - prev) / max(np.linalg.norm(cur), 1e-300)
            prev = cur.copy()
            if ch < rtol:
                break
    out = s.f_hat.copy()
    s.close()
    return out, it


def run_iterations(lib, single, N, x, m, y, iters, w=None, refresh=0, w_hat=None):
    """Run `iters` CGNR steps timed (enqueued back to back, one host
    synchronisation); returns (f_hat_iter after the last step, seconds,
    per-step dot_r)."""
    s = CGNR(lib, single, N, x, m, y, w=w, refresh=refresh if single else 0, w_hat=w_hat)
    s.set_sync(0)
    t0 = time.perf_counter()
    s.before_loop()
    dots = list(s.steps(iters))
    s.sync()
    t1 = time.perf_counter()
    out = s.f_hat.copy()
    s.close()
    return out, t1 - t0, dots


class TrueResidual:
    """||y - A f|| / ||y|| with A the FP64 transform of the same nodes: the
    residual a solver has actually reached, whatever precision it iterates
    in (a single-precision solver's own r_iter is updated recursively and can
    drift from it)."""

    def __init__(self, lib, N, x, m, y):
        n = [2 * (1 << (int(v) - 1).bit_length()) for v in N]
        self.plan = Plan(lib, False, N, len(x), n=n, m=m, flags=PLAN_FLAGS)
        self.plan.x[:] = np.asarray(x, dtype=np.float64)
        self.plan.precompute_one_psi()
        self.y = np.asarray(y, dtype=np.complex128)
        self.ny = np.linalg.norm(self.y)

    def __call__(self, f_hat):
        self.plan.f_hat[:] = f_hat
        self.plan.trafo()
        return float(np.linalg.norm(self.y - self.plan.f) / self.ny)

    def close(self):
        self.plan.finalize()


def image_errors(f, f_true, radius=0.45):
    """Relative image error against f_true over the whole image, and over the
    part of it the samples determine: the band of spatial frequencies
    |nu| <= radius (the trajectories sample the disk |x| <= 1/2 of the
    transform's domain [-1/2, 1/2)^2), from a DFT of the error on the N x N
    grid (N even, natural pixel order)."""
    N = int(round(np.sqrt(len(f_true))))
    j = np.arange(N) - N // 2
    band = (j[:, None] ** 2 + j[None, :] ** 2) <= (radius * N) ** 2

    def spec(v):
        return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(np.asarray(v).reshape(N, N))))

    E, F = spec(f - f_true), spec(f_true)
    return (float(np.linalg.norm(f - f_true) / np.linalg.norm(f_true)),
            float(np.linalg.norm(E[band]) / np.linalg.norm(F)))


def time_to_tolerance(lib, single, N, x, m, y, tol=1e-5, w=None, refresh=0, max_iter=3000, check_every=5):
    """Iterations and wall time for CGNR to bring the true relative data
    residual ||y - A f|| / ||y|| (A in FP64, TrueResidual) below tol.

    A first, untimed run checks the residual every check_every steps and
    finds the iteration count k; a second run of exactly k iterations is
    timed (the steps enqueued back to back, the iterate copied back once at
    the end).  The reference's own iterative reconstructions stop on their
    residual too (applications/mri/mri2d/reconstruct_data_2d.c:123-131).
    The two runs agree only to rounding: B^T adds the window contributions
    with atomics (in either precision), whose order varies from run to run,
    so the timed run's final residual can sit a fraction of a percent on
    either side of the first run's.
    Returns dict(iters, seconds, resid (the timed run's final residual),
    resid_found (the first run's at iters), reached (resid_found < tol), f)."""
    res = TrueResidual(lib, N, x, m, y)
    s = CGNR(lib, single, N, x, m, y, w=w, refresh=refresh if single else 0)
    s.set_sync(0)
    s.before_loop()
    k, r = 0, np.inf
    while k < max_iter:
        s.steps(check_every)
        s.sync()
        k += check_every
        r = res(s.f_hat)
        if r < tol:
            break
    s.close()
    reached = r < tol
    s = CGNR(lib, single, N, x, m, y, w=w, refresh=refresh if single else 0)
    s.set_sync(0)
    t0 = time.perf_counter()
    s.before_loop()
    s.steps(k)
    s.sync()
    t1 = time.perf_counter()
    f_end = s.f_hat.copy()
    s.close()
    r_end = res(f_end)
    res.close()
    return dict(iters=k, seconds=t1 - t0, resid=r_end, resid_found=float(r), reached=bool(reached), f=f_end)
