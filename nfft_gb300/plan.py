"""Host-side mirror of the NFFT plan interface.

``Plan`` drives an ``nfft_plan`` / ``nfftf_plan`` through the C ABI exactly the
way C callers of the reference do (examples/nfft/simple_test.c.in,
tests/nfft.c:300-360): init, fill ``x``, ``precompute_one_psi``, fill
``f_hat`` or ``f``, ``trafo`` / ``adjoint``, read the other vector, finalize.
Because the ABI is the reference's, the same class drives the GPU library and
the reference library built in place as an oracle.

``Solver`` does the same for ``solver_plan_complex`` (include/nfft3.h:760-786).
"""
import ctypes as C

import numpy as np

from . import abi


def _view(ptr, n, dtype):
    if not ptr or n == 0:
        return np.zeros(0, dtype=dtype)
    base = np.ctypeslib.as_array(ptr, shape=(int(n),))
    return base.view(dtype) if dtype != base.dtype else base


class Plan:
    """One NFFT plan of dimension d behind the C ABI of ``lib``.

    init: "guru" (nfft_init_guru with n, m, flags), "default" (nfft_init) or
    "1d"/"2d"/"3d" (nfft_init_1d/2d/3d).
    """

    def __init__(self, lib, single, N, M, n=None, m=None, flags=None,
                 fftw_flags=None, init="guru"):
        self.prec = abi.SINGLE if single else abi.DOUBLE
        self.lib = lib
        self.fn = abi.bind(lib, self.prec)
        self.N = [int(v) for v in N]
        self.d = len(self.N)
        self.M = int(M)
        self.p = self.prec.plan()
        self._pp = C.byref(self.p)
        Nc = (C.c_int * self.d)(*self.N)
        if init == "guru":
            if n is None:
                n = [2 * int(self.fn["next_power_of_2"](v)) for v in self.N]
            if m is None:
                m = int(self.fn["get_default_window_cut_off"]())
            if flags is None:
                flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT
                         | abi.MALLOC_F | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE)
                if self.d > 1:
                    flags |= abi.NFFT_SORT_NODES
            if fftw_flags is None:
                fftw_flags = abi.FFTW_ESTIMATE | abi.FFTW_DESTROY_INPUT
            nc = (C.c_int * self.d)(*[int(v) for v in n])
            self.fn["init_guru"](self._pp, self.d, Nc, self.M, nc, int(m), int(flags), int(fftw_flags))
        elif init == "default":
            self.fn["init"](self._pp, self.d, Nc, self.M)
        elif init in ("1d", "2d", "3d"):
            self.fn["init_" + init](self._pp, *self.N, self.M)
        else:
            raise ValueError("unknown init %r" % init)
        self._alive = True

    # ---- fields ----
    @property
    def n(self):
        return [int(self.p.n[t]) for t in range(self.d)]

    @property
    def m(self):
        return int(self.p.m)

    @property
    def flags(self):
        return int(self.p.flags)

    @property
    def N_total(self):
        return int(self.p.N_total)

    @property
    def x(self):
        return _view(self.p.x, self.M * self.d, np.dtype(self.prec.np_real)).reshape(self.M, self.d)

    @property
    def f_hat(self):
        return _view(self.p.f_hat, 2 * self.N_total, np.dtype(self.prec.np_real)).view(self.prec.np_complex)

    @property
    def f(self):
        return _view(self.p.f, 2 * self.M, np.dtype(self.prec.np_real)).view(self.prec.np_complex)

    @property
    def index_x(self):
        if not self.p.index_x:
            return None
        return np.ctypeslib.as_array(self.p.index_x, shape=(2 * self.M,)).copy()

    @property
    def c_phi_inv(self):
        if not self.p.c_phi_inv:
            return None
        return [np.ctypeslib.as_array(self.p.c_phi_inv[t], shape=(self.N[t],)).copy()
                for t in range(self.d)]

    @property
    def measure_time(self):
        return [float(v) for v in self.p.MEASURE_TIME_t]

    # ---- calls ----
    def precompute_one_psi(self):
        if self.p.flags & abi.PRE_ONE_PSI:
            self.fn["precompute_one_psi"](self._pp)

    def check(self):
        r = self.fn["check"](self._pp)
        return None if r is None else r.decode()

    def trafo(self):
        self.fn["trafo"](self._pp)

    def adjoint(self):
        self.fn["adjoint"](self._pp)

    def trafo_direct(self):
        self.fn["trafo_direct"](self._pp)

    def adjoint_direct(self):
        self.fn["adjoint_direct"](self._pp)

    def call(self, name):
        self.fn[name](self._pp)

    def finalize(self):
        if self._alive:
            self.fn["finalize"](self._pp)
            self._alive = False

    def __del__(self):
        try:
            self.finalize()
        except Exception:
            pass


class Solver:
    """solver_plan_complex over a Plan (the plan is the mv operator)."""

    def __init__(self, plan, flags=abi.CGNR):
        self.plan = plan
        self.prec = plan.prec
        self.fn = plan.fn
        self.s = self.prec.solver()
        self._sp = C.byref(self.s)
        mv = C.cast(C.pointer(plan.p), C.POINTER(self.prec.mv))
        self.fn["solver_init_advanced_complex"](self._sp, mv, int(flags))
        self.flags = int(flags)
        self._alive = True

    def _cvec(self, name, n):
        return _view(getattr(self.s, name), 2 * n, np.dtype(self.prec.np_real)).view(self.prec.np_complex)

    @property
    def y(self):
        return self._cvec("y", self.plan.M)

    @property
    def f_hat_iter(self):
        return self._cvec("f_hat_iter", self.plan.N_total)

    @property
    def r_iter(self):
        return self._cvec("r_iter", self.plan.M)

    @property
    def w(self):
        return _view(self.s.w, self.plan.M, np.dtype(self.prec.np_real))

    @property
    def w_hat(self):
        return _view(self.s.w_hat, self.plan.N_total, np.dtype(self.prec.np_real))

    def scalars(self):
        s = self.s
        return dict(alpha=s.alpha_iter, beta=s.beta_iter, dot_r=s.dot_r_iter,
                    dot_r_old=s.dot_r_iter_old, dot_z=s.dot_z_hat_iter,
                    dot_z_old=s.dot_z_hat_iter_old, dot_p=s.dot_p_hat_iter,
                    dot_v=s.dot_v_iter)

    def before_loop(self):
        self.fn["solver_before_loop_complex"](self._sp)

    def loop_one_step(self):
        self.fn["solver_loop_one_step_complex"](self._sp)

    def finalize(self):
        if self._alive:
            self.fn["solver_finalize_complex"](self._sp)
            self._alive = False

    def __del__(self):
        try:
            self.finalize()
        except Exception:
            pass


class NnPlan:
    """An NNFFT plan (nonequispaced space and frequency nodes, double
    precision) driven through the nnfft_* entry points of ``lib`` as C callers
    of the reference do (reference kernel/nnfft/nnfft.c): init_guru, fill x
    (M x d) and v (N_total x d), precompute_one_psi, fill f_hat or f,
    trafo / adjoint (or their _direct forms), read the other vector."""

    def __init__(self, lib, N, N_total, M, N1, m, flags):
        self.lib = lib
        self.d = len(N)
        self.N_total, self.M = int(N_total), int(M)
        self.p = abi.nnfft_plan()
        for name in ("init_guru", "trafo", "adjoint", "trafo_direct", "adjoint_direct",
                     "precompute_one_psi", "finalize"):
            fn = getattr(lib, "nnfft_" + name)
            fn.restype = None
        Nc = (C.c_int * self.d)(*[int(v) for v in N])
        N1c = (C.c_int * self.d)(*[int(v) for v in N1])
        lib.nnfft_init_guru(C.byref(self.p), self.d, self.N_total, self.M, Nc, N1c, int(m), C.c_uint(flags))
        self.x = _view(self.p.x, self.M * self.d, np.float64)
        self.v = _view(self.p.v, self.N_total * self.d, np.float64)
        self.f = _view(self.p.f, 2 * self.M, np.float64).view(np.complex128)
        self.f_hat = _view(self.p.f_hat, 2 * self.N_total, np.float64).view(np.complex128)

    def _call(self, name):
        getattr(self.lib, "nnfft_" + name)(C.byref(self.p))

    def precompute_one_psi(self):
        self._call("precompute_one_psi")

    def trafo(self):
        self._call("trafo")

    def adjoint(self):
        self._call("adjoint")

    def trafo_direct(self):
        self._call("trafo_direct")

    def adjoint_direct(self):
        self._call("adjoint_direct")

    def finalize(self):
        if self.p is not None:
            self._call("finalize")
            self.p = None


class MriPlan:
    """An MRI operator with a field inhomogeneity (kind "2d1d" or "3d",
    double precision) driven through the mri_inh_* entry points of ``lib``
    (reference kernel/mri/mri.c): init_guru, fill plan.x (the k-space nodes,
    M x 2 for 2d1d, M x 3 for 3d), nfft_precompute_one_psi on the embedded
    plan, t (2d1d: sample times) and w (field map), then trafo / adjoint."""

    def __init__(self, lib, kind, N, M, n, m, sigma, flags, fftw_flags=None):
        self.lib, self.kind = lib, kind
        self.M = int(M)
        self.p = (abi.mri_inh_2d1d_plan if kind == "2d1d" else abi.mri_inh_3d_plan)()
        pre = "mri_inh_%s_" % kind
        self._fn = {k: getattr(lib, pre + k) for k in ("init_guru", "trafo", "adjoint", "finalize")}
        for fn in self._fn.values():
            fn.restype = None
        self._fn["init_guru"].argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int,
                                          C.c_double, C.c_uint, C.c_uint]
        if fftw_flags is None:
            fftw_flags = abi.FFTW_ESTIMATE | abi.FFTW_DESTROY_INPUT
        d = 2 if kind == "2d1d" else 3
        Nc = (C.c_int * 3)(*[int(v) for v in N])
        nc = (C.c_int * d)(*[int(v) for v in n])
        self._fn["init_guru"](C.addressof(self.p), Nc, self.M, nc, int(m), float(sigma), int(flags), int(fftw_flags))
        self.N_total = int(self.p.N_total)
        self.d = d
        self.x = _view(self.p.plan.x, self.M * d, np.float64)
        self.w = _view(self.p.w, self.N_total, np.float64)
        self.t = _view(self.p.t, self.M, np.float64) if kind == "2d1d" else None
        pc = getattr(lib, "nfft_precompute_one_psi")
        pc.restype = None
        self._precompute = pc

    @property
    def f(self):
        return _view(self.p.f, 2 * self.M, np.float64).view(np.complex128)

    @property
    def f_hat(self):
        return _view(self.p.f_hat, 2 * self.N_total, np.float64).view(np.complex128)

    def precompute(self):
        self._precompute(C.pointer(self.p.plan))  # the embedded plan, in place

    def trafo(self):
        self._fn["trafo"](C.c_void_p(C.addressof(self.p)))

    def adjoint(self):
        self._fn["adjoint"](C.c_void_p(C.addressof(self.p)))

    def finalize(self):
        if self.p is not None:
            self._fn["finalize"](C.c_void_p(C.addressof(self.p)))
            self.p = None


class TrigPlan:
    """An NFCT or NFST plan (kind "nfct" or "nfst") driven through the nfct_* / nfctf_* entry
    points (or nfst_* / nfstf_*) of ``lib`` as C callers of the reference do
    (reference kernel/nfct/nfct.c, kernel/nfst/nfst.c): init_guru, fill x (M x d in [0, 1/2)),
    precompute_one_psi, fill f_hat (real, N_total) or f, trafo / adjoint or
    their _direct forms."""

    def __init__(self, lib, kind, single, N, M, n=None, m=None, flags=None, fftw_flags=None):
        self.lib = lib
        self.pfx = kind + ("f_" if single else "_")
        self.dt = np.float32 if single else np.float64
        self.p = (getattr(abi, kind + ("f_plan" if single else "_plan")))()
        self.d = len(N)
        self.M = int(M)
        if fftw_flags is None:
            fftw_flags = abi.FFTW_ESTIMATE | abi.FFTW_DESTROY_INPUT
        Nc = (C.c_int * self.d)(*[int(v) for v in N])
        if n is None:  # the reference's defaults (X(init): n, m and flags chosen by the library)
            fn = getattr(lib, self.pfx + "init")
            fn.restype = None
            fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int]
            fn(C.addressof(self.p), self.d, Nc, self.M)
        else:
            fn = getattr(lib, self.pfx + "init_guru")
            fn.restype = None
            fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int,
                           C.c_uint, C.c_uint]
            nc = (C.c_int * self.d)(*[int(v) for v in n])
            fn(C.addressof(self.p), self.d, Nc, self.M, nc, int(m), int(flags), int(fftw_flags))
        self.N_total = int(self.p.N_total)
        self.x = _view(self.p.x, self.M * self.d, self.dt)
        self.f = _view(self.p.f, self.M, self.dt)
        self.f_hat = _view(self.p.f_hat, self.N_total, self.dt)

    def _call(self, name):
        fn = getattr(self.lib, self.pfx + name)
        fn.restype = C.c_char_p if name == "check" else None
        return fn(C.c_void_p(C.addressof(self.p)))

    def precompute_one_psi(self):
        self._call("precompute_one_psi")

    def trafo(self):
        self._call("trafo")

    def adjoint(self):
        self._call("adjoint")

    def trafo_direct(self):
        self._call("trafo_direct")

    def adjoint_direct(self):
        self._call("adjoint_direct")

    def check(self):
        r = self._call("check")
        return r.decode() if r else None

    def finalize(self):
        if self.p is not None:
            self._call("finalize")
            self.p = None
