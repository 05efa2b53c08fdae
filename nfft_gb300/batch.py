"""Host wrapper of the batched 2-D transforms (nfftf_gb_batch_* in
include/nfft_gb300.h): many single-precision plans transformed by persistent
kernels over one device work queue, optionally replayed as a CUDA graph."""
import ctypes as C

import numpy as np

from . import abi
from .plan import Plan

PLAN_FLAGS = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
              | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE)


def _fn(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def cudart():
    """The CUDA runtime the library is linked against (already loaded)."""
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


class Batch:
    def __init__(self, lib, plans):
        vp = C.c_void_p
        self.lib = lib
        self.plans = plans
        self._create = _fn(lib, "nfftf_gb_batch_create", vp, [C.POINTER(vp), C.c_int])
        self._destroy = _fn(lib, "nfftf_gb_batch_destroy", None, [vp])
        self._autotune = _fn(lib, "nfftf_gb_batch_autotune", C.c_int, [vp, C.c_int])
        self._run = _fn(lib, "nfftf_gb_batch_run", C.c_int, [vp, C.c_int, C.c_int])
        self._time = _fn(lib, "nfftf_gb_batch_time", C.c_float, [vp, C.c_int, C.c_int])
        self._nodes = _fn(lib, "nfftf_gb_batch_nodes", C.c_longlong, [vp])
        self._items = _fn(lib, "nfftf_gb_batch_items", C.c_int, [vp])
        self._cfg = _fn(lib, "nfftf_gb_batch_plan_config", C.c_int,
                        [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)])
        self._set_cfg = _fn(lib, "nfftf_gb_batch_set_config", C.c_int, [vp, C.c_int, C.c_int, C.c_int])
        arr = (vp * len(plans))(*[C.addressof(p.p) for p in plans])
        self.h = self._create(arr, len(plans))
        if not self.h:
            raise RuntimeError("batch creation failed: %s" % lib.nfft_gb_last_error())

    def autotune(self, reps=3):
        return self._autotune(self.h, reps)

    def run(self, what=3, mode=0):
        return self._run(self.h, what, mode)

    def time(self, reps, mode):
        return float(self._time(self.h, reps, mode))

    @property
    def nodes(self):
        return int(self._nodes(self.h))

    @property
    def items(self):
        return int(self._items(self.h))

    def config(self, k):
        T, tpn = C.c_int(), C.c_int()
        self._cfg(self.h, k, C.byref(T), C.byref(tpn))
        return T.value, tpn.value

    def set_config(self, k, T, tpn):
        """Plan k on tiles of edge T with tpn threads per node, or (32, 0)
        for the column kernels; returns the library's status (0 = done)."""
        return self._set_cfg(self.h, k, T, tpn)

    def close(self):
        if self.h:
            self._destroy(self.h)
            self.h = None


def device_io(lib):
    """Copy helpers between numpy and a plan's device f_hat / f."""
    rt = cudart()
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaMemcpy.restype = C.c_int
    dfh = _fn(lib, "nfftf_gb_device_f_hat", C.c_void_p, [C.c_void_p])
    df = _fn(lib, "nfftf_gb_device_f", C.c_void_p, [C.c_void_p])

    def put(plan, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.complex64)
        dst = dfh(C.addressof(plan.p)) if which == "f_hat" else df(C.addressof(plan.p))
        assert rt.cudaMemcpy(dst, a.ctypes.data, a.nbytes, 1) == 0

    def get(plan, which, count):
        a = np.empty(count, dtype=np.complex64)
        src = dfh(C.addressof(plan.p)) if which == "f_hat" else df(C.addressof(plan.p))
        assert rt.cudaMemcpy(a.ctypes.data, src, a.nbytes, 2) == 0
        return a

    return put, get


def random_plans(lib, count, seed=0, sizes=(32, 64, 128, 256), mmin=1024, mmax=65536, ms=(4, 6)):
    """Plans of the batched workload: N_t log-uniform over `sizes`, m uniform
    over `ms`, M log-uniform in [mmin, mmax], nodes uniform (seeded per plan)."""
    rng = np.random.default_rng(seed)
    plans, data = [], []
    for k in range(count):
        N = [int(rng.choice(sizes)), int(rng.choice(sizes))]
        m = int(rng.choice(ms))
        M = int(np.exp(rng.uniform(np.log(mmin), np.log(mmax))))
        r = np.random.default_rng([seed, k])
        x = r.uniform(-0.5, 0.5, (M, 2)).astype(np.float32)
        p = Plan(lib, True, N, M, n=[2 * N[0], 2 * N[1]], m=m, flags=PLAN_FLAGS)
        p.x[:] = x
        p.precompute_one_psi()
        plans.append(p)
        data.append((N, m, M, x))
    return plans, data
