"""CPU oracle for the NFFT transform path -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package; the product library never uses it.

Two checkers live here:

* ``liborc_d.so`` / ``liborc_s.so``: the project-written C restatement of the
  reference algorithm (``nfft_oracle.c`` + ``fft_cpu.c``), built on any host;
* ``_ref/libnfft3_ref_{d,s}.so``: the reference NFFT's own C sources compiled
  in place (``ref/Makefile``) -- only where the reference checkout exists.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# The reference checkout: NFFT_REFERENCE_SRC, else a "reference" directory
# beside this repository's root.
REFERENCE_SRC = os.environ.get("NFFT_REFERENCE_SRC") or os.path.normpath(
    os.path.join(HERE, os.pardir, os.pardir, "reference"))

ORC_SORT = 1
ORC_BLOCKWISE = 2
ORC_PRE_PSI = 4
ORC_CGNR = 4
ORC_CGNE = 8
ORC_PRECOMPUTE_WEIGHT = 32
ORC_PRECOMPUTE_DAMP = 64


def _so(single):
    return os.path.join(HERE, "liborc_%s.so" % ("s" if single else "d"))


def build(force=False):
    """Compile the C restatement (both precisions) with gcc + OpenMP."""
    srcs = [os.path.join(HERE, "nfft_oracle.c"), os.path.join(HERE, "fft_cpu.c")]
    for single in (False, True):
        out = _so(single)
        if not force and os.path.exists(out) and all(
                os.path.getmtime(out) > os.path.getmtime(s) for s in srcs):
            continue
        cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-Wl,-Bsymbolic", "-o", out] + srcs + ["-lm"]
        if single:
            cmd.insert(1, "-DORC_SINGLE")
        subprocess.check_call(cmd)


def build_reference(force=False):
    """Compile the reference NFFT in place into _ref/ when its sources exist.

    Returns True when the libraries are present afterwards."""
    outs = [os.path.join(REF_DIR, "libnfft3_ref_%s.so" % s) for s in ("d", "s")]
    if not os.path.isdir(os.path.join(REFERENCE_SRC, "kernel", "nfft")):
        return all(os.path.exists(o) and _is_native(o) for o in outs)
    if force or not all(os.path.exists(o) and _is_native(o) for o in outs):
        for o in outs:
            if os.path.exists(o):
                os.remove(o)
        for o in outs:
            subprocess.check_call(["make", "-C", os.path.join(HERE, "ref"),
                                   "REF=" + REFERENCE_SRC, "../_ref/" + os.path.basename(o)],
                                  stdout=subprocess.DEVNULL)
    return all(os.path.exists(o) for o in outs)


def _is_native(path):
    """True when the shared object matches this host's machine type."""
    import platform
    try:
        with open(path, "rb") as fh:
            hdr = fh.read(20)
    except OSError:
        return False
    if len(hdr) < 20 or hdr[:4] != b"\x7fELF":
        return False
    mach = int.from_bytes(hdr[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or mach == want


_libs = {}


def load(single=False):
    """ctypes handle of the C restatement, built on demand."""
    key = ("orc", single)
    if key not in _libs:
        if not os.path.exists(_so(single)):
            build()
        lib = C.CDLL(_so(single))
        _declare(lib, "orcf_" if single else "orc_", C.c_float if single else C.c_double)
        _libs[key] = lib
    return _libs[key]


def load_reference(single=False):
    """ctypes handle of the reference library built in place, or None."""
    key = ("ref", single)
    if key not in _libs:
        path = os.path.join(REF_DIR, "libnfft3_ref_%s.so" % ("s" if single else "d"))
        if not (os.path.exists(path) and _is_native(path)):
            return None
        _libs[key] = C.CDLL(path)
    return _libs[key]


def _declare(lib, pfx, R):
    P = C.c_void_p
    Rp = C.POINTER(R)
    sig = {
        "plan_create": (P, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_long, C.c_uint]),
        "plan_destroy": (None, [P]),
        "set_nodes": (None, [P, Rp]),
        "precompute": (None, [P]),
        "trafo": (None, [P, Rp, Rp]),
        "adjoint": (None, [P, Rp, Rp]),
        "trafo_direct": (None, [P, Rp, Rp]),
        "adjoint_direct": (None, [P, Rp, Rp]),
        "get_index_x": (None, [P, C.POINTER(C.c_int64)]),
        "get_c_phi_inv": (None, [P, C.POINTER(C.c_double)]),
        "stage_times": (None, [P, C.POINTER(C.c_double)]),
        "bessel_i0": (C.c_double, [C.c_double]),
        "phi": (R, [C.c_int, C.c_int, R, R]),
        "fft": (None, [C.c_int, C.POINTER(C.c_int), Rp, C.c_int]),
        "solver_create": (P, [P, C.c_uint]),
        "solver_destroy": (None, [P]),
        "solver_set": (None, [P, Rp, Rp, Rp, Rp]),
        "solver_before_loop": (None, [P]),
        "solver_step": (None, [P]),
        "solver_get": (None, [P, Rp, Rp, C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, pfx + name)
        fn.restype = res
        fn.argtypes = args


def _ptr(a, R):
    return a.ctypes.data_as(C.POINTER(R))


class OraclePlan:
    """The C restatement driven like an nfft plan (test checker only)."""

    def __init__(self, N, M, n=None, m=None, single=False, sort=True,
                 blockwise=False, pre_psi=False):
        self.single = single
        self.R = C.c_float if single else C.c_double
        self.rdt = np.float32 if single else np.float64
        self.cdt = np.complex64 if single else np.complex128
        self.pfx = "orcf_" if single else "orc_"
        self.lib = load(single)
        self.N = [int(v) for v in N]
        self.d = len(self.N)
        if n is None:
            n = [2 * (1 << (int(v) - 1).bit_length()) for v in self.N]
        if m is None:
            m = 4 if single else 8
        self.n = [int(v) for v in n]
        self.m = int(m)
        self.M = int(M)
        flags = (ORC_SORT if sort else 0) | (ORC_BLOCKWISE if blockwise else 0) | \
                (ORC_PRE_PSI if pre_psi else 0)
        Nc = (C.c_int * self.d)(*self.N)
        nc = (C.c_int * self.d)(*self.n)
        self.h = self._f("plan_create")(self.d, Nc, nc, self.m, self.M, flags)
        self.N_total = int(np.prod(self.N))

    def _f(self, name):
        return getattr(self.lib, self.pfx + name)

    def set_nodes(self, x):
        x = np.ascontiguousarray(x, dtype=self.rdt).reshape(-1)
        assert x.size == self.M * self.d
        self._f("set_nodes")(self.h, _ptr(x, self.R))

    def precompute(self):
        self._f("precompute")(self.h)

    def _run(self, name, inp, nout):
        inp = np.ascontiguousarray(inp, dtype=self.cdt).reshape(-1)
        out = np.zeros(nout, dtype=self.cdt)
        self._f(name)(self.h, _ptr(inp.view(self.rdt), self.R), _ptr(out.view(self.rdt), self.R))
        return out

    def trafo(self, f_hat):
        return self._run("trafo", f_hat, self.M)

    def adjoint(self, f):
        return self._run("adjoint", f, self.N_total)

    def trafo_direct(self, f_hat):
        return self._run("trafo_direct", f_hat, self.M)

    def adjoint_direct(self, f):
        return self._run("adjoint_direct", f, self.N_total)

    def index_x(self):
        out = np.zeros(2 * self.M, dtype=np.int64)
        self._f("get_index_x")(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)))
        return out

    def c_phi_inv(self):
        out = np.zeros(sum(self.N), dtype=np.float64)
        self._f("get_c_phi_inv")(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def stage_times(self):
        out = np.zeros(3, dtype=np.float64)
        self._f("stage_times")(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def close(self):
        if self.h:
            self._f("plan_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleSolver:
    """CGNR/CGNE restatement over an OraclePlan (test checker only)."""

    def __init__(self, plan, flags):
        self.plan = plan
        self.h = plan._f("solver_create")(plan.h, int(flags))

    def set(self, y=None, w=None, w_hat=None, f_hat_iter=None):
        p = self.plan
        args = []
        keep = []
        for v, dt in ((y, p.cdt), (w, p.rdt), (w_hat, p.rdt), (f_hat_iter, p.cdt)):
            if v is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(v, dtype=dt).reshape(-1)
                keep.append(a)
                args.append(_ptr(a.view(p.rdt), p.R))
        p._f("solver_set")(self.h, *args)

    def before_loop(self):
        self.plan._f("solver_before_loop")(self.h)

    def step(self):
        self.plan._f("solver_step")(self.h)

    def get(self):
        p = self.plan
        fh = np.zeros(p.N_total, dtype=p.cdt)
        r = np.zeros(p.M, dtype=p.cdt)
        sc = np.zeros(8, dtype=np.float64)
        p._f("solver_get")(self.h, _ptr(fh.view(p.rdt), p.R), _ptr(r.view(p.rdt), p.R),
                           sc.ctypes.data_as(C.POINTER(C.c_double)))
        names = ("alpha", "beta", "dot_r", "dot_r_old", "dot_z", "dot_z_old", "dot_p", "dot_v")
        return fh, r, dict(zip(names, sc.tolist()))

    def close(self):
        if self.h:
            self.plan._f("solver_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fft(data, sign, single=False):
    """Unnormalised n-D complex DFT of the oracle's own FFT (in a copy)."""
    lib = load(single)
    R = C.c_float if single else C.c_double
    a = np.ascontiguousarray(data, dtype=np.complex64 if single else np.complex128).copy()
    shp = (C.c_int * a.ndim)(*a.shape)
    getattr(lib, ("orcf_" if single else "orc_") + "fft")(a.ndim, shp, _ptr(a.reshape(-1).view(np.float32 if single else np.float64), R), int(sign))
    return a


def bessel_i0(x, single=False):
    return getattr(load(single), ("orcf_" if single else "orc_") + "bessel_i0")(float(x))


# --- reading the reference's golden files (tests/data/nfft_*.txt format,
# parsed like tests/nfft.c:379-448): d, N_1..N_d, M, x (M*d), f_hat
# (N_total complex) and f (M complex); adjoint files carry f then f_hat in the
# same positions (tests/check_nfft.m:55-75). ---
def parse_golden_text(text):
    tok = text.split()
    pos = 0
    d = int(tok[pos]); pos += 1
    N = [int(tok[pos + i]) for i in range(d)]; pos += d
    M = int(tok[pos]); pos += 1
    x = np.array([float(v) for v in tok[pos:pos + M * d]], dtype=np.float64); pos += M * d
    NN = int(np.prod(N))
    a = np.array([float(v) for v in tok[pos:pos + 2 * NN]], dtype=np.float64); pos += 2 * NN
    b = np.array([float(v) for v in tok[pos:pos + 2 * M]], dtype=np.float64); pos += 2 * M
    return dict(d=d, N=N, M=M, x=x.reshape(M, d),
                first=a[0::2] + 1j * a[1::2], second=b[0::2] + 1j * b[1::2])
