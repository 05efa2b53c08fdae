"""nfft_gb300 -- GB300-native NFFT transform path behind the NFFT 3 C API.

The product is the shared library ``libnfft3_gb300.so`` (C ABI of
``include/nfft3.h`` plus the extensions of ``include/nfft_gb300.h``), built
from ``csrc/`` for sm_103a by ``build.py``.  This package only loads it and
offers ctypes mirrors (``abi``) and a host-side plan wrapper (``plan``).

There is no CPU fallback: ``lib()`` raises if the library was not built, and
every transform runs on the GPU.
"""
import ctypes as _C
import os as _os

HERE = _os.path.dirname(_os.path.abspath(__file__))
LIB_PATH = _os.environ.get("NFFT_GB300_LIB") or _os.path.join(HERE, "libnfft3_gb300.so")

_lib = None


def build(force=False, verbose=False):
    from . import builder as _b
    return _b.build(force=force, verbose=verbose)


def lib():
    """The loaded GPU library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not _os.path.exists(LIB_PATH):
            raise RuntimeError("libnfft3_gb300.so is not built; run nfft_gb300.build() "
                               "(there is no CPU fallback)")
        _lib = _C.CDLL(LIB_PATH)
        _lib.nfft_gb_last_error.restype = _C.c_char_p
        _lib.nfft_gb_device_ok.restype = _C.c_int
        for pfx in ("nfft_", "nfftf_"):
            for name in ("gb_device_f_hat", "gb_device_f", "gb_device_x", "gb_get_stream"):
                fn = getattr(_lib, pfx + name)
                fn.restype = _C.c_void_p
                fn.argtypes = [_C.c_void_p]
            for name in ("gb_trafo_device", "gb_adjoint_device", "gb_precompute_device"):
                fn = getattr(_lib, pfx + name)
                fn.restype = None
                fn.argtypes = [_C.c_void_p]
            fn = getattr(_lib, pfx + "gb_set_stream")
            fn.restype = _C.c_int
            fn.argtypes = [_C.c_void_p, _C.c_void_p]
            fn = getattr(_lib, pfx + "gb_stage_times")
            fn.restype = None
            fn.argtypes = [_C.c_void_p, _C.POINTER(_C.c_float)]
            fn = getattr(_lib, pfx + "gb_last_launch_count")
            fn.restype = _C.c_int
            fn.argtypes = [_C.c_void_p]
    return _lib


def last_error():
    return lib().nfft_gb_last_error().decode()
