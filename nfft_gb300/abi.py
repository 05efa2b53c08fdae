"""ctypes mirror of the NFFT 3 C ABI (the nfft3.h structures and prototypes).

The GPU library ``libnfft3_gb300.so`` exports the reference's own C entry
points with the reference's own structure layouts, so the same mirror binds
either library.  Layouts follow the reference header:

* ``MACRO_MV_PLAN`` members (include/nfft3.h:54-60);
* ``nfft_plan`` / ``nfftf_plan`` (include/nfft3.h:108-161);
* ``solver_plan_complex`` / ``solverf_plan_complex`` (include/nfft3.h:760-780);
* plan flags (include/nfft3.h:195-208) and solver flags (include/nfft3.h:822-829).
"""
import ctypes as C

# ---- plan flags (include/nfft3.h:195-208) ----
PRE_PHI_HUT = 1 << 0
FG_PSI = 1 << 1
PRE_LIN_PSI = 1 << 2
PRE_FG_PSI = 1 << 3
PRE_PSI = 1 << 4
PRE_FULL_PSI = 1 << 5
MALLOC_X = 1 << 6
MALLOC_F_HAT = 1 << 7
MALLOC_F = 1 << 8
FFT_OUT_OF_PLACE = 1 << 9
FFTW_INIT = 1 << 10
NFFT_SORT_NODES = 1 << 11
NFFT_OMP_BLOCKWISE_ADJOINT = 1 << 12
PRE_ONE_PSI = PRE_LIN_PSI | PRE_FG_PSI | PRE_PSI | PRE_FULL_PSI

# ---- FFTW planner flags as spelled by FFTW 3 (values of fftw3.h) ----
FFTW_MEASURE = 0
FFTW_DESTROY_INPUT = 1 << 0
FFTW_ESTIMATE = 1 << 6

# ---- solver flags (include/nfft3.h:822-829) ----
LANDWEBER = 1 << 0
STEEPEST_DESCENT = 1 << 1
CGNR = 1 << 2
CGNE = 1 << 3
NORMS_FOR_LANDWEBER = 1 << 4
PRECOMPUTE_WEIGHT = 1 << 5
PRECOMPUTE_DAMP = 1 << 6

INT = C.c_ssize_t  # NFFT_INT is ptrdiff_t (include/nfft3.h:51)
VOIDFN = C.CFUNCTYPE(None, C.c_void_p)


def _mv_fields(R):
    # complex vectors are (re, im) pairs of R: expose them as R* (interleaved)
    return [
        ("N_total", INT),
        ("M_total", INT),
        ("f_hat", C.POINTER(R)),
        ("f", C.POINTER(R)),
        ("mv_trafo", C.c_void_p),
        ("mv_adjoint", C.c_void_p),
    ]


def _plan_struct(R, name):
    fields = _mv_fields(R) + [
        ("d", INT),
        ("N", C.POINTER(INT)),
        ("sigma", C.POINTER(R)),
        ("n", C.POINTER(INT)),
        ("n_total", INT),
        ("m", INT),
        ("b", C.POINTER(R)),
        ("K", INT),
        ("flags", C.c_uint),
        ("fftw_flags", C.c_uint),
        ("x", C.POINTER(R)),
        ("MEASURE_TIME_t", R * 3),
        ("my_fftw_plan1", C.c_void_p),
        ("my_fftw_plan2", C.c_void_p),
        ("c_phi_inv", C.POINTER(C.POINTER(R))),
        ("psi", C.POINTER(R)),
        ("psi_index_g", C.POINTER(INT)),
        ("psi_index_f", C.POINTER(INT)),
        ("g", C.POINTER(R)),
        ("g_hat", C.POINTER(R)),
        ("g1", C.POINTER(R)),
        ("g2", C.POINTER(R)),
        ("spline_coeffs", C.POINTER(R)),
        ("index_x", C.POINTER(INT)),
    ]
    return type(name, (C.Structure,), {"_fields_": fields})


def _mv_struct(R, name):
    return type(name, (C.Structure,), {"_fields_": _mv_fields(R)})


def _solver_struct(R, mv, name):
    fields = [
        ("mv", C.POINTER(mv)),
        ("flags", C.c_uint),
        ("w", C.POINTER(R)),
        ("w_hat", C.POINTER(R)),
        ("y", C.POINTER(R)),
        ("f_hat_iter", C.POINTER(R)),
        ("r_iter", C.POINTER(R)),
        ("z_hat_iter", C.POINTER(R)),
        ("p_hat_iter", C.POINTER(R)),
        ("v_iter", C.POINTER(R)),
        ("alpha_iter", R),
        ("beta_iter", R),
        ("dot_r_iter", R),
        ("dot_r_iter_old", R),
        ("dot_z_hat_iter", R),
        ("dot_z_hat_iter_old", R),
        ("dot_p_hat_iter", R),
        ("dot_v_iter", R),
    ]
    return type(name, (C.Structure,), {"_fields_": fields})


nfft_plan = _plan_struct(C.c_double, "nfft_plan")
nfftf_plan = _plan_struct(C.c_float, "nfftf_plan")
nfft_mv_plan_complex = _mv_struct(C.c_double, "nfft_mv_plan_complex")
nfftf_mv_plan_complex = _mv_struct(C.c_float, "nfftf_mv_plan_complex")
solver_plan_complex = _solver_struct(C.c_double, nfft_mv_plan_complex, "solver_plan_complex")
solverf_plan_complex = _solver_struct(C.c_float, nfftf_mv_plan_complex, "solverf_plan_complex")
# the NNFFT plan (include/nfft3.h:387-432), double precision
nnfft_plan = type("nnfft_plan", (C.Structure,), {"_fields_": _mv_fields(C.c_double) + [
    ("d", C.c_int),
    ("sigma", C.POINTER(C.c_double)),
    ("a", C.POINTER(C.c_double)),
    ("N", C.POINTER(C.c_int)),
    ("N1", C.POINTER(C.c_int)),
    ("aN1", C.POINTER(C.c_int)),
    ("m", C.c_int),
    ("b", C.POINTER(C.c_double)),
    ("K", C.c_int),
    ("aN1_total", C.c_int),
    ("direct_plan", C.POINTER(nfft_plan)),
    ("nnfft_flags", C.c_uint),
    ("n", C.POINTER(C.c_int)),
    ("x", C.POINTER(C.c_double)),
    ("v", C.POINTER(C.c_double)),
    ("c_phi_inv", C.POINTER(C.c_double)),
    ("psi", C.POINTER(C.c_double)),
    ("size_psi", C.c_int),
    ("psi_index_g", C.POINTER(C.c_int)),
    ("psi_index_f", C.POINTER(C.c_int)),
    ("F", C.POINTER(C.c_double)),
    ("spline_coeffs", C.POINTER(C.c_double)),
]})
MALLOC_V = 1 << 11

# the NFCT plan (include/nfft3.h:224-265), both precisions
def _nfct_struct(R, name, extra=()):
    P = C.POINTER(R)
    return type(name, (C.Structure,), {"_fields_": _mv_fields(R) + [
        ("d", INT), ("N", C.POINTER(INT)), ("n", C.POINTER(INT)), ("n_total", INT),
        ("sigma", P), ("m", INT), ("b", P), ("K", INT), ("flags", C.c_uint), ("fftw_flags", C.c_uint),
        ("x", P), ("MEASURE_TIME_t", C.c_double * 3), ("my_fftw_r2r_plan", C.c_void_p),
        ("r2r_kind", C.POINTER(C.c_int)), ("c_phi_inv", C.POINTER(P)), ("psi", P), ("size_psi", INT),
        ("psi_index_g", C.POINTER(INT)), ("psi_index_f", C.POINTER(INT)),
        ("g", P), ("g_hat", P), ("g1", P), ("g2", P), ("spline_coeffs", P),
    ] + list(extra)})


nfct_plan = _nfct_struct(C.c_double, "nfct_plan")
nfctf_plan = _nfct_struct(C.c_float, "nfctf_plan")
# the NFST plan (include/nfft3.h:299-343): the same layout and one more field
nfst_plan = _nfct_struct(C.c_double, "nfst_plan", [("nfst_full_psi_eps", C.c_double)])
nfstf_plan = _nfct_struct(C.c_float, "nfstf_plan", [("nfstf_full_psi_eps", C.c_float)])

# the MRI operators (include/nfft3.h:510-540), double precision; both plan
# types share one layout
def _mri_struct(name):
    return type(name, (C.Structure,), {"_fields_": _mv_fields(C.c_double) + [
        ("plan", nfft_plan),
        ("N3", C.c_int),
        ("sigma3", C.c_double),
        ("t", C.POINTER(C.c_double)),
        ("w", C.POINTER(C.c_double)),
    ]})


mri_inh_2d1d_plan = _mri_struct("mri_inh_2d1d_plan")
mri_inh_3d_plan = _mri_struct("mri_inh_3d_plan")

# the real-valued operator and solver (include/nfft3.h:67, 788-815)
nfft_mv_plan_double = _mv_struct(C.c_double, "nfft_mv_plan_double")
nfftf_mv_plan_double = _mv_struct(C.c_float, "nfftf_mv_plan_double")
solver_plan_double = _solver_struct(C.c_double, nfft_mv_plan_double, "solver_plan_double")
solverf_plan_double = _solver_struct(C.c_float, nfftf_mv_plan_double, "solverf_plan_double")


class Precision:
    """Names and types of one precision of the ABI (nfft_ or nfftf_)."""

    def __init__(self, single):
        self.single = single
        self.R = C.c_float if single else C.c_double
        self.np_real = "float32" if single else "float64"
        self.np_complex = "complex64" if single else "complex128"
        self.pfx = "nfftf_" if single else "nfft_"
        self.spfx = "solverf_" if single else "solver_"
        self.plan = nfftf_plan if single else nfft_plan
        self.solver = solverf_plan_complex if single else solver_plan_complex
        self.mv = nfftf_mv_plan_complex if single else nfft_mv_plan_complex


DOUBLE = Precision(False)
SINGLE = Precision(True)

# Entry points shared by the reference library and the GPU library, with
# their ctypes signatures (include/nfft3.h:163-187, 782-786, 839-890).
def bind(lib, prec):
    """Attach argtypes/restype for ``prec`` to the functions of ``lib``."""
    P = C.POINTER(prec.plan)
    S = C.POINTER(prec.solver)
    MV = C.POINTER(prec.mv)
    R = prec.R
    sig = {
        "init_guru": (None, [P, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int, C.c_uint, C.c_uint]),
        "init": (None, [P, C.c_int, C.POINTER(C.c_int), C.c_int]),
        "init_1d": (None, [P, C.c_int, C.c_int]),
        "init_2d": (None, [P, C.c_int, C.c_int, C.c_int]),
        "init_3d": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int]),
        "precompute_one_psi": (None, [P]),
        "precompute_psi": (None, [P]),
        "precompute_full_psi": (None, [P]),
        "trafo": (None, [P]),
        "adjoint": (None, [P]),
        "trafo_1d": (None, [P]),
        "trafo_2d": (None, [P]),
        "trafo_3d": (None, [P]),
        "adjoint_1d": (None, [P]),
        "adjoint_2d": (None, [P]),
        "adjoint_3d": (None, [P]),
        "trafo_direct": (None, [P]),
        "adjoint_direct": (None, [P]),
        "check": (C.c_char_p, [P]),
        "finalize": (None, [P]),
        "malloc": (C.c_void_p, [C.c_size_t]),
        "free": (None, [C.c_void_p]),
        "next_power_of_2": (INT, [INT]),
        "get_default_window_cut_off": (INT, []),
        "get_window_name": (C.c_char_p, []),
        "dot_complex": (R, [C.POINTER(R), INT]),
    }
    out = {}
    for name, (res, args) in sig.items():
        fn = getattr(lib, prec.pfx + name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
        out[name] = fn
    ssig = {
        "init_advanced_complex": (None, [S, MV, C.c_uint]),
        "init_complex": (None, [S, MV]),
        "before_loop_complex": (None, [S]),
        "loop_one_step_complex": (None, [S]),
        "finalize_complex": (None, [S]),
    }
    for name, (res, args) in ssig.items():
        fn = getattr(lib, prec.spfx + name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
        out["solver_" + name] = fn
    return out
