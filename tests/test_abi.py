"""The drop-in boundary, checked without a GPU.

* the library loads and exports every function that include/nfft3.h and
  include/nfft_gb300.h declare;
* the structure layouts of include/nfft3.h (compiled with gcc) equal the
  ctypes mirror and, where the reference checkout exists, the reference's own
  include/nfft3.h;
* host utilities keep the reference semantics (kernel/util/int.c:101-133,
  vector3.c:22-29 and 113-144, vector1.c:22-30).
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import nfft_gb300
from nfft_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _declared_functions():
    names = set()
    text = open(os.path.join(INC, "nfft3.h")).read()
    # functions declared through the X(...) / Y(...) macros, per prefix
    api = {
        "NFFT_DEFINE_MALLOC_API": ["nfft_", "nfftf_"],
        "NFFT_DEFINE_API": ["nfft_", "nfftf_"],
        "SOLVER_DEFINE_API": ["solver_", "solverf_"],
        "NFFT_DEFINE_UTIL_API": ["nfft_", "nfftf_"],
        "NNFFT_DEFINE_API": ["nnfft_"],
        "MRI_DEFINE_API": ["mri_"],
        "NFCT_DEFINE_API": ["nfct_", "nfctf_"],
        "NFST_DEFINE_API": ["nfst_", "nfstf_"],
    }
    for macro, prefixes in api.items():
        body = re.search(r"#define %s\(.*?\)(.*?)\n\n" % macro, text, re.S).group(1)
        for fn in re.findall(r"(?:X|Y)\((\w+)\)\s*\(", body):
            if fn.endswith("_type_function"):
                continue
            for p in prefixes:
                names.add(p + fn)
    gb = open(os.path.join(INC, "nfft_gb300.h")).read()
    body = re.search(r"#define NFFTGB_DEFINE_API\(X\)(.*?)\n\n", gb, re.S).group(1)
    for fn in re.findall(r"X\((\w+)\)\s*\(", body):
        names.update({"nfft_" + fn, "nfftf_" + fn})
    for fn in re.findall(r"^\w[\w\s\*]*?\b(nfft_gb_\w+)\s*\(", gb, re.M):
        names.add(fn)
    return names


def test_library_exports_every_declared_function():
    lib = nfft_gb300.lib()
    names = _declared_functions()
    assert len(names) > 120
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


LAYOUT_PROG = r"""
#include <stdio.h>
#include <stddef.h>
#include <complex.h>
#include <nfft3.h>
#define F(T, f) printf(#T " " #f " %zu\n", offsetof(T, f));
#define PLAN(T) F(T,N_total) F(T,M_total) F(T,f_hat) F(T,f) F(T,mv_trafo) F(T,mv_adjoint) \
  F(T,d) F(T,N) F(T,sigma) F(T,n) F(T,n_total) F(T,m) F(T,b) F(T,K) F(T,flags) F(T,fftw_flags) \
  F(T,x) F(T,MEASURE_TIME_t) F(T,my_fftw_plan1) F(T,my_fftw_plan2) F(T,c_phi_inv) F(T,psi) \
  F(T,psi_index_g) F(T,psi_index_f) F(T,g) F(T,g_hat) F(T,g1) F(T,g2) F(T,spline_coeffs) F(T,index_x) \
  printf(#T " sizeof %zu\n", sizeof(T));
#define SOLV(T) F(T,mv) F(T,flags) F(T,w) F(T,w_hat) F(T,y) F(T,f_hat_iter) F(T,r_iter) F(T,z_hat_iter) \
  F(T,p_hat_iter) F(T,v_iter) F(T,alpha_iter) F(T,beta_iter) F(T,dot_r_iter) F(T,dot_r_iter_old) \
  F(T,dot_z_hat_iter) F(T,dot_z_hat_iter_old) F(T,dot_p_hat_iter) F(T,dot_v_iter) \
  printf(#T " sizeof %zu\n", sizeof(T));
#define NN(T) F(T,N_total) F(T,M_total) F(T,f_hat) F(T,f) F(T,mv_trafo) F(T,mv_adjoint) F(T,d) F(T,sigma) \
  F(T,a) F(T,N) F(T,N1) F(T,aN1) F(T,m) F(T,b) F(T,K) F(T,aN1_total) F(T,direct_plan) F(T,nnfft_flags) F(T,n) \
  F(T,x) F(T,v) F(T,c_phi_inv) F(T,psi) F(T,size_psi) F(T,psi_index_g) F(T,psi_index_f) F(T,F) \
  F(T,spline_coeffs) printf(#T " sizeof %zu\n", sizeof(T));
#define MRI(T) F(T,N_total) F(T,M_total) F(T,f_hat) F(T,f) F(T,mv_trafo) F(T,mv_adjoint) F(T,plan) F(T,N3) \
  F(T,sigma3) F(T,t) F(T,w) printf(#T " sizeof %zu\n", sizeof(T));
#define CT(T) F(T,N_total) F(T,M_total) F(T,f_hat) F(T,f) F(T,mv_trafo) F(T,mv_adjoint) F(T,d) F(T,N) F(T,n) \
  F(T,n_total) F(T,sigma) F(T,m) F(T,b) F(T,K) F(T,flags) F(T,fftw_flags) F(T,x) F(T,MEASURE_TIME_t) \
  F(T,my_fftw_r2r_plan) F(T,r2r_kind) F(T,c_phi_inv) F(T,psi) F(T,size_psi) F(T,psi_index_g) \
  F(T,psi_index_f) F(T,g) F(T,g_hat) F(T,g1) F(T,g2) F(T,spline_coeffs) printf(#T " sizeof %zu\n", sizeof(T));
int main(void) { CT(nfct_plan) CT(nfctf_plan) CT(nfst_plan) CT(nfstf_plan) F(nfst_plan,nfst_full_psi_eps)
  F(nfstf_plan,nfstf_full_psi_eps) PLAN(nfft_plan) PLAN(nfftf_plan) SOLV(solver_plan_complex) SOLV(solverf_plan_complex)
  SOLV(solver_plan_double) SOLV(solverf_plan_double) NN(nnfft_plan) MRI(mri_inh_2d1d_plan) MRI(mri_inh_3d_plan)
  return 0; }
"""


def _layout(include_dirs, tmp_path, tag):
    src = tmp_path / ("layout_%s.c" % tag)
    exe = tmp_path / ("layout_%s" % tag)
    src.write_text(LAYOUT_PROG)
    cmd = ["gcc", "-std=gnu11", "-o", str(exe), str(src)] + ["-I" + d for d in include_dirs]
    subprocess.check_call(cmd)
    out = subprocess.check_output([str(exe)], text=True)
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.strip().splitlines()}


def _ctypes_layout():
    out = {}
    for name, st in (("nfft_plan", abi.nfft_plan), ("nfftf_plan", abi.nfftf_plan),
                     ("solver_plan_complex", abi.solver_plan_complex),
                     ("solverf_plan_complex", abi.solverf_plan_complex),
                     ("solver_plan_double", abi.solver_plan_double),
                     ("solverf_plan_double", abi.solverf_plan_double),
                     ("nnfft_plan", abi.nnfft_plan),
                     ("mri_inh_2d1d_plan", abi.mri_inh_2d1d_plan),
                     ("mri_inh_3d_plan", abi.mri_inh_3d_plan),
                     ("nfct_plan", abi.nfct_plan), ("nfctf_plan", abi.nfctf_plan),
                     ("nfst_plan", abi.nfst_plan), ("nfstf_plan", abi.nfstf_plan)):
        for f, _ in st._fields_:
            out[(name, f)] = getattr(st, f).offset
        out[(name, "sizeof")] = C.sizeof(st)
    return out


def test_struct_layout_matches_ctypes_mirror(tmp_path):
    ours = _layout([INC], tmp_path, "ours")
    assert ours == _ctypes_layout()


def test_struct_layout_matches_reference_header(tmp_path):
    import oracle
    ref_inc = os.path.join(oracle.REFERENCE_SRC, "include")
    if not os.path.exists(os.path.join(ref_inc, "nfft3.h")):
        pytest.skip("reference checkout not present")
    ref = _layout([ref_inc, os.path.join(ROOT, "oracle", "ref", "shim")], tmp_path, "ref")
    ours = _layout([INC], tmp_path, "ours2")
    assert ours == ref


def _util(name, restype, argtypes):
    fn = getattr(nfft_gb300.lib(), name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


def test_next_power_of_2_semantics():
    f = _util("nfft_next_power_of_2", C.c_ssize_t, [C.c_ssize_t])
    assert [f(v) for v in (-3, 0, 1, 2, 3, 4, 5, 255, 256, 257)] == [-1, 1, 2, 2, 4, 4, 8, 256, 256, 512]

    def by_halving(N):
        # the reference test's loop (tests/util.c:85-113): the smallest power
        # of two >= N, 1 for N = 0 and 2 for N = 1
        if N == 1:
            return 2
        n, logn, odd = N, 0, False
        while n != 1:
            odd = odd or n % 2 == 1
            n //= 2
            logn += 1
        if not odd:
            logn -= 1
        for _ in range(logn + 1):
            n *= 2
        return n
    # powers of two and one less, as tests/util.c:116-153 (64-bit index)
    for i in range(62):
        j = 1 << i
        assert f(j) == by_halving(j), j
        if j > 1:
            assert f(j - 1) == by_halving(j - 1), j - 1
    assert _util("nfft_exp2i", C.c_ssize_t, [C.c_ssize_t])(10) == 1024


def test_default_window_and_version():
    assert _util("nfft_get_default_window_cut_off", C.c_ssize_t, [])() == 8
    assert _util("nfftf_get_default_window_cut_off", C.c_ssize_t, [])() == 4
    assert _util("nfft_get_window_name", C.c_char_p, [])() == b"KAISER_BESSEL"


def test_blas1_helpers():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(37) + 1j * rng.standard_normal(37)).astype(np.complex128)
    y = (rng.standard_normal(37) + 1j * rng.standard_normal(37)).astype(np.complex128)
    dp = C.POINTER(C.c_double)
    dot = _util("nfft_dot_complex", C.c_double, [dp, C.c_ssize_t])
    assert abs(dot(x.ctypes.data_as(dp), 37) - np.vdot(x, x).real) < 1e-12
    upd = _util("nfft_upd_axpy_complex", None, [dp, C.c_double, dp, C.c_ssize_t])
    x2 = x.copy()
    upd(x2.ctypes.data_as(dp), 0.5, y.ctypes.data_as(dp), 37)
    assert np.allclose(x2, 0.5 * x + y)
    sh = _util("nfft_fftshift_complex", None, [dp, C.c_ssize_t, C.POINTER(C.c_ssize_t)])
    a = (rng.standard_normal((6, 8)) + 1j * rng.standard_normal((6, 8))).astype(np.complex128)
    b = a.copy()
    N = (C.c_ssize_t * 2)(6, 8)
    sh(b.ctypes.data_as(dp), 2, N)
    assert np.array_equal(b, np.fft.fftshift(a))


def test_malloc_hooks_roundtrip():
    lib = nfft_gb300.lib()
    mal = _util("nfft_malloc", C.c_void_p, [C.c_size_t])
    fre = _util("nfft_free", None, [C.c_void_p])
    for n in (0, 16, 1 << 20):
        p = mal(n)
        assert p
        C.memset(p, 1, max(n, 1))
        fre(p)
    assert lib is not None
