"""A compiled C program calls the drop-in ABI the way the reference's examples do.

tests/c_caller/simple_calls.c is built with gcc against include/ only and
linked with libnfft3_gb300.so; it follows examples/nfft/simple_test.c.in
(init_1d, init_guru with PRE_FULL_PSI, init_3d in single precision: direct
and fast trafo / adjoint) and examples/solver/simple_test.c.in (CGNR through
solver_init_complex with the plan / solver f_hat pointer swap).  The program
writes its inputs and outputs to files; each result is recomputed here with
the oracle on the same inputs.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from helpers import rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "simple_calls.c")


@pytest.fixture(scope="module")
def run_dir(gpulib, tmp_path_factory):
    d = tmp_path_factory.mktemp("c_caller")
    exe = str(d / "simple_calls")
    libdir = os.path.join(ROOT, "nfft_gb300")
    subprocess.check_call(["gcc", "-std=c99", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), SRC,
                           "-L" + libdir, "-lnfft3_gb300", "-Wl,-rpath," + libdir, "-lm", "-o", exe])
    out = d / "out"
    out.mkdir()
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "all calls done" in r.stdout
    return out


def load(d, name, dtype):
    return np.fromfile(str(d / (name + ".bin")), dtype=dtype)


def oracle_plan(N, M, n, m, x, single=False):
    o = oracle.OraclePlan(N, M, n=n, m=m, single=single)
    o.set_nodes(x)
    o.precompute()
    return o


@pytest.mark.parametrize("tag,N,n,m", [("d1", [14], [32], 8), ("d2", [32, 14], [64, 32], 7)])
def test_double_plans_match_oracle(run_dir, tag, N, n, m):
    x = load(run_dir, tag + "_x", np.float64)
    M = len(x) // len(N)
    fh = load(run_dir, tag + "_fhat", np.complex128)
    o = oracle_plan(N, M, n, m, x)
    f = load(run_dir, tag + "_f", np.complex128)
    assert rel_l2(f, o.trafo(fh)) < 1e-12
    assert rel_l2(load(run_dir, tag + "_f_direct", np.complex128), o.trafo_direct(fh)) < 1e-12
    # both adjoints take the fast trafo's samples, as in the example
    assert rel_l2(load(run_dir, tag + "_fhat_adj", np.complex128), o.adjoint(f)) < 1e-12
    assert rel_l2(load(run_dir, tag + "_fhat_direct", np.complex128), o.adjoint_direct(f)) < 1e-12


def test_single_3d_plan_matches_oracle(run_dir):
    x = load(run_dir, "s3_x", np.float32)
    M = len(x) // 3
    fh = load(run_dir, "s3_fhat", np.complex64)
    o = oracle_plan([16] * 3, M, [32] * 3, 4, x.astype(np.float64))
    f = load(run_dir, "s3_f", np.complex64)
    assert rel_l2(f.astype(np.complex128), o.trafo(fh.astype(np.complex128))) < 1e-5
    fa = load(run_dir, "s3_fhat_adj", np.complex64)
    assert rel_l2(fa.astype(np.complex128), o.adjoint(f.astype(np.complex128))) < 1e-5


def test_solver_loop_matches_oracle(run_dir):
    N, n, m = [32, 32], [64, 64], 6
    x = load(run_dir, "cg_x", np.float64)
    M = len(x) // 2
    y = load(run_dir, "cg_y", np.complex128)
    dot_r = load(run_dir, "cg_dot_r", np.float64)
    o = oracle_plan(N, M, n, m, x)
    s = oracle.OracleSolver(o, oracle.ORC_CGNR)
    s.set(y=y, f_hat_iter=np.zeros(1024, np.complex128))
    s.before_loop()
    want = [s.get()[2]["dot_r"]]
    for _ in range(len(dot_r) - 1):
        s.step()
        want.append(s.get()[2]["dot_r"])
    fh = s.get()[0]
    np.testing.assert_allclose(dot_r, want, rtol=1e-9)
    assert rel_l2(load(run_dir, "cg_fhat_iter", np.complex128), fh) < 1e-10
    assert rel_l2(load(run_dir, "cg_fit", np.complex128), o.trafo(fh)) < 1e-10
