"""The allocation-free node sort (nfft_gb_sort_nodes_noalloc) through the C ABI.

It serves callers that cannot allocate device memory where they sort nodes
(memory owned by a caching allocator or a fixed budget, or no room for the
synchronisation cudaMalloc implies).  Its output must equal index_x of the
regular node set-up (nfft_precompute_one_psi with NFFT_SORT_NODES) bit for
bit, call after call, although every call reuses one static scratch array.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import next_pow2
from nfft_gb300 import abi
from nfft_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def _entry(lib):
    fn = lib.nfft_gb_sort_nodes_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    return fn


def _regular_index(lib, single, N, x, m):
    n = [2 * next_pow2(v) for v in N]
    flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.NFFT_SORT_NODES)
    p = Plan(lib, single, N, len(x), n=n, m=m, flags=flags)
    p.x[:] = x
    p.precompute_one_psi()
    idx = p.index_x
    p.finalize()
    return idx, n


@pytest.mark.parametrize("single", [True, False])
def test_noalloc_sort_matches_precompute_twice(gpulib, single):
    import torch  # a GPU run without torch fails here rather than skipping
    fn = _entry(gpulib)
    dev = torch.device("cuda", 0)
    dt = torch.float32 if single else torch.float64
    # calls in a row on the shared scratch array; the last at the stated
    # maximum of 2^18 nodes, where its room is tightest
    cases = [([32, 32, 32], 200000, 4, 7), ([64, 48], 150000, 6, 8), ([64, 64, 64], 1 << 18, 4, 9)]
    for N, M, m, seed in cases:
        rng = np.random.default_rng(seed)
        x = rng.uniform(-0.5, 0.5, size=(M, len(N)))
        x = x.astype(np.float32) if single else x
        want, n = _regular_index(gpulib, single, N, x, m)
        xd = torch.from_numpy(np.ascontiguousarray(x).reshape(-1)).to(dev, dtype=dt)
        out = torch.full((2 * M,), -1, dtype=torch.int64, device=dev)
        nn = (C.c_int * len(n))(*n)
        rc = fn(1 if single else 0, xd.data_ptr(), len(N), nn, m, M, out.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == 0, gpulib.nfft_gb_last_error()
        got = out.cpu().numpy()
        assert np.array_equal(got, want), (N, M)


def test_noalloc_sort_rejects_too_many_nodes(gpulib):
    fn = _entry(gpulib)
    n = (C.c_int * 3)(64, 64, 64)
    # M beyond the stated maximum: rejected on the host, nothing is launched
    rc = fn(1, None, 3, n, 4, (1 << 18) + 1, None, None)
    assert rc == -1
    gpulib.nfft_gb_last_error.restype = C.c_char_p
    assert b"exceeds the maximum" in gpulib.nfft_gb_last_error()


def test_noalloc_sort_rejects_grid_beyond_32bit_keys(gpulib):
    fn = _entry(gpulib)
    # 65536 * 65536 * 2 = 2^33 grid points: the 32-bit sort keys cannot hold
    # them; rejected on the host before any multiplication can overflow
    n = (C.c_int * 3)(65536, 65536, 2)
    rc = fn(1, None, 3, n, 4, 0, None, None)
    assert rc == -1
    gpulib.nfft_gb_last_error.restype = C.c_char_p
    assert b"below 2^32" in gpulib.nfft_gb_last_error()
