"""Shared helpers of the test suite: the reference's error measures and bounds."""
import math

import numpy as np

from nfft_gb300 import abi

EPS = {False: np.finfo(np.float64).eps, True: np.finfo(np.float32).eps}


def err_trafo_bound(m, single):
    """Kaiser-Bessel bound of the reference tests (tests/nfft.c:217-284)."""
    a, b = (0.4, 2000.0) if single else (0.3, 2100.0)
    err = math.pi * (math.sqrt(m) + m) * math.sqrt(math.sqrt(1.0 - 0.5)) * \
        math.exp(-2.0 * math.pi * m * math.sqrt(1.0 - 0.5))
    return max(a * err, b * EPS[single], 48.0 * EPS[single])


def err_direct_bound(single):
    return 48.0 * EPS[single]  # tests/nfft.c:211-215


def compare_trafo(f, f_ref, f_hat):
    """||f - f_ref||_inf / ||f_hat||_1 (tests/nfft.c:739-759)."""
    num = np.max(np.abs(f - f_ref)) if len(f) else 0.0
    return 0.0 if num == 0 else num / np.sum(np.abs(f_hat))


def compare_adjoint(f_hat, f_hat_ref, f):
    """||f_hat - f_hat_ref||_inf / ||f||_1 (tests/nfft.c:761-781)."""
    num = np.max(np.abs(f_hat - f_hat_ref)) if len(f_hat) else 0.0
    return 0.0 if num == 0 else num / np.sum(np.abs(f))


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def next_pow2(v):
    """nfft_next_power_of_2 semantics (kernel/util/int.c:101-133)."""
    v = int(v)
    if v < 0:
        return -1
    if v < 2:
        return v + 1
    return 1 << (v - 1).bit_length()


def default_guru_flags():
    """PRE_PHI_HUT | PRE_PSI | DEFAULT_NFFT_FLAGS of the reference tests (tests/nfft.c:131,696)."""
    return (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F | abi.MALLOC_F_HAT
            | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE)


def seeded_case(N, M, seed=0):
    rng = np.random.default_rng(seed)
    d = len(N)
    x = rng.uniform(-0.5, 0.5, size=(M, d))
    NN = int(np.prod(N))
    fh = rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)
    f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return x, fh, f
