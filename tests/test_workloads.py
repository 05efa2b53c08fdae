"""The synthetic workload generators against their specification (CPU): the
shapes, ranges and geometry of the benchmark inputs, the byte and flop
counts the roofline uses, and determinism of the seeded streams."""
import os
import sys

import numpy as np

from nfft_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_radial_lines():
    x = workloads.radial_nodes(402, 512)
    assert x.shape == (402 * 512, 2)
    assert np.all(x >= -0.5) and np.all(x < 0.5)
    # spoke s at angle pi s / 402 through the centre, radii -1/2 + k/512
    r = -0.5 + np.arange(512) / 512
    s = 137
    ang = np.pi * s / 402
    spoke = x[s * 512:(s + 1) * 512]
    exp = workloads.wrap_nodes(np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1))
    assert np.allclose(spoke, exp, atol=1e-15)
    # every spoke passes the centre once
    assert np.sum(np.all(x == 0.0, axis=1)) == 402


def test_spiral_arms():
    rng = np.random.default_rng(3)
    x = workloads.spiral_nodes(16, 8192, turns=24.0, rotation=0.7, jitter=0.0, rng=rng)
    assert x.shape == (16 * 8192, 2)
    t = np.arange(8192) / 8192
    a = 5
    arm = x[a * 8192:(a + 1) * 8192]
    ang = 2 * np.pi * (24.0 * t + a / 16) + 0.7
    exp = workloads.wrap_nodes(np.stack([0.5 * t * np.cos(ang), 0.5 * t * np.sin(ang)], axis=1))
    assert np.allclose(arm, exp, atol=1e-15)
    assert np.max(np.hypot(x[:, 0], x[:, 1])) < 0.5 + 1e-12


def test_wrap_is_the_torus():
    x = workloads.wrap_nodes(np.array([[-0.5, 0.5], [0.75, -0.75], [1.0 - 1e-17, 0.2]]))
    assert np.all(x >= -0.5) and np.all(x < 0.5)
    assert np.allclose(x[1], [-0.25, 0.25])


def test_ellipse_phantom_is_seeded():
    a = workloads.ellipse_phantom(64, 20, seed=1)
    b = workloads.ellipse_phantom(64, 20, seed=1)
    c = workloads.ellipse_phantom(64, 20, seed=2)
    assert a.shape == (64 * 64,) and np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.all(a.imag == 0) and np.count_nonzero(a) > 0


def test_noise_level():
    rng = np.random.default_rng(0)
    y = np.ones(200000, complex)
    n = workloads.add_noise(y, 40.0, rng) - y
    assert abs(np.linalg.norm(n) / np.linalg.norm(y) - 1e-2) < 2e-4


def test_benchmark_nodes_and_roofline_counts():
    wl = bench.workload("uniform")
    assert wl["N"] == [128] * 3 and wl["n"] == [256] * 3 and wl["m"] == 4 and wl["M"] == 1 << 24
    small = dict(wl, M=4096)
    x = bench.make_nodes(small, 0)
    assert x.shape == (4096, 3) and x.dtype == np.float32 and np.all((x >= -0.5) & (x < 0.5))
    assert np.array_equal(x, bench.make_nodes(small, 0))
    cl = dict(bench.workload("clustered"), M=4096)
    xc = bench.make_nodes(cl, 0)
    assert np.all((xc >= -0.5) & (xc < 0.5))
    # algorithmic bytes of one B launch: M (3 x 4 B + 8 B) + n_total x 8 B = 469.8 MB
    assert bench.algorithmic_bytes_B(wl) == (1 << 24) * 20 + 256 ** 3 * 8 == 469762048
    assert bench.flops_B(wl) == 4.0 * 1000 * (1 << 24)
