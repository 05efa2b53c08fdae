"""Synthetic inputs of the benchmark workloads (seeded numpy generators).

The reference has no public benchmark data set; these stand in with the shapes
and value distributions of the workloads the benchmark is quoted on:

* uniform or clustered nodes on the d-torus: iid U[-1/2, 1/2)^d, or a
  mixture of 32 isotropic Gaussians (centres uniform, std 0.02) wrapped to
  the torus;
* radial k-space: `spokes` spokes at angles pi*s/spokes, `samples` radial
  positions uniformly spaced in [-1/2, 1/2);
* interleaved Archimedean spirals: arm a, t in [0, 1): r = 0.5 t,
  angle 2 pi (turns t + a/arms) + a global rotation, radius jitter N(0, s^2);
* ellipse phantoms: a sum of random filled ellipses on the N x N pixel grid
  (pixel k at k/N, k = -N/2..N/2-1), the image being the Fourier-coefficient
  vector f_hat of the NFFT in natural order.
"""
import numpy as np


def cube_nodes(M, d, dist="uniform", seed=0, dtype=np.float32):
    """M nodes in [-1/2, 1/2)^d: "uniform" or "clustered" (32 Gaussians, std 0.02)."""
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        return rng.uniform(-0.5, 0.5, size=(M, d)).astype(dtype)
    if dist != "clustered":
        raise ValueError("unknown node distribution %r" % dist)
    c = rng.uniform(-0.5, 0.5, size=(32, d))
    x = c[rng.integers(0, 32, M)] + 0.02 * rng.standard_normal((M, d))
    x = (((x + 0.5) % 1.0) - 0.5).astype(dtype)
    x[x >= 0.5] = -0.5
    return x


def radial_nodes(spokes=402, samples=512):
    s = np.arange(spokes)
    ang = np.pi * s / spokes
    r = -0.5 + np.arange(samples) / samples
    x0 = np.outer(np.cos(ang), r).reshape(-1)
    x1 = np.outer(np.sin(ang), r).reshape(-1)
    x = np.stack([x0, x1], axis=1)
    return wrap_nodes(x)


def spiral_nodes(arms=16, samples=8192, turns=24.0, rotation=0.0, jitter=1e-4, rng=None):
    rng = np.random.default_rng(0) if rng is None else rng
    t = np.arange(samples) / samples
    out = []
    for a in range(arms):
        r = 0.5 * t + jitter * rng.standard_normal(samples)
        ang = 2 * np.pi * (turns * t + a / arms) + rotation
        out.append(np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1))
    return wrap_nodes(np.concatenate(out, axis=0))


def wrap_nodes(x):
    """Map coordinates to the torus [-1/2, 1/2)."""
    x = ((np.asarray(x, dtype=np.float64) + 0.5) % 1.0) - 0.5
    x[x >= 0.5] = -0.5
    return x


def ellipse_phantom(N, count=20, seed=1):
    rng = np.random.default_rng(seed)
    k = (np.arange(N) - N // 2) / N
    u0, u1 = np.meshgrid(k, k, indexing="ij")
    img = np.zeros((N, N))
    for _ in range(count):
        c = rng.uniform(-0.4, 0.4, 2)
        ax = rng.uniform(0.02, 0.3, 2)
        th = rng.uniform(0.0, np.pi)
        val = rng.uniform(-1.0, 1.0)
        d0, d1 = u0 - c[0], u1 - c[1]
        p = np.cos(th) * d0 + np.sin(th) * d1
        q = -np.sin(th) * d0 + np.cos(th) * d1
        img[(p / ax[0]) ** 2 + (q / ax[1]) ** 2 <= 1.0] += val
    return img.reshape(-1).astype(np.complex128)


def add_noise(y, snr_db, rng):
    """Complex Gaussian noise with ||noise|| = ||y|| 10^(-snr/20)."""
    y = np.asarray(y)
    scale = np.linalg.norm(y) * 10 ** (-snr_db / 20.0) / np.sqrt(len(y))
    n = (rng.standard_normal(len(y)) + 1j * rng.standard_normal(len(y))) / np.sqrt(2.0)
    return y + scale * n
