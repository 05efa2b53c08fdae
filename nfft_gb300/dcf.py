"""Learned density-compensation weights for the inverse NFFT (host driver).

All arithmetic runs in the library's kernels (include/nfft_gb300.h): the
fixed-point weights w <- w / |A A^H w| on the GPU transforms, the per-node
features, and the MLP's forward, gradient and Adam steps.  PyTorch tensors
only hold device memory.

Training targets are the standardised log density weights of each
trajectory (log(w / mean w)) after FP_ITERS steps of the fixed-point
iteration from w = 1, by default one: w = 1 / |A A^H 1|, the classic
density estimate.  Further steps make the weights worse for the solver: the
point-spread function of the full frequency box (A A^H) has negative
sidelobes, and iterating against it amplifies them (measured on 16 held-out
16-arm spirals of the learned workload, N = 256^2, m = 6: median FP32 CGNR
steps to a 1e-5 relative data residual 67.5 after one step, 70 after three,
92.5 after five, 297.5 after twenty, no convergence in 3000 after eighty;
495 unweighted).
The network predicts the targets from the features; the weights go to the
solver's `w` (PRECOMPUTE_WEIGHT) unchanged.
"""
import ctypes as C
import time

import numpy as np

from . import abi, infft, workloads
from .plan import Plan

F_IN = 8
FP_ITERS = 1  # fixed-point steps of the density weights (see above)


def _fn(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


class Kernels:
    def __init__(self, lib):
        vp = C.c_void_p
        self.lib = lib
        self.count = _fn(lib, "nfft_gb_mlp_param_count", C.c_int, [])()
        self.features = _fn(lib, "nfft_gb_dcf_features", C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, vp])
        self.affine = _fn(lib, "nfft_gb_affine_columns", C.c_int,
                          [vp, C.c_longlong, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), vp])
        self.forward = _fn(lib, "nfft_gb_mlp_forward", C.c_int, [vp, vp, C.c_int, vp, vp])
        self.grad = _fn(lib, "nfft_gb_mlp_grad", C.c_int, [vp, vp, vp, C.c_int, vp, vp, vp])
        self.adam = _fn(lib, "nfft_gb_mlp_adam", C.c_int,
                        [vp, vp, vp, vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, vp])
        self.fixed_point = _fn(lib, "nfftf_gb_dcf_fixed_point", C.c_int, [vp, vp, C.c_int])


def init_params(count, seed=0):
    """Glorot-uniform weights, zero biases (layout W1[8][64], b1, W2[64][64], b2, W3, b3)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(count, dtype=np.float32)
    o = 0
    for fan_in, fan_out in ((8, 64), (64, 64), (64, 1)):
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        p[o:o + fan_in * fan_out] = rng.uniform(-lim, lim, fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    return p


def plan_for(lib, N, x, m):
    n = [2 * (1 << (int(v) - 1).bit_length()) for v in N]
    p = Plan(lib, True, N, len(x), n=n, m=m, flags=infft.PLAN_FLAGS)
    p.x[:] = x.astype(np.float32)
    p.precompute_one_psi()
    return p, n


def fixed_point_weights(lib, N, x, m, iters=FP_ITERS):
    """Density weights of one trajectory after `iters` fixed-point steps
    w <- w / |A A^H w| from w = 1 (torch tensor, device)."""
    import torch
    k = Kernels(lib)
    p, _ = plan_for(lib, N, x, m)
    w = torch.ones(len(x), dtype=torch.float32, device="cuda")
    k.fixed_point(C.addressof(p.p), w.data_ptr(), iters)
    p.finalize()
    return w


def raw_features(lib, x, n):
    import torch
    k = Kernels(lib)
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32).reshape(-1)).cuda()
    feat = torch.empty(len(x) * F_IN, dtype=torch.float32, device="cuda")
    k.features(xd.data_ptr(), len(x), n[0], n[1], feat.data_ptr(), None)
    return feat


class DensityNet:
    """The MLP with its feature standardisation."""

    def __init__(self, lib, seed=0):
        import torch
        self.k = Kernels(lib)
        self.params = torch.from_numpy(init_params(self.k.count, seed)).cuda()
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.scale = np.ones(F_IN, np.float32)
        self.shift = np.zeros(F_IN, np.float32)
        self.step_no = 0

    def standardise(self, feat, rows):
        s = (C.c_float * F_IN)(*self.scale)
        t = (C.c_float * F_IN)(*self.shift)
        self.k.affine(feat.data_ptr(), rows, F_IN, s, t, None)

    def fit_standardisation(self, feats):
        f = np.concatenate([a.view(-1, F_IN).cpu().numpy() for a in feats], axis=0)
        mu, sd = f.mean(axis=0), f.std(axis=0)
        sd[sd < 1e-6] = 1.0
        self.scale = (1.0 / sd).astype(np.float32)
        self.shift = (-mu / sd).astype(np.float32)

    def predict_log(self, feat, rows):
        import torch
        out = torch.empty(rows, dtype=torch.float32, device="cuda")
        self.k.forward(self.params.data_ptr(), feat.data_ptr(), rows, out.data_ptr(), None)
        return out

    def weights(self, lib, x, n):
        import torch
        feat = raw_features(lib, x, n)
        self.standardise(feat, len(x))
        return torch.exp(self.predict_log(feat, len(x)))

    def train(self, feat, target, epochs=4, batch=1 << 16, lr=2e-3, seed=0, log=None):
        """Adam on the mean squared error of the log weights; feat/target are
        device tensors (rows x 8, rows) of standardised features / targets."""
        import torch
        rows = target.numel()
        grad = torch.empty_like(self.params)
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for ep in range(epochs):
            order = torch.randperm(rows, generator=g).cuda()
            tot, nb = 0.0, 0
            for b0 in range(0, rows, batch):
                idx = order[b0:b0 + batch]
                fb = feat.view(-1, F_IN)[idx].contiguous()
                tb = target[idx].contiguous()
                self.k.grad(self.params.data_ptr(), fb.data_ptr(), tb.data_ptr(), tb.numel(),
                            grad.data_ptr(), loss.data_ptr(), None)
                self.step_no += 1
                self.k.adam(self.params.data_ptr(), grad.data_ptr(), self.m1.data_ptr(), self.m2.data_ptr(),
                            self.step_no, lr, 0.9, 0.999, 1e-8, None)
                tot += float(loss.item())
                nb += 1
            hist.append(tot / max(nb, 1))
            if log:
                log("epoch %d loss %.5f" % (ep, hist[-1]))
        return hist


def spiral(i, arms=16, samples=8192, jitter=1e-4, seed_base=0):
    rng = np.random.default_rng(seed_base + i)
    rot = rng.uniform(0.0, 2.0 * np.pi)
    return workloads.spiral_nodes(arms, samples, 24.0, rot, jitter, rng)


def build_training_set(lib, N, m, ids, arms=16, samples=8192, fp_iters=FP_ITERS):
    """Features (raw) and standardised log density weights per trajectory."""
    import torch
    n = [2 * (1 << (int(v) - 1).bit_length()) for v in N]
    feats, targets = [], []
    for i in ids:
        x = spiral(i, arms, samples)
        w = fixed_point_weights(lib, N, x, m, fp_iters)
        lw = torch.log(w / w.mean())
        feats.append(raw_features(lib, x, n))
        targets.append(lw)
    return feats, targets
