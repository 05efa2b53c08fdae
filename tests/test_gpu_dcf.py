"""Learned density compensation: the hand-written MLP kernels against PyTorch
CPU autograd (FP64), the feature kernel against a numpy restatement, the
fixed-point weights against the oracle's transforms, and the learned weights
speeding up CGNR against the unweighted solver."""
import ctypes as C

import numpy as np
import pytest

import oracle
from nfft_gb300 import dcf, infft, workloads
from nfft_gb300.plan import Plan

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def torch_mlp(p, x):
    """Reference MLP in FP64 on the CPU with the library's parameter layout."""
    W1 = p[0:512].view(8, 64)
    b1 = p[512:576]
    W2 = p[576:4672].view(64, 64)
    b2 = p[4672:4736]
    W3 = p[4736:4800]
    b3 = p[4800]
    h1 = torch.nn.functional.gelu(x @ W1 + b1)
    h2 = torch.nn.functional.gelu(h1 @ W2 + b2)
    return h2 @ W3 + b3


def test_mlp_forward_and_gradient_match_autograd(gpulib):
    k = dcf.Kernels(gpulib)
    assert k.count == 4801
    rng = np.random.default_rng(0)
    p = dcf.init_params(k.count, seed=3) + 0.01 * rng.standard_normal(k.count).astype(np.float32)
    M = 3000
    x = rng.standard_normal((M, 8)).astype(np.float32)
    t = rng.standard_normal(M).astype(np.float32)
    pd, xd, td = (torch.from_numpy(a).cuda() for a in (p, x.reshape(-1), t))
    out = torch.empty(M, device="cuda")
    k.forward(pd.data_ptr(), xd.data_ptr(), M, out.data_ptr(), None)
    grad = torch.empty(k.count, device="cuda")
    loss = torch.empty(1, device="cuda")
    k.grad(pd.data_ptr(), xd.data_ptr(), td.data_ptr(), M, grad.data_ptr(), loss.data_ptr(), None)
    torch.cuda.synchronize()
    pr = torch.from_numpy(p.astype(np.float64)).requires_grad_(True)
    yr = torch_mlp(pr, torch.from_numpy(x.astype(np.float64)))
    lr = ((yr - torch.from_numpy(t.astype(np.float64))) ** 2).mean()
    lr.backward()
    assert np.allclose(out.cpu().numpy(), yr.detach().numpy(), rtol=1e-4, atol=1e-5)
    assert abs(loss.item() - lr.item()) <= 1e-4 * abs(lr.item())
    g_ref = pr.grad.numpy()
    g = grad.cpu().numpy()
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-4


def test_adam_step_matches_torch(gpulib):
    k = dcf.Kernels(gpulib)
    rng = np.random.default_rng(1)
    p = rng.standard_normal(k.count).astype(np.float32)
    g = rng.standard_normal(k.count).astype(np.float32)
    pd, gd = torch.from_numpy(p.copy()).cuda(), torch.from_numpy(g).cuda()
    m1, m2 = torch.zeros_like(pd), torch.zeros_like(pd)
    for step in (1, 2):
        k.adam(pd.data_ptr(), gd.data_ptr(), m1.data_ptr(), m2.data_ptr(), step, 1e-2, 0.9, 0.999, 1e-8, None)
    pr = torch.from_numpy(p.astype(np.float64)).requires_grad_(True)
    opt = torch.optim.Adam([pr], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    for _ in range(2):
        opt.zero_grad()
        pr.grad = torch.from_numpy(g.astype(np.float64))
        opt.step()
    assert np.allclose(pd.cpu().numpy(), pr.detach().numpy(), rtol=1e-5, atol=1e-6)


def test_features_match_numpy(gpulib):
    x = workloads.spiral_nodes(4, 2000, 6.0, 0.3, 1e-4, np.random.default_rng(2)).astype(np.float32)
    n = [128, 128]
    f = dcf.raw_features(gpulib, x, n).view(-1, 8).cpu().numpy()
    c = np.floor((x.astype(np.float32) + np.float32(0.5)) * np.float32(128)).astype(np.int64) % 128
    cnt = np.zeros((128, 128), np.int64)
    np.add.at(cnt, (c[:, 0], c[:, 1]), 1)
    for q, r in enumerate((1, 2, 4)):
        box = np.zeros_like(cnt)
        for a in range(-r, r + 1):
            for b in range(-r, r + 1):
                box += np.roll(np.roll(cnt, -a, 0), -b, 1)
        assert np.allclose(f[:, q], np.log1p(box[c[:, 0], c[:, 1]]), rtol=1e-5)
    th = np.arctan2(x[:, 1], x[:, 0])
    assert np.allclose(f[:, 3], 2 * np.hypot(x[:, 0], x[:, 1]), atol=1e-6)
    assert np.allclose(f[:, 4], np.cos(th), atol=1e-5)
    assert np.allclose(f[:, 7], np.sin(2 * th), atol=1e-5)


def test_fixed_point_weights_match_oracle(gpulib):
    N, m = [32, 32], 6
    x = workloads.spiral_nodes(4, 512, 6.0, 0.7, 1e-4, np.random.default_rng(3))
    x32 = x.astype(np.float32)
    w = dcf.fixed_point_weights(gpulib, N, x32, m, iters=5).cpu().numpy().astype(np.float64)
    o = oracle.OraclePlan(N, len(x), n=[64, 64], m=m, single=False)
    o.set_nodes(x32.astype(np.float64))
    o.precompute()
    wr = np.ones(len(x))
    for _ in range(5):
        wr = wr / np.abs(o.trafo(o.adjoint(wr.astype(complex))))
    assert np.linalg.norm(w - wr) / np.linalg.norm(wr) < 1e-4


def test_learned_weights_speed_up_cgnr(gpulib):
    """Small end-to-end run: trained on 6 spirals, the learned weights bring
    the relative data residual below 1e-5 in fewer CGNR iterations than the
    unweighted solver on a held-out spiral (noiseless data)."""
    N, m, arms, samples = [64, 64], 6, 8, 1024
    feats, targets = dcf.build_training_set(gpulib, N, m, range(6), arms, samples)
    net = dcf.DensityNet(gpulib)
    net.fit_standardisation(feats)
    for f in feats:
        net.standardise(f, f.numel() // 8)
    feat = torch.cat(feats)
    target = torch.cat(targets)
    hist = net.train(feat, target, epochs=30, batch=4096, lr=3e-3)
    assert hist[-1] < 0.9 * hist[0], hist
    x = dcf.spiral(1000, arms, samples)
    w = net.weights(gpulib, x, [128, 128]).cpu().numpy()
    f_true = workloads.ellipse_phantom(64, 20, seed=7)
    p = Plan(gpulib, False, N, len(x), n=[128, 128], m=m, flags=infft.PLAN_FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = f_true
    p.trafo()
    y = p.f.copy()
    p.finalize()
    plain = infft.time_to_tolerance(gpulib, False, N, x, m, y, tol=1e-5, max_iter=4000)
    learned = infft.time_to_tolerance(gpulib, False, N, x, m, y, tol=1e-5, w=w, max_iter=4000)
    plain.pop("f")
    learned.pop("f")
    print("plain", plain, "learned", learned, "loss", hist[0], hist[-1])
    assert learned["reached"], learned
    assert learned["iters"] < plain["iters"], (learned, plain)
