"""Batched 2-D transforms: every plan's batched result equals its own
single-plan nfftf_trafo / nfftf_adjoint (which the parity tests pin to the
reference), in stream and CUDA-graph mode, before and after autotuning."""
import numpy as np
import pytest

from helpers import rel_l2
from nfft_gb300 import batch

pytestmark = pytest.mark.gpu


def _single_results(plans, data, seed):
    refs = []
    for k, (p, (N, m, M, x)) in enumerate(zip(plans, data)):
        r = np.random.default_rng([seed, k, 1])
        fh = (r.uniform(-1, 1, N[0] * N[1]) + 1j * r.uniform(-1, 1, N[0] * N[1])).astype(np.complex64)
        f = (r.uniform(-1, 1, M) + 1j * r.uniform(-1, 1, M)).astype(np.complex64)
        p.f_hat[:] = fh
        p.trafo()
        tf = p.f.copy()
        p.f[:] = f
        p.adjoint()
        tfh = p.f_hat.copy()
        p.f[:] = tf
        p.adjoint()
        tff = p.f_hat.copy()  # A^H A f_hat
        refs.append((fh, f, tf, tfh, tff))
    return refs


@pytest.mark.parametrize("autotune", [False, True, "column", "mixed"])
def test_batch_matches_single_plans(gpulib, autotune):
    plans, data = batch.random_plans(gpulib, 24, seed=3, sizes=(32, 64), mmin=300, mmax=5000)
    refs = _single_results(plans, data, 3)
    b = batch.Batch(gpulib, plans)
    if autotune in ("column", "mixed"):
        # every plan (or every other one) on the column kernels, the rest per node
        for k in range(len(plans)):
            cfg = (32, 0) if autotune == "column" or k % 2 == 0 else (16, 4)
            assert b.set_config(k, *cfg) == 0
            assert b.config(k) == cfg
        assert b.set_config(0, 8, 0) == -1
    elif autotune:
        assert b.autotune(reps=2) >= 1
        cfgs = {b.config(k) for k in range(len(plans))}
        assert all((T in (8, 16, 32) and t in (1, 4, 16)) or (T, t) == (32, 0) for T, t in cfgs)
    put, get = batch.device_io(gpulib)
    for p, (fh, f, *_r) in zip(plans, refs):
        put(p, "f_hat", fh)
    b.run(what=1, mode=0)
    for p, (N, m, M, x), (fh, f, tf, tfh, tff) in zip(plans, data, refs):
        assert rel_l2(get(p, "f", M), tf) < 1e-5
        put(p, "f", f)
    b.run(what=2, mode=0)
    for p, (N, m, M, x), (fh, f, tf, tfh, tff) in zip(plans, data, refs):
        assert rel_l2(get(p, "f_hat", N[0] * N[1]), tfh) < 1e-5
        put(p, "f_hat", fh)
    # graph mode: trafo then adjoint of its result, A^H A f_hat
    b.run(what=3, mode=1)
    for p, (N, m, M, x), (fh, f, tf, tfh, tff) in zip(plans, data, refs):
        assert rel_l2(get(p, "f_hat", N[0] * N[1]), tff) < 1e-5
        put(p, "f_hat", fh)
    b.run(what=3, mode=1)  # the replay gives the same
    for p, (N, m, M, x), (fh, f, tf, tfh, tff) in zip(plans, data, refs):
        assert rel_l2(get(p, "f_hat", N[0] * N[1]), tff) < 1e-5
    assert b.nodes == sum(d[2] for d in data)
    b.close()
    for p in plans:
        p.finalize()


def test_batch_at_full_scale_matches_oracle(gpulib):
    """The batched workload itself -- 1024 plans, N_t in {32..256}, m in {4, 6},
    M log-uniform in [1024, 65536] -- autotuned, each direction one persistent launch; a
    sample of its plans (both cut-offs, both kernel families the autotuner
    chose) checked against the oracle's trafo and adjoint on the same
    single-precision nodes (the reference has no batched form: each plan must
    equal its own nfft_trafo_2d / nfft_adjoint_2d, nfft.c:3808-3998)."""
    import oracle
    plans, data = batch.random_plans(gpulib, 1024, seed=0)
    b = batch.Batch(gpulib, plans)
    assert b.autotune(reps=2) >= 1
    put, get = batch.device_io(gpulib)
    rng = np.random.default_rng(21)
    fhs, fs = [], []
    for p, (N, m, M, x) in zip(plans, data):
        fh = (rng.uniform(-1, 1, N[0] * N[1]) + 1j * rng.uniform(-1, 1, N[0] * N[1])).astype(np.complex64)
        f = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
        fhs.append(fh)
        fs.append(f)
        put(p, "f_hat", fh)
    b.run(what=1, mode=0)
    got_f = [get(p, "f", d[2]) for p, d in zip(plans, data)]
    for p, f in zip(plans, fs):
        put(p, "f", f)
    b.run(what=2, mode=0)
    got_fh = [get(p, "f_hat", d[0][0] * d[0][1]) for p, d in zip(plans, data)]
    cfgs = [b.config(k) for k in range(len(plans))]
    b.close()
    # sample: per (m, kernel family), the first plans in order
    picks, seen = [], {}
    for k, ((N, m, M, x), cfg) in enumerate(zip(data, cfgs)):
        key = (m, cfg[1] == 0)
        if seen.get(key, 0) < 3:
            seen[key] = seen.get(key, 0) + 1
            picks.append(k)
    assert len({(data[k][1], cfgs[k][1] == 0) for k in picks}) >= 3, seen
    for k in picks:
        N, m, M, x = data[k]
        o = oracle.OraclePlan(N, M, n=[2 * N[0], 2 * N[1]], m=m)
        o.set_nodes(x.astype(np.float64))
        o.precompute()
        et = rel_l2(got_f[k].astype(np.complex128), o.trafo(fhs[k].astype(np.complex128)))
        ea = rel_l2(got_fh[k].astype(np.complex128), o.adjoint(fs[k].astype(np.complex128)))
        o.close()
        assert et < 1e-5 and ea < 1e-5, (k, N, m, M, cfgs[k], et, ea)
    for p in plans:
        p.finalize()
