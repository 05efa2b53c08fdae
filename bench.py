#!/usr/bin/env python3
"""Benchmark of the NFFT transform path: nodes/s for one trafo + one adjoint.

Workload (default): 3-D single-precision NFFT, N = 128^3, sigma = 2
(n = 256^3), Kaiser-Bessel window m = 4, M = 2^24 nodes iid uniform in
[-1/2, 1/2)^3 (seed 0), f_hat and the adjoint input with real and imaginary
parts iid U(-1, 1).  A step is one nfftf_trafo plus one nfftf_adjoint over
all M nodes; value = nodes per step / step time (whole job over all ranks).

* value:  device-resident operands (gb_trafo_ptr / gb_adjoint_ptr), timed
          with CUDA events on the plan's stream;
* e2e:    the reference-facing C ABI (nfftf_trafo / nfftf_adjoint) on host
          arrays, host<->device copies inside the timed region;
* cpu_baseline / --impl reference: the oracle's OpenMP restatement of the
          reference algorithm (PRE_PSI tables, sorted nodes, blockwise
          adjoint) on all of this host's cores, over the whole workload.

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "nodes/s fwd+adj, %HBM roofline; iNFFT time to 1e-5 rel. err: learned vs plain"
UNIT = "nodes/s"


def workload(name):
    k3 = ("k_b3_cell", "k_bt3_col")
    if name == "small":  # for profiler captures of the same kernels
        return dict(name="3-D NFFT FP32 N=64^3 n=128^3 m=4 M=2^21 uniform", d=3, N=[64] * 3,
                    n=[128] * 3, m=4, M=1 << 21, dist="uniform", kernels=k3, l2="inputs larger than L2 "
                    "(x 25 MB, grid 16.8 MB, f 16.8 MB: not all); profiler captures only")
    if name == "radial-pair":  # the inverse-NFFT workload's transforms (2-D column kernels)
        return dict(name="2-D NFFT FP32 N=256^2 n=512^2 m=6 radial 402x512", d=2, N=[256, 256], n=[512, 512],
                    m=6, M=402 * 512, dist="radial", kernels=("k_b2_col", "k_bt2_col"),
                    l2="L2-resident: grid 2.1 MB, nodes 1.6 MB, f 1.6 MB stay in L2 between steps, as "
                       "they do between the steps of the iterative inverse NFFT")
    dist = "clustered" if name == "clustered" else "uniform"
    return dict(name="3-D NFFT FP32 N=128^3 n=256^3 m=4 M=2^24 %s" % dist, d=3, N=[128] * 3,
                n=[256] * 3, m=4, M=1 << 24, dist=dist, kernels=k3,
                l2="inputs larger than L2 (x 201 MB, grid 134 MB, f 134 MB per rank); no flush")


def make_nodes(wl, seed):
    from nfft_gb300 import workloads
    if wl["dist"] == "radial":
        return workloads.radial_nodes(402, 512).astype(np.float32)
    return workloads.cube_nodes(wl["M"], wl["d"], wl["dist"], seed)


def algorithmic_bytes_B(wl):
    """Bytes of one B or B^T launch: nodes (d reals), samples (one complex)
    and the oversampled grid once (FP32: r = 4, c = 8)."""
    n_total = int(np.prod(wl["n"]))
    return wl["M"] * (wl["d"] * 4 + 8) + n_total * 8


def flops_B(wl):
    w = 2 * wl["m"] + 2
    return 4.0 * w ** wl["d"] * wl["M"]


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the first sample is in (nvidia-smi
            # takes some 0.1 s to start; a region of a few ms would otherwise
            # end before it reports)
            t_end = time.perf_counter() + 2.0
            while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.005)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [v.strip() for v in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def cpu_pair(wl, x, steps, warmup):
    """Time the oracle's restatement of the reference (OpenMP over all host
    cores, PRE_PSI tables, sorted nodes, the blockwise adjoint) on the whole
    workload: node set-up once, then warmup + steps trafo + adjoint pairs, as
    the reference's examples/nfft/nfft_benchomp_detail.c:96-118 times them
    (D, FFT and B of each call from its stage timers).  Returns per-step dicts
    and the set-up time."""
    import oracle
    o = oracle.OraclePlan(wl["N"], wl["M"], n=wl["n"], m=wl["m"], single=True, sort=True,
                          blockwise=True, pre_psi=True)
    o.set_nodes(x)
    t0 = time.perf_counter()
    o.precompute()
    t_pre = time.perf_counter() - t0
    rng = np.random.default_rng(1)
    NN = int(np.prod(wl["N"]))
    fh = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f = (rng.uniform(-1, 1, wl["M"]) + 1j * rng.uniform(-1, 1, wl["M"])).astype(np.complex64)
    out = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        o.trafo(fh)
        t1 = time.perf_counter()
        st_t = o.stage_times()
        o.adjoint(f)
        t2 = time.perf_counter()
        st_a = o.stage_times()
        if it >= warmup:
            out.append(dict(pair_s=t2 - t0, trafo_s=t1 - t0, adjoint_s=t2 - t1,
                            stages_s={"trafo_D": st_t[0], "trafo_FFT": st_t[1], "trafo_B": st_t[2],
                                      "adjoint_BT": st_a[2], "adjoint_FFT": st_a[1], "adjoint_DT": st_a[0]},
                            nodes_per_s=wl["M"] / (t2 - t0)))
    o.close()
    return out, t_pre


def cpu_summary(wl, steps, t_pre):
    """Median pair rate and stage times of cpu_pair's steps."""
    rate = statistics.median(s["nodes_per_s"] for s in steps)
    stages = {k: round(1e3 * statistics.median(s["stages_s"][k] for s in steps), 2) for k in steps[0]["stages_s"]}
    sample = ("oracle OpenMP restatement of the reference (PRE_PSI tables, sorted nodes, blockwise adjoint, "
              "project radix-2 FFT) on all %d nodes with the full grid, %d threads; median of %d "
              "trafo + adjoint pairs after the node set-up (%.1f s)" % (wl["M"], cpu_cores(), len(steps), t_pre))
    return rate, stages, sample


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    x = make_nodes(wl, 0)
    steps, t_pre = cpu_pair(wl, x, args.steps, args.warmup)
    value, stages, sample = cpu_summary(wl, steps, t_pre)
    ms = statistics.mean(s["pair_s"] for s in steps) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(wl),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "stages_ms_median": stages, "precompute_s": round(t_pre, 3)}
    print(json.dumps(line), flush=True)
    return 0


def config_of(wl):
    return {"workload": wl["name"], "d": wl["d"], "N": wl["N"], "n": wl["n"], "m": wl["m"],
            "M": wl["M"], "nodes": wl["dist"], "precision": "complex64",
            "window": "Kaiser-Bessel", "l2_between_steps": wl["l2"]}


# ------------------------------------------------------------------ GPU side
def accuracy_sample(lib, wl, x, fh_host, f_host, f_out, n_trafo=256, n_adj=1024):
    """Relative l2 error against the FP64 NDFT (nfft_trafo_direct /
    nfft_adjoint_direct on the GPU): the benchmark's own trafo output on its
    first n_trafo nodes, and the adjoint of a subset plan of n_adj nodes with
    the same N, n, m (the adjoint of a subset is its own problem)."""
    from nfft_gb300 import abi
    from nfft_gb300.plan import Plan
    N, n, m = wl["N"], wl["n"], wl["m"]
    flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE)
    got = f_out[: 2 * n_trafo].cpu().numpy().view(np.complex64).astype(np.complex128)
    q = Plan(lib, False, N, n_trafo, n=n, m=m, flags=flags)
    q.x[:] = x[:n_trafo].astype(np.float64)
    q.f_hat[:] = fh_host.astype(np.complex128)
    q.trafo_direct()
    e_t = float(np.linalg.norm(got - q.f) / np.linalg.norm(q.f))
    q.finalize()
    s = Plan(lib, True, N, n_adj, n=n, m=m, flags=flags)
    s.x[:] = x[:n_adj]
    s.precompute_one_psi()
    s.f[:] = f_host[:n_adj]
    s.adjoint()
    got_a = s.f_hat.astype(np.complex128)
    s.finalize()
    q = Plan(lib, False, N, n_adj, n=n, m=m, flags=flags)
    q.x[:] = x[:n_adj].astype(np.float64)
    q.f[:] = f_host[:n_adj].astype(np.complex128)
    q.adjoint_direct()
    e_a = float(np.linalg.norm(got_a - q.f_hat) / np.linalg.norm(q.f_hat))
    q.finalize()
    return {"trafo_rel_l2_vs_ndft": e_t, "trafo_nodes": n_trafo,
            "adjoint_rel_l2_vs_ndft": e_a, "adjoint_subset_nodes": n_adj}


def max_over_ranks(v, dist=None, device="cpu"):
    """The largest of the ranks' values v (v itself on one rank): a replica
    run is as slow as its slowest rank."""
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(ms_total, nodes_per_rank, steps, dist=None, device="cpu"):
    """Whole-job rate of replicas (each rank transforms its own nodes, no data
    exchange): (ms per step from the slowest rank, nodes of all ranks / s)."""
    world = dist.get_world_size() if dist is not None else 1
    ms_step = max_over_ranks(ms_total, dist, device) / steps
    return ms_step, nodes_per_rank * world / (ms_step * 1e-3)


def run_gpu(args, wl):
    import torch
    import nfft_gb300
    from nfft_gb300 import abi
    from nfft_gb300.plan import Plan

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    lib = nfft_gb300.lib()
    M, N, n, m = wl["M"], wl["N"], wl["n"], wl["m"]
    NN = int(np.prod(N))
    flags = (abi.PRE_PHI_HUT | abi.PRE_PSI | abi.MALLOC_X | abi.MALLOC_F_HAT | abi.MALLOC_F
             | abi.FFTW_INIT | abi.FFT_OUT_OF_PLACE | abi.NFFT_SORT_NODES)
    p = Plan(lib, True, N, M, n=n, m=m, flags=flags)
    x = make_nodes(wl, rank)
    p.x[:] = x
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p.precompute_one_psi()
    t_pre = time.perf_counter() - t0
    if wl["d"] == 3:  # which form of B node set-up chose for this density
        qk = lib.nfftf_gb_b3_kernel
        qk.restype, qk.argtypes = C.c_int, [C.c_void_p]
        wl = dict(wl, kernels=("k_b3_col" if qk(C.addressof(p.p)) == 1 else "k_b3_cell", wl["kernels"][1]))

    rng = np.random.default_rng(100 + rank)
    fh_host = (rng.uniform(-1, 1, NN) + 1j * rng.uniform(-1, 1, NN)).astype(np.complex64)
    f_host = (rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).astype(np.complex64)
    dev = torch.device("cuda", local)
    fh_in = torch.from_numpy(fh_host.view(np.float32)).to(dev)
    f_in = torch.from_numpy(f_host.view(np.float32)).to(dev)
    f_out = torch.empty(2 * M, dtype=torch.float32, device=dev)
    fh_out = torch.empty(2 * NN, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    pp = C.byref(p.p)
    lib.nfftf_gb_set_stream(pp, C.c_void_p(stream.cuda_stream))
    trafo = lib.nfftf_gb_trafo_ptr
    adjoint = lib.nfftf_gb_adjoint_ptr
    trafo.argtypes = adjoint.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    pa = C.addressof(p.p)

    def step():
        trafo(pa, fh_in.data_ptr(), f_out.data_ptr())
        adjoint(pa, f_in.data_ptr(), fh_out.data_ptr())

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()

    # ---- timed region (device-resident)
    begin = lib.nfftf_gb_timing_begin
    begin.argtypes = [C.c_void_p, C.c_int]
    end = lib.nfftf_gb_timing_end
    end.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int)]
    begin(pa, 2 * args.steps)
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms_total = ev0.elapsed_time(ev1)
    sums = (C.c_float * 7)()
    counts = (C.c_int * 2)()
    end(pa, sums, counts)
    # trafo: k_d_pad + B; adjoint: B^T + k_d_crop (cuFFT and memsets not counted)
    launches = 4 * args.steps
    ms_step, value = replica_rate(ms_total, M, args.steps, dist, dev)

    # ---- accuracy of this very run against the FP64 NDFT (on the GPU)
    accuracy = None
    if not args.no_accuracy:
        accuracy = accuracy_sample(lib, wl, x, fh_host, f_host, f_out)

    # ---- e2e through the C ABI on host arrays (copies inside the timed region)
    e2e_times = []
    for it in range(args.warmup + args.steps):
        p.f_hat[:] = fh_host
        barrier()
        t0 = time.perf_counter()
        p.trafo()
        p.adjoint()
        t1 = time.perf_counter()
        if it >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_s = max_over_ranks(sum(e2e_times) / len(e2e_times), dist, dev)
    e2e_value = M * world / e2e_s
    h2d = NN * 8 + M * 8
    d2h = M * 8 + NN * 8

    # ---- roofline of the dominant kernel
    nT, nA = max(counts[0], 1), max(counts[1], 1)
    stage = {"trafo_D_ms": sums[0] / nT, "trafo_FFT_ms": sums[1] / nT, "trafo_B_ms": sums[2] / nT,
             "adjoint_memset_ms": sums[3] / nA, "adjoint_BT_ms": sums[4] / nA,
             "adjoint_FFT_ms": sums[5] / nA, "adjoint_DT_ms": sums[6] / nA}
    b_ms, bt_ms = stage["trafo_B_ms"], stage["adjoint_BT_ms"]
    kb, kbt = wl["kernels"]
    dom, dom_ms = (kbt + " (B^T spreading)", bt_ms) if bt_ms >= b_ms else (kb + " (B interpolation)", b_ms)
    peaks, peak_kind = measured_peaks()
    bytes_b = algorithmic_bytes_B(wl)
    achieved = bytes_b / (dom_ms * 1e-3) / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            tr = json.load(fh)
        key = (kbt if bt_ms >= b_ms else kb) + "/" + wl["dist"]
        traffic = tr.get(key)
    except Exception:
        pass
    fp32_peak = 152 * 128 * 2 * (clk["sm_mhz"] if clk else 1900.0) * 1e6 / 1e12
    roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 5), "traffic": traffic,
            "kernel": dom, "algorithmic_bytes_per_launch": bytes_b, "launch_ms": round(dom_ms, 4),
            "peak_source": peak_kind,
            "fp32_issue": {"flops_per_launch": flops_B(wl),
                           "achieved_tflops": round(flops_B(wl) / (dom_ms * 1e-3) / 1e12, 3),
                           "peak_tflops_at_clock": round(fp32_peak, 1),
                           "frac": round(flops_B(wl) / (dom_ms * 1e-3) / 1e12 / fp32_peak, 4)}}
    pair_bytes = 2 * (bytes_b + 2 * int(np.prod(n)) * 8 + (NN + int(np.prod(n))) * 8)
    hbm_pair = pair_bytes / (ms_step * 1e-3) / 1e9

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        steps, t_pre_cpu = cpu_pair(wl, x, 5, 1)
        v, stages_cpu, sample = cpu_summary(wl, steps, t_pre_cpu)
        cpu = {"value": v, "unit": UNIT, "cores": cpu_cores(), "kind": "port", "sample": sample,
               "stages_ms_median": stages_cpu}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(wl), "parallelism": "replicas x%d" % world,
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                    "ms_per_step_median": float(np.median(e2e_times)) * 1e3,
                    "ms_per_step_min": float(np.min(e2e_times)) * 1e3},
            "clocks": clk, "gpu_launches": launches,
            "stages_ms": {k: round(v, 4) for k, v in stage.items()},
            "pair_hbm_gbs_algorithmic": round(hbm_pair, 1),
            "pair_hbm_frac": round(hbm_pair / peaks["hbm_gbs"], 4),
            "precompute_s": round(t_pre, 4), "accuracy": accuracy}
    p.finalize()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_infft(args):
    """Mixed-precision inverse NFFT on 2-D radial k-space: N = 256^2, sigma = 2,
    m = 6, 402 spokes x 512 samples, 20-ellipse phantom (seed 1), y = A f_true
    (FP64 transform) + complex Gaussian noise at 40 dB SNR.  K CGNR steps per
    solver -- FP64; FP32 transforms with FP64 inner products; the same with an
    FP64 residual refresh every 10 steps -- enqueued back to back and timed
    (value: the FP32 solver's time); reported per solver: ms per step, the
    error against f_true after K steps and its smallest value over the steps
    (noisy data: CGNR semi-converges), the distance to the FP64 solver's
    iterate, and the true data residual (FP64 transform)."""
    import torch
    import nfft_gb300
    from nfft_gb300 import infft, workloads
    from nfft_gb300.plan import Plan
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lib = nfft_gb300.lib()
    N, m, K = [256, 256], 6, args.iters
    x = workloads.radial_nodes(402, 512)
    f_true = workloads.ellipse_phantom(256, 20, seed=1)
    M = len(x)
    p = Plan(lib, False, N, M, n=[512, 512], m=m, flags=infft.PLAN_FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = f_true
    p.trafo()
    y = workloads.add_noise(p.f.copy(), 40.0, np.random.default_rng(1))
    p.finalize()
    nt = np.linalg.norm(f_true)
    solvers = {"fp64": (False, 0), "fp32": (True, 0), "fp32_refresh10": (True, 10)}
    if args.solver != "all":
        solvers = {args.solver: solvers[args.solver]}
    runs = {}
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    for name, (single, refresh) in solvers.items():
        infft.run_iterations(lib, single, N, x, m, y, 3, refresh=refresh)  # warm-up
        f, sec, dots = infft.run_iterations(lib, single, N, x, m, y, K, refresh=refresh)
        runs[name] = dict(f=f, seconds=sec)
    clk = clocks.stop()
    res = infft.TrueResidual(lib, N, x, m, y)
    out = {}
    for name, (single, refresh) in solvers.items():
        # the error trajectory over the steps (untimed: 10 steps at a time)
        s = infft.CGNR(lib, single, N, x, m, y, refresh=refresh)
        s.set_sync(0)
        s.before_loop()
        errs = []
        for _ in range(K // 10):
            s.steps(10)
            s.sync()
            errs.append(float(np.linalg.norm(s.f_hat - f_true) / nt))
        s.close()
        r = runs[name]
        out[name] = {"seconds": r["seconds"], "ms_per_step": 1e3 * r["seconds"] / K,
                     "rel_err_vs_f_true": float(np.linalg.norm(r["f"] - f_true) / nt),
                     "min_rel_err_vs_f_true": min(errs) if errs else None,
                     "true_rel_residual": res(r["f"])}
        if "fp64" in runs:
            f64 = runs["fp64"]["f"]
            out[name]["rel_dist_to_fp64_iterate"] = float(np.linalg.norm(r["f"] - f64) / np.linalg.norm(f64))
    res.close()
    head = "fp32" if "fp32" in out else next(iter(out))
    line = {"metric": "iNFFT CGNR wall time for K steps, 2-D radial (FP32 transforms, FP64 inner products)",
            "value": out[head]["seconds"], "unit": "s", "n_gpus": 1, "higher_is_better": False,
            "dtype": "f32 (FP64 inner products)", "data": "synthetic",
            "config": {"workload": "2-D radial iNFFT N=256^2 n=512^2 m=6 402x512 spokes, 20 ellipses, 40 dB",
                       "M": M, "solver": "CGNR", "iterations": K},
            "clocks": clk, "runs": out}
    print(json.dumps(line), flush=True)
    return 0


def run_convergence(args):
    """Where CGNR gets on the spiral trajectory of the learned workload (one
    trajectory, noiseless data, 20-ellipse phantom): for the FP64 solver, the
    FP32 solver with FP64 inner products and the same with an FP64 residual
    refresh every 10 steps, unweighted and with the density weights after
    `--fp-iters` fixed-point steps, every
    10 steps the true relative data residual (FP64 transform), the relative
    image error against the phantom and the image error in the band
    |nu| <= 0.45 the samples determine; reported: the steps to a 1e-5 residual
    and the smallest errors reached within --iters steps (unweighted; half as
    many with weights; the same for the weights after twenty steps, for
    comparison).  A last setting runs the FP64 solver with the damping
    of the reference's MRI reconstruction (PRECOMPUTE_DAMP, w_hat = 1 on the
    image's inscribed disk, applications/mri/mri2d/reconstruct_data_2d.c) on
    the phantom restricted to that disk."""
    import torch
    import nfft_gb300
    from nfft_gb300 import dcf, infft, workloads
    from nfft_gb300.plan import Plan
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lib = nfft_gb300.lib()
    N, m = [256, 256], 6
    x = dcf.spiral(1000, 16, 8192)
    f_true = workloads.ellipse_phantom(256, 20, seed=1000)
    p = Plan(lib, False, N, len(x), n=[512, 512], m=m, flags=infft.PLAN_FLAGS)
    p.x[:] = x
    p.precompute_one_psi()
    p.f_hat[:] = f_true
    p.trafo()
    y = p.f.copy()
    p.finalize()
    res = infft.TrueResidual(lib, N, x, m, y)
    wfp = dcf.fixed_point_weights(lib, N, x.astype(np.float32), m, args.fp_iters).cpu().numpy()
    # twenty steps, for comparison: the iteration amplifies the sidelobes of
    # the point-spread function, and the solver slows down
    wfp20 = dcf.fixed_point_weights(lib, N, x.astype(np.float32), m, 20).cpu().numpy()
    out = {}
    # the damped setting solves for the phantom restricted to the image's
    # inscribed disk, from the data of that restricted phantom
    damp = infft.disk_damping(256)
    q = Plan(lib, False, N, len(x), n=[512, 512], m=m, flags=infft.PLAN_FLAGS)
    q.x[:] = x
    q.precompute_one_psi()
    q.f_hat[:] = f_true * damp
    q.trafo()
    y_disk = q.f.copy()
    q.finalize()
    res_disk = infft.TrueResidual(lib, N, x, m, y_disk)
    settings = (("unweighted", None, None, args.iters), ("fixed_point_weights", wfp, None, args.iters // 2),
                ("fixed_point_weights_20_steps", wfp20, None, args.iters // 2),
                ("disk_damped", None, damp, args.iters))
    for wname, w, wh, total in settings:
        yy, ft, rr = (y_disk, f_true * damp, res_disk) if wh is not None else (y, f_true, res)
        for sname, single, refresh in (("fp64", False, 0), ("fp32", True, 0), ("fp32_refresh10", True, 10)):
            if wh is not None and sname != "fp64":
                continue
            s = infft.CGNR(lib, single, N, x, m, yy, w=w, refresh=refresh, w_hat=wh)
            s.set_sync(0)
            s.before_loop()
            rows = []
            for k in range(total // 10):
                s.steps(10)
                s.sync()
                f = s.f_hat
                rows.append(((k + 1) * 10, rr(f)) + infft.image_errors(f, ft))
            s.close()
            a = np.array(rows)
            out["%s/%s" % (wname, sname)] = {
                "steps_to_resid_1e-5": next((int(r[0]) for r in rows if r[1] < 1e-5), None),
                "min_resid": float(a[:, 1].min()), "min_image_err": float(a[:, 2].min()),
                "min_band_err": float(a[:, 3].min()), "steps": total}
    res.close()
    res_disk.close()
    line = {"metric": "CGNR convergence on one spiral trajectory (2-D, N=256^2, m=6, noiseless)",
            "value": out["unweighted/fp32"]["steps_to_resid_1e-5"], "unit": "steps", "n_gpus": 1,
            "higher_is_better": False, "data": "synthetic", "runs": out}
    print(json.dumps(line), flush=True)
    return 0


def run_dcf_steps(args):
    """Steps of FP32 CGNR (FP64 inner products) to a 1e-5 true relative data
    residual on held-out spirals of the learned workload (ellipse phantoms,
    noiseless data), with the density weights after k fixed-point steps
    w <- w/|A A^H w| from w = 1, for each k of --fp-list, and unweighted:
    how many steps the density weights should take.  value = the k with the
    smallest median step count."""
    import torch
    import nfft_gb300
    from nfft_gb300 import dcf, infft, workloads
    from nfft_gb300.plan import Plan
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lib = nfft_gb300.lib()
    N, m, n = [256, 256], 6, [512, 512]
    ks = [int(v) for v in args.fp_list.split(",")]
    steps = {"unweighted": []}
    for i in range(args.test):
        x = dcf.spiral(1000 + i, 16, 8192)
        f_true = workloads.ellipse_phantom(256, 20, seed=1000 + i)
        p = Plan(lib, False, N, len(x), n=n, m=m, flags=infft.PLAN_FLAGS)
        p.x[:] = x
        p.precompute_one_psi()
        p.f_hat[:] = f_true
        p.trafo()
        y = p.f.copy()
        p.finalize()
        r = infft.time_to_tolerance(lib, True, N, x, m, y, tol=1e-5, max_iter=args.max_iter)
        steps["unweighted"].append(r["iters"] if r["reached"] else None)
        for k in ks:
            w = dcf.fixed_point_weights(lib, N, x.astype(np.float32), m, k).cpu().numpy()
            r = infft.time_to_tolerance(lib, True, N, x, m, y, tol=1e-5, w=w, max_iter=args.max_iter)
            steps.setdefault("fixed_point_%d" % k, []).append(r["iters"] if r["reached"] else None)

    def median(v):  # a run that did not converge counts as more than the cap
        return float(np.median([args.max_iter + 1 if s is None else s for s in v]))

    med = {name: median(v) for name, v in steps.items()}
    best = min(ks, key=lambda k: med["fixed_point_%d" % k])
    line = {"metric": "FP32 CGNR steps to a 1e-5 relative data residual vs fixed-point steps of the density "
            "weights (2-D spirals)", "value": best, "unit": "fixed-point steps", "n_gpus": 1,
            "higher_is_better": False, "data": "synthetic",
            "config": {"workload": "2-D spiral iNFFT N=256^2 n=512^2 m=6, 16 arms x 8192", "trajectories": args.test,
                       "cap": args.max_iter, "criterion": "||y - A f|| / ||y|| < 1e-5, A in FP64, "
                       "checked every 5 steps"},
            "median_steps": med,
            "not_reached": {name: int(sum(s is None for s in v)) for name, v in steps.items()},
            "per_trajectory": steps}
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args):
    """1024 independent 2-D complex64 plans: N_t log-uniform over {32..256},
    sigma = 2, m in {4, 6}, M log-uniform in [1024, 65536], uniform nodes.
    value = all plans' nodes per (trafo + adjoint of every plan) / time, with
    the autotuned batch replayed as one CUDA graph; also reported: the same
    batch as stream launches, before autotuning, and the plans one at a time
    through their own device transforms."""
    import torch
    import nfft_gb300
    from nfft_gb300 import batch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lib = nfft_gb300.lib()
    t0 = time.perf_counter()
    plans, data = batch.random_plans(lib, args.plans, seed=0)
    t_setup = time.perf_counter() - t0
    nodes = sum(d[2] for d in data)
    put, _ = batch.device_io(lib)
    rng = np.random.default_rng(5)
    for p, (N, m, M, x) in zip(plans, data):
        put(p, "f_hat", (rng.uniform(-1, 1, N[0] * N[1]) + 1j * rng.uniform(-1, 1, N[0] * N[1])))
    # one plan at a time (each plan's own D / cuFFT / B launches, no host sync in between)
    tr = lib.nfftf_gb_trafo_device
    ad = lib.nfftf_gb_adjoint_device
    tr.argtypes = ad.argtypes = [C.c_void_p]
    addrs = [C.addressof(p.p) for p in plans]
    for a in addrs[:8]:
        tr(a)
        ad(a)
    torch.cuda.synchronize()
    reps = args.steps
    t0 = time.perf_counter()
    for _ in range(reps):
        for a in addrs:
            tr(a)
            ad(a)
    torch.cuda.synchronize()
    t_seq = (time.perf_counter() - t0) / reps
    b = batch.Batch(lib, plans)
    b.time(args.warmup, 0)
    ms_stream_untuned = b.time(reps, 0)
    ms_graph_untuned = b.time(reps, 1)
    t0 = time.perf_counter()
    classes = b.autotune(reps=3)
    t_tune = time.perf_counter() - t0
    b.time(args.warmup, 1)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ms_stream = b.time(reps, 0)
    ms_graph = b.time(max(reps, 50), 1)
    clk = clocks.stop()
    cfgs = {}
    for k in range(len(plans)):
        cfgs.setdefault("%s" % (b.config(k),), 0)
        cfgs["%s" % (b.config(k),)] += 1
    line = {"metric": "nodes/s fwd+adj, batched uneven 2-D plans (one persistent graph-captured launch)",
            "value": nodes / (ms_graph * 1e-3), "unit": "nodes/s", "n_gpus": 1, "steps": reps,
            "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "%d 2-D complex64 plans, N_t in {32..256}, m in {4,6}, M in [1024,65536]"
                       % len(plans), "nodes": nodes, "work_items": b.items},
            "ms_per_round": {"graph_autotuned": ms_graph, "stream_autotuned": ms_stream,
                             "graph_untuned": ms_graph_untuned, "stream_untuned": ms_stream_untuned,
                             "one_plan_at_a_time_own_streams": t_seq * 1e3},
            "speedup_vs_one_at_a_time": t_seq * 1e3 / ms_graph, "clocks": clk,
            "autotune": {"classes": classes, "seconds": t_tune, "chosen_T_tpn_counts": cfgs},
            "setup_s": t_setup}
    b.close()
    # the same plans one after another on one stream
    ss = lib.nfftf_gb_set_stream
    ss.argtypes = [C.c_void_p, C.c_void_p]
    s = torch.cuda.Stream()
    for a in addrs:
        ss(a, C.c_void_p(s.cuda_stream))
    for a in addrs[:8]:
        tr(a)
        ad(a)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        for a in addrs:
            tr(a)
            ad(a)
    torch.cuda.synchronize()
    line["ms_per_round"]["one_plan_at_a_time_one_stream"] = (time.perf_counter() - t0) / reps * 1e3
    for a in addrs:
        ss(a, None)
    for p in plans:
        p.finalize()
    print(json.dumps(line), flush=True)
    return 0


def run_learned(args):
    """Learned density-compensation weights on 2-D spirals: N = 256^2, m = 6,
    16 interleaved Archimedean arms x 8192 samples (r = t/2, angle
    2 pi (24 t + a/16) + random rotation, radius jitter 1e-4).  The MLP is
    trained on `--train` seeded trajectories against the density weights after
    `--fp-iters` steps w <- w/|A A^H w| from w = 1 (one by default: 1/|A A^H 1|);
    on `--test` held-out trajectories with ellipse phantoms (noiseless data)
    FP32 CGNR (FP64 inner products) runs with the learned weights, with those
    density weights and unweighted until the true
    relative data residual ||y - A f|| / ||y|| (A the FP64 transform) falls
    below 1e-5.  value = median wall time with the learned weights, their
    inference (features + network) included; the image errors at that point
    (whole image, and the band |nu| <= 0.45 the samples determine) are
    reported beside it."""
    import torch
    import nfft_gb300
    from nfft_gb300 import dcf, infft, workloads
    from nfft_gb300.plan import Plan
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lib = nfft_gb300.lib()
    N, m, arms, samples = [256, 256], 6, 16, 8192
    n = [512, 512]
    t0 = time.perf_counter()
    feats, targets = dcf.build_training_set(lib, N, m, range(args.train), arms, samples, fp_iters=args.fp_iters)
    t_data = time.perf_counter() - t0
    net = dcf.DensityNet(lib)
    net.fit_standardisation(feats[: min(16, len(feats))])
    for f in feats:
        net.standardise(f, f.numel() // 8)
    feat, target = torch.cat(feats), torch.cat(targets)
    del feats, targets
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = net.train(feat, target, epochs=args.epochs, batch=1 << 16, lr=2e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del feat, target
    rows = []
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    for i in range(args.test):
        x = dcf.spiral(1000 + i, arms, samples)
        f_true = workloads.ellipse_phantom(256, 20, seed=1000 + i)
        p = Plan(lib, False, N, len(x), n=n, m=m, flags=infft.PLAN_FLAGS)
        p.x[:] = x
        p.precompute_one_psi()
        p.f_hat[:] = f_true
        p.trafo()
        y = p.f.copy()
        p.finalize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w = net.weights(lib, x, n).cpu().numpy()
        t_w = time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        wfp = dcf.fixed_point_weights(lib, N, x.astype(np.float32), m, args.fp_iters).cpu().numpy()
        t_fp = time.perf_counter() - t0
        row = {"weights_s": t_w, "fixed_point_weights_s": t_fp}
        for name, ww in (("plain", None), ("learned", w), ("fixed_point", wfp)):
            r = infft.time_to_tolerance(lib, True, N, x, m, y, tol=1e-5, w=ww, max_iter=args.max_iter)
            f = r.pop("f")
            r["rel_err_vs_f_true"], r["band_err_vs_f_true"] = infft.image_errors(f, f_true)
            if name == "learned":
                r["seconds_with_inference"] = r["seconds"] + t_w
            if name == "fixed_point":
                r["seconds_with_weights"] = r["seconds"] + t_fp
            row[name] = r
        rows.append(row)
    clk = clocks.stop()

    def med(name, key):
        return float(np.median([r[name][key] for r in rows]))

    line = {"metric": "iNFFT time to 1e-5 relative data residual: learned vs plain (2-D spirals)",
            "value": med("learned", "seconds_with_inference"), "unit": "s", "n_gpus": 1,
            "higher_is_better": False, "dtype": "f32 (FP64 inner products)", "data": "synthetic",
            "config": {"workload": "2-D spiral iNFFT N=256^2 n=512^2 m=6, 16 arms x 8192, MLP 8-64-64-1",
                       "train_trajectories": args.train, "test_trajectories": args.test,
                       "epochs": args.epochs, "fixed_point_steps": args.fp_iters,
                       "criterion": "||y - A f|| / ||y|| < 1e-5, A in FP64, checked every 5 steps"},
            "clocks": clk,
            "median": {k: {"seconds": med(k, "seconds"), "iters": med(k, "iters"),
                           "rel_err_vs_f_true": med(k, "rel_err_vs_f_true"),
                           "band_err_vs_f_true": med(k, "band_err_vs_f_true")}
                       for k in ("plain", "learned", "fixed_point")},
            "reached": {k: int(sum(r[k]["reached"] for r in rows)) for k in ("plain", "learned", "fixed_point")},
            "speedup_learned_vs_plain": med("plain", "seconds") / max(med("learned", "seconds_with_inference"), 1e-12),
            "training": {"data_s": t_data, "train_s": t_train, "loss_first": hist[0], "loss_last": hist[-1],
                         "loss_per_epoch": hist},
            "weights_inference_s_median": float(np.median([r["weights_s"] for r in rows])),
            "fixed_point_weights_s_median": float(np.median([r["fixed_point_weights_s"] for r in rows])),
            "speedup_fixed_point_vs_plain": med("plain", "seconds") / max(med("fixed_point", "seconds_with_weights"),
                                                                          1e-12),
            "per_trajectory": rows}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="uniform",
                    choices=["uniform", "clustered", "small", "radial-pair", "infft", "learned", "batched",
                             "convergence", "dcf-steps"])
    ap.add_argument("--plans", type=int, default=1024, help="plans of the batched workload")
    ap.add_argument("--train", type=int, default=256, help="training trajectories (learned)")
    ap.add_argument("--test", type=int, default=32, help="held-out trajectories (learned)")
    ap.add_argument("--epochs", type=int, default=20, help="training epochs (learned)")
    ap.add_argument("--max-iter", type=int, default=3000, help="CGNR iteration cap (learned)")
    ap.add_argument("--fp-iters", type=int, default=1,
                    help="fixed-point steps of the density weights (learned, convergence)")
    ap.add_argument("--fp-list", default="1,2,3,5,10,20,40,80",
                    help="fixed-point step counts compared by the dcf-steps workload")
    ap.add_argument("--iters", type=int, default=100, help="CGNR iterations of the iNFFT workload")
    ap.add_argument("--solver", default="all", choices=["all", "fp64", "fp32", "fp32_refresh10"],
                    help="solvers of the iNFFT workload")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the NDFT accuracy sample")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.workload == "infft":
        return run_infft(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "dcf-steps":
        return run_dcf_steps(args)
    if args.workload == "convergence":
        return run_convergence(args)
    wl =workload(args.workload)
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
