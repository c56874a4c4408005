#!/usr/bin/env python
"""Benchmark: full-MPS construction throughput on GB300 (one JSON line).

Workload (default): the large single instance -- M=144 modes, Haar-random
interferometer, r_i ~ U[1.2, 1.6], eta = 0.45, d = 8, chi = 1024 -- built
end to end: all 143 cut spectra (truncation to chi) and all 144 site
tensors Gamma_i [chi, chi, d] (complex64, the reference's layout) with
split-precision hafnians.  A step is one full build; `value` is sites/s with
the covariance resident in HBM; `e2e` is the same through the public host
API (covariance H2D, every Gamma/Lambda D2H into pinned host memory).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
  torchrun --nproc-per-node N bench.py --gpus N ...   (independent instances per rank)
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "full-MPS build throughput (sites/s), split-precision batched kernels"
UNIT = "sites/s"
# DRAM bytes (read + write) per complex multiply-add of the split hafnian DP,
# from the ncu capture of the M=50, d=6, chi=256 build's DP launches (1001 MB
# for 2.66e8 multiply-adds, profiles/dp_kernel_traffic_M50_d6_chi256.md),
# scaled to each launch's work.
DP_DRAM_BYTES_PER_CMAC = 1001e6 / 2.66e8


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="M144_d8_chi1024",
                   help="M144_d8_chi1024 (default), M50_d6_chi256, M16_d4_chi64, M216_d10_chi2048_banded or batch64")
    p.add_argument("--precision", default="split", choices=["split", "fp64", "fp32"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-budget", type=float, default=20.0)
    p.add_argument("--no-contract", action="store_true")
    p.add_argument("--contract-workload", default="M50_d6_chi256")
    p.add_argument("--contract-photons", type=int, default=4)
    p.add_argument("--no-largest", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-sampler", action="store_true")
    p.add_argument("--no-decomp", action="store_true")
    p.add_argument("--decomp-M", type=int, default=50)
    p.add_argument("--decomp-cpu-M", type=int, default=24)
    p.add_argument("--sampler-workload", default="M50_d6_chi256")
    p.add_argument("--sampler-n", type=int, default=100000)
    return p.parse_args()


def dist_init():
    import torch
    import torch.distributed as dist

    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        with open(self.tmp.name) as f:
            rows = [ln.strip().split(",") for ln in f if ln.strip()]
        os.unlink(self.tmp.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1].split()[0]))
                mx.append(float(r[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def profile_read(lib, h, host=False):
    from bosonsupremacy_gb300 import _lib

    out = {}
    for k, name in (_lib.HOST_CLASSES if host else _lib.KERNEL_CLASSES).items():
        ms, n, w = C.c_double(), C.c_int64(), C.c_double()
        _lib.check(lib.bsg_profile_read(h, k, C.byref(ms), C.byref(n), C.byref(w)), "bsg_profile_read")
        out[name] = {"ms": ms.value, "launches": n.value, "work": w.value}
    return out


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def link_probe(dev_bufs, host_bufs, reps=2):
    """Device-to-host link rate (GB/s): the best of `reps` bare copies of
    every device buffer into its pinned host twin."""
    import torch

    nbytes = sum(b.numel() * b.element_size() for b in dev_bufs)
    best = 0.0
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for h, d in zip(host_bufs, dev_bufs):
            h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()
        best = max(best, nbytes / (time.perf_counter() - t0) / 1e9)
    return best


def measure_contraction(args, lib, handle, peaks):
    """Bond contraction (amplitudes of all patterns with <= k photons) of a
    freshly built FP64 MPS: the sliced tensor-core path (FP64-accurate, the
    parity path) and the fast approximate 3xTF32 path, each timed with CUDA
    events on its stream; the plain FP64 CUDA-core path once for the error."""
    import numpy as np
    import torch

    from bosonsupremacy_gb300 import _lib, ops, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps

    cfg = synthetic.NAMED[args.contract_workload]
    _, sq = synthetic.lossy_covariances(cfg)
    pats = torch.as_tensor(synthetic.low_photon_patterns(cfg.M, args.contract_photons, cfg.d)).cuda()
    mps64 = build_mps(sq, cfg.d, cfg.chi, precision="fp64", out_dtype=torch.complex128)
    g32 = [g.to(torch.complex64) for g in mps64.Gammas]
    stream = torch.cuda.current_stream()
    for _ in range(2):
        ops.pattern_amplitudes(g32, mps64.Lambdas, pats, precision="split")
    torch.cuda.synchronize()
    lib.bsg_profile_reset(handle.h)
    lib.bsg_profile_enable(handle.h, 1)
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        amp = ops.pattern_amplitudes(g32, mps64.Lambdas, pats, precision="split")
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    lib.bsg_profile_enable(handle.h, 0)
    prof = profile_read(lib, handle.h)["contract"]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    amp64 = ops.pattern_amplitudes(mps64.Gammas, mps64.Lambdas, pats, precision="fp64")
    e1.record(stream)
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1)
    # the sliced tensor-core path: complex128 Gamma, FP64 environments, BF16
    # fixed-point slice products with exact FP32 accumulation per level
    ops.pattern_amplitudes(mps64.Gammas, mps64.Lambdas, pats, precision="sliced")
    torch.cuda.synchronize()
    lib.bsg_profile_reset(handle.h)
    lib.bsg_profile_enable(handle.h, 1)
    sl_times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        amp_sl = ops.pattern_amplitudes(mps64.Gammas, mps64.Lambdas, pats, precision="sliced")
        e1.record(stream)
        torch.cuda.synchronize()
        sl_times.append(e0.elapsed_time(e1))
    lib.bsg_profile_enable(handle.h, 0)
    prof_sl = profile_read(lib, handle.h)["contract"]
    p = (amp.abs() ** 2).cpu().numpy()
    p64 = (amp64.abs() ** 2).cpu().numpy()
    psl = (amp_sl.abs() ** 2).cpu().numpy()
    big = p64 > 1e-10 * p64.max()
    rel = np.abs(p - p64)[big] / p64[big]
    rel_sl = np.abs(psl - p64)[big] / p64[big]
    sl_ms = statistics.mean(sl_times)
    sl_useful = prof_sl["work"] / max(1, prof_sl["launches"])
    ms = statistics.mean(times)
    useful = prof["work"] / max(1, prof["launches"])  # real flops of one contraction
    kern_ms = prof["ms"] / max(1, prof["launches"])
    tf32_peak = peaks.get("bf16_tflops")
    achieved = useful / (kern_ms / 1e3) / 1e12
    bf16_peak = peaks.get("bf16_tflops")
    sl_kern_ms = prof_sl["ms"] / max(1, prof_sl["launches"])
    sl_achieved = sl_useful / (sl_kern_ms / 1e3) / 1e12
    return {
        "workload": cfg.label(), "patterns": int(pats.shape[0]), "max_photons": args.contract_photons,
        "path": "sliced: FP64-accurate tensor-core contraction (the parity path)",
        "ms": sl_ms, "patterns_per_s": pats.shape[0] / (sl_ms / 1e3), "fp64_ms": t64, "speedup_vs_fp64": t64 / sl_ms,
        "prob_rel_err_vs_fp64": {"max": float(rel_sl.max()), "median": float(np.median(rel_sl))},
        "note": "complex128 Gamma, FP64 environments; every level's complex GEMM as BF16 fixed-point slice "
                "products (tcgen05 kind::f16) summed exactly per slice level in TMEM",
        "roofline": {"kernel": "sliced_gemm_kernel (BF16 slices, tcgen05) + slicing/env kernels", "bound": "tensor",
                     "achieved": sl_achieved, "unit": "TFLOP/s", "peak": bf16_peak,
                     "frac": sl_achieved / bf16_peak if bf16_peak else None,
                     "peak_source": "measured cuBLAS bf16 burst rate (MEASURED_PEAKS.json)",
                     "work": "8 real flops per complex MAC of the trie contraction (useful; each is S(S+1)/2 "
                             "BF16 slice products, 28 at S = 7)"},
        "tf32x3_fast": {
            "ms": ms, "patterns_per_s": pats.shape[0] / (ms / 1e3), "speedup_vs_fp64": t64 / ms,
            "prob_rel_err_vs_fp64": {"max": float(rel.max()), "median": float(np.median(rel))},
            "note": "approximate: complex64 Gamma, 3xTF32 products accumulated in FP32 -- misses the 1e-6 "
                    "probability tolerance, so it is not the parity path",
            "roofline": {"kernel": "umma_gemm_kernel (3xTF32 tcgen05) + gather/env kernels", "bound": "tensor",
                         "achieved": achieved, "unit": "TFLOP/s",
                         "peak": tf32_peak / 2 if tf32_peak else None,
                         "frac": achieved / (tf32_peak / 2) if tf32_peak else None,
                         "peak_source": "TF32 dense = half the measured cuBLAS bf16 burst rate (nominal ratio)",
                         "work": "8 real flops per complex MAC of the trie contraction (useful; the 3xTF32 split "
                                 "issues 3 tensor products per useful one)"}},
    }


def measure_sampler(args, lib, handle, peaks):
    """GPU sampler (sampling_cpu.py:30-117) on a freshly built MPS: n samples
    in one batch, split precision (3xTF32 chain GEMMs on the tensor cores)
    timed with CUDA events, and the FP32 CUDA-core path once for comparison."""
    import numpy as np
    import torch

    from bosonsupremacy_gb300 import _lib, ops, sampling, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps

    cfg = synthetic.NAMED[args.sampler_workload]
    cov, sq = synthetic.lossy_covariances(cfg)
    mps = build_mps(sq, cfg.d, cfg.chi, precision="split")
    sqrtW = sampling.thermal_sqrtW(cov, sq)
    n = args.sampler_n
    z, u = sampling.draw_random(cfg.M, n, np.random.RandomState(0))
    zd = torch.as_tensor(z).cuda()
    ud = torch.as_tensor(u).cuda()
    dd = cfg.d + 2
    stream = torch.cuda.current_stream()

    def timed(prec, reps):
        ops.sample(mps.Gammas, mps.Lambdas, sqrtW, zd, ud, dd, precision=prec)  # warm-up
        torch.cuda.synchronize()
        lib.bsg_profile_reset(handle.h)
        lib.bsg_profile_enable(handle.h, 1)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ops.sample(mps.Gammas, mps.Lambdas, sqrtW, zd, ud, dd, precision=prec)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        lib.bsg_profile_enable(handle.h, 0)
        prof = profile_read(lib, handle.h)
        return statistics.mean(ts), prof, out

    ms, prof, out = timed("split", 3)
    ms32, _, out32 = timed("fp32", 1)
    same = float((out == out32).all(dim=1).float().mean().item())
    g = prof["contract"]
    achieved = g["work"] / (g["ms"] / 1e3) / 1e12
    tf32 = peaks.get("bf16_tflops")
    return {
        "workload": cfg.label(), "samples": n, "dd": dd, "ms": ms, "samples_per_s": n / (ms / 1e3),
        "fp32_cuda_core_ms": ms32, "rows_equal_split_vs_fp32": same,
        "chain_gemm": {"kernel": "umma_tf32x3_kernel (3xTF32 tcgen05)", "bound": "tensor", "achieved": achieved,
                       "unit": "TFLOP/s", "peak": tf32 / 2 if tf32 else None,
                       "frac": achieved / (tf32 / 2) if tf32 else None,
                       "tensor_issue_frac": 3 * achieved / (tf32 / 2) if tf32 else None,
                       "ms": g["ms"] / 3, "peak_source": "TF32 dense = half the measured cuBLAS bf16 burst rate"},
        "sample_step_ms": prof["sample"]["ms"] / 3,
    }


def measure_batch(args, lib, handle, steps: int = 3, warmup: int = 1):
    """The 64-instance uneven workload (M ~ U{8..48}, d ~ U{4..8}, chi in
    {32..256}): one bsg_build_mps_batch call (one launch per phase, one DP
    launch set over every instance's items) against 64 bsg_build_mps calls
    back to back; CUDA events on the launching stream, one untimed run of
    each first."""
    import torch

    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps, build_mps_batch

    cfgs = synthetic.batch_configs(64)
    sqs = [torch.as_tensor(synthetic.lossy_covariances(c)[1]).cuda() for c in cfgs]
    ds, chis = [c.d for c in cfgs], [c.chi for c in cfgs]
    outs = [[torch.empty(c.chi, c.chi, c.d, dtype=torch.complex64, device="cuda") for _ in range(c.M)] for c in cfgs]
    stream = torch.cuda.current_stream()

    def batched():
        build_mps_batch(sqs, ds, chis, precision=args.precision, outs=outs)

    def looped():
        for c, q, o in zip(cfgs, sqs, outs):
            build_mps(q, c.d, c.chi, precision=args.precision, out=o)

    res = {}
    for name, fn in (("batched", batched), ("looped", looped)):
        for _ in range(max(1, warmup)):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(1, steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        res[name] = statistics.mean(ts)
    sites = sum(c.M for c in cfgs)
    # the DP launch knobs searched for this workload (autotune.tune_batch),
    # then the defaults restored for the rest of the line
    from bosonsupremacy_gb300 import autotune

    saved = autotune.get_knobs()
    try:
        best, table = autotune.tune_batch(sqs, ds, chis, precision=args.precision)
    finally:
        autotune.set_knobs(**saved)
    names = ("small_entries", "dp_quantum", "blocks_per_sm")
    return {"workload": "batch64: 64 instances, M~U{8..48}, d~U{4..8}, chi in {32,64,128,256}, r~U[0.5,1.4], "
                        "eta~U[0.2,0.6]", "instances": len(cfgs), "sites": sites,
            "batched_ms": res["batched"], "looped_ms": res["looped"],
            "batched_sites_per_s": sites / (res["batched"] / 1e3), "looped_sites_per_s": sites / (res["looped"] / 1e3),
            "speedup_vs_looped": res["looped"] / res["batched"],
            "tuned": {"knobs": best, "batched_ms": min(table.values()),
                      "speedup_vs_looped": res["looped"] / min(table.values()),
                      "grid_ms": {"/".join(f"{n}={v}" for n, v in zip(names, k)): round(t, 3)
                                  for k, t in table.items()}}}


def measure_decomposition(args):
    """The covariance decomposition (get_decomposition.py:16-29 SDP) on the
    GPU at M = args.decomp_M: a uniform-loss covariance of the medium
    workload's parameters, whose optimum is known in closed form (error
    reported), and a mode-dependent-loss covariance (loss between two
    interferometers), whose optimum is certified by the duality gap and by
    purity (every symplectic eigenvalue of X equal to 1).  Wall time of the
    whole solve (one warm-up solve at M=4 first), iterations and gap."""
    import dataclasses

    import numpy as np
    import torch

    from bosonsupremacy_gb300 import decomposition, synthetic

    M = args.decomp_M
    decomposition.decompose(synthetic.nonuniform_lossy_covariance(4, seed=1))
    cfg = dataclasses.replace(synthetic.MEDIUM, M=M)
    cov_u, sq_u = synthetic.lossy_covariances(cfg)
    cov_n = synthetic.nonuniform_lossy_covariance(M, seed=0)
    out = {"M": M, "schur_order": M * (2 * M + 1), "precision": "fp64"}
    for name, cov in (("uniform_loss", cov_u), ("mode_dependent_loss", cov_n)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, meta = decomposition.decompose(cov)
        ms = 1e3 * (time.perf_counter() - t0)
        Om = np.kron(np.array([[0.0, 1.0], [-1.0, 0.0]]), np.eye(M))
        nu = np.sort(np.abs(np.linalg.eigvals(1j * Om @ X).real))[::2]
        r = {"ms": ms, "iterations": meta["iterations"], "rel_gap": meta["rel_gap"],
             "primal_res": meta["primal_res"], "dual_res": meta["dual_res"], "trace": meta["primal_obj"],
             "max_symplectic_eig_dev": float(np.abs(nu - 1.0).max())}
        if name == "uniform_loss":
            r["rel_err_vs_closed_form"] = float(np.abs(X - sq_u).max() / np.abs(sq_u).max())
        out[name] = r
    if not args.no_cpu:
        # CPU leg: the oracle's interior-point restatement (numpy / LAPACK on
        # the host's cores) against the GPU solver on one mode-dependent-loss
        # covariance of a size the oracle solves in seconds
        from oracle import decomposition as oracle_decomposition
        Mc = args.decomp_cpu_M
        cov_c = synthetic.nonuniform_lossy_covariance(Mc, seed=1)
        t0 = time.perf_counter()
        ref = oracle_decomposition.decompose(cov_c)
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Xg, meta = decomposition.decompose(cov_c)
        gpu_ms = 1e3 * (time.perf_counter() - t0)
        out["cpu_baseline"] = {"M": Mc, "kind": "port", "cores": os.cpu_count(), "cpu_ms": cpu_ms,
                               "cpu_iterations": ref.iterations, "gpu_ms": gpu_ms, "gpu_iterations": meta["iterations"],
                               "max_abs_diff": float(np.abs(Xg - ref.X).max())}
    return out


def measure_largest(args, lib, handle):
    """The largest single-GPU workload (M=216 banded, d=10, chi=2048; 72 GB
    of complex64 Gamma): full-build time of the split build (CUDA events,
    one untimed build first), the plain-FP64 build's time, and per cut /
    site the error of the first 32: Lambda against the reference's FP64
    kron_cpu.py weights (tests/golden/largest_M216.npz) and Gamma of the
    split build against the FP64 build (max |difference| over the site's
    largest entry)."""
    import numpy as np
    import torch

    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps

    cfg = synthetic.LARGEST
    M, d, chi = cfg.M, cfg.d, cfg.chi
    _, sq = synthetic.lossy_covariances(cfg)
    fx = os.path.join(REPO, "tests", "golden", "largest_M216.npz")
    ref = np.load(fx) if os.path.exists(fx) else None
    if ref is not None:
        sq = ref["sq_cov"]
    sq_dev = torch.as_tensor(sq).cuda()
    stream = torch.cuda.current_stream()

    def timed(prec, out):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m = build_mps(sq_dev, d, chi, precision=prec, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), m

    split = [torch.empty(chi, chi, d, dtype=torch.complex64, device="cuda") for _ in range(M)]
    timed(args.precision, split)
    ms, m = timed(args.precision, split)
    n = 32
    lam_err, lam_err_hi = None, None
    if ref is not None:
        res = m.res.cpu().numpy()
        lam_err, lam_err_hi = [], []
        for c in range(n):
            k = int(ref["kept"][c])
            a = np.sort(res[c, :k])[::-1]
            b = ref["res"][c, :k]
            rel = np.abs(np.sqrt(a) - np.sqrt(b)) / np.sqrt(b)
            lam_err.append(float(rel[b > 1e-10].max()))
            lam_err_hi.append(float(rel[b > 1e-6].max()))
    # the FP64 build writes its first 32 sites to their own buffers and the
    # rest over the split build's (not compared)
    fp64 = [torch.empty(chi, chi, d, dtype=torch.complex64, device="cuda") for _ in range(n)] + split[n:]
    timed("fp64", fp64)  # untimed: the FP64 DP kernel loaded, as the split build was warmed above
    ms64, _ = timed("fp64", fp64)
    g_err = [float((split[i] - fp64[i]).abs().max().item() / fp64[i].abs().max().item()) for i in range(n)]
    out = {"workload": cfg.label(), "build_ms": ms, "sites_per_s": M / (ms / 1e3), "fp64_build_ms": ms64,
           "split_speedup": ms64 / ms,
           "lambda_rel_err_vs_reference_kron_first32": lam_err,
           "lambda_rel_err_vs_reference_kron_first32_weights_above_1e-6": lam_err_hi if lam_err else None,
           "lambda_source": "tests/golden/largest_M216.npz (kron_cpu.py FP64-promoted, cuts 0-31)" if lam_err else None,
           "gamma_err_split_vs_fp64_first32": g_err,
           "note": "Gamma errors: max |split - fp64| / max |fp64| per site, both complex64"}
    del split, fp64, m
    torch.cuda.empty_cache()
    return out


def run_reference(args, ws, rank):
    """The reference's own CPU MPS construction (oracle port of kron_cpu.py +
    MPS_cpu.py) on all the host's cores: each step runs one bounded timed
    sample per core at once and spreads the workload's cuts and sites over
    the cores (the reference's multi-process form gives each rank whole cuts
    and sites), extrapolated to the full build of the same workload."""
    if rank != 0:
        return
    import numpy as np

    from bosonsupremacy_gb300 import synthetic
    from oracle import cpu_baseline, reference_mps as R

    cfg = synthetic.NAMED[args.workload]
    _, sq = synthetic.lossy_covariances(cfg)
    # cut data for the group sizes (pruning to chi per step selects the same
    # top-chi set as the reference's max_dim = 1e5, at a fraction of the cost)
    cuts = [R.get_cumsum_kron(sq, c + 1, chi=cfg.chi, max_dim=cfg.chi, cutoff=cfg.d) for c in range(cfg.M - 1)]
    procs = max(1, len(os.sched_getaffinity(0)))
    vals = []
    est = None
    note = None
    step_s = []
    for i in range(args.warmup + args.steps):
        t_step = time.perf_counter()
        try:
            est = cpu_baseline.estimate_full_build_parallel(sq, cfg.d, cfg.chi, cuts, procs,
                                                            budget_s=args.cpu_budget / 2, seed=i,
                                                            timeout_s=max(120.0, 6.0 * args.cpu_budget))
        except Exception as e:  # a failed sample process: the one-core estimate instead
            note = f"parallel sample failed ({type(e).__name__}); one core"
            procs = 1
            est = cpu_baseline.estimate_full_build(sq, cfg.d, cfg.chi, cuts, budget_s=args.cpu_budget / 2, seed=i)
        if i >= args.warmup:
            vals.append(est["sites_per_s"])
            step_s.append(time.perf_counter() - t_step)
    v = statistics.median(vals)
    sample = (f"oracle (FP64 restatement of kron_cpu.py + MPS_cpu.py) on {procs} host cores, one process per "
              f"core: each timed one middle cut at max_dim=1e5, one williamson(sq_cov) + Bloch-Messiah and "
              f"~20 A_elem batches (n=6..12) fitted to the per-group cost model; the workload's cuts and "
              f"sites (exact (j, size) groups) spread over the cores longest first; value is the extrapolated "
              f"full build, ms_per_step the wall time of one step's timed sample")
    if note:
        sample = note + "; " + sample
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(step_s), "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None, "dtype": "c128/f64", "data": "synthetic",
        "config": {"workload": cfg.label(), "M": cfg.M, "d": cfg.d, "chi": cfg.chi},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample,
                         "extrapolated_build_s": est["build_s"], "extrapolated_ms_per_build": 1e3 * cfg.M / v,
                         "one_core_equivalent_s": est.get("serial_s", est["build_s"])},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import numpy as np
    import torch

    from bosonsupremacy_gb300 import _lib, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps, build_mps_host

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = _lib.load()
    handle = _lib.Handle.get(local)
    if args.workload == "batch64":
        # the 64 uneven instances alone: one line for the batched build
        clocks = ClockSampler(local)
        clocks.start()
        b = measure_batch(args, lib, handle, steps=args.steps, warmup=args.warmup)
        clk = clocks.stop()
        if rank == 0:
            print(json.dumps({
                "metric": "batched full-MPS build throughput (sites/s), 64 independent uneven instances",
                "value": b["batched_sites_per_s"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": b["batched_ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp32x2 (split) hafnian, f64 factorisations",
                "data": "synthetic (64 seeded lossy GBS covariances)",
                "config": {"workload": b["workload"], "precision": args.precision, "gamma_dtype": "complex64"},
                "clocks": clk, "batch64": b}), flush=True)
        return
    cfg = synthetic.NAMED[args.workload]
    _, sq = synthetic.lossy_covariances(cfg, seed=cfg.seed + rank)  # independent instance per rank
    sq_dev = torch.as_tensor(sq).to(dev)
    M, d, chi = cfg.M, cfg.d, cfg.chi
    outs = [torch.empty(chi, chi, d, dtype=torch.complex64, device=dev) for _ in range(M)]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        build_mps(sq_dev, d, chi, precision=args.precision, out=outs)
    torch.cuda.synchronize()
    lib.bsg_profile_reset(handle.h)
    lib.bsg_profile_enable(handle.h, 1)
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    stream = torch.cuda.current_stream()
    gc.collect()
    gc.disable()  # as timeit does: no collector pauses inside the timed steps
    try:
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between steps (outside the timed region)
            torch.cuda.synchronize()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            build_mps(sq_dev, d, chi, precision=args.precision, out=outs)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    finally:
        gc.enable()
    clk = clocks.stop()
    lib.bsg_profile_enable(handle.h, 0)
    prof = profile_read(lib, handle.h)
    host_prof = profile_read(lib, handle.h, host=True)
    ms = statistics.mean(times)
    if ws > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * M / (ms / 1e3)

    # end to end through the public host API
    e2e = None
    if not args.no_e2e:
        host_sq = torch.as_tensor(sq).pin_memory()
        host_out = [torch.empty(chi, chi, d, dtype=torch.complex64, pin_memory=True) for _ in range(M)]
        host_lam = torch.empty(M - 1, chi, dtype=torch.float64, pin_memory=True)
        # every pinned page touched twice before timing (first-touch / pinning costs stay outside)
        for _ in range(2):
            build_mps_host(host_sq, d, chi, host_out, host_lam, precision=args.precision, device_out=outs)
        torch.cuda.synchronize()
        link_before = link_probe(outs, host_out)
        et = []
        gc.collect()
        gc.disable()  # as timeit does: no collector pauses inside the timed steps
        try:
            for _ in range(args.steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                barrier()
                t0 = time.perf_counter()
                build_mps_host(host_sq, d, chi, host_out, host_lam, precision=args.precision, device_out=outs)
                torch.cuda.synchronize()
                et.append(time.perf_counter() - t0)
        finally:
            gc.enable()
        es = statistics.mean(et)
        if ws > 1:
            t = torch.tensor([es], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            es = float(t.item())
        link_after = link_probe(outs, host_out)
        d2h = int(sum(o.numel() * 8 for o in host_out) + host_lam.numel() * 8)
        e2e = {"value": ws * M / es, "unit": UNIT, "h2d_bytes_per_step": int(host_sq.numel() * 8),
               "d2h_bytes_per_step": d2h, "ms_per_step": es * 1e3,
               "step_ms": {"min": min(et) * 1e3, "median": statistics.median(et) * 1e3, "max": max(et) * 1e3,
                           "all": [round(x * 1e3, 2) for x in et]},
               "link_d2h_gbs": {"before": link_before, "after": link_after,
                                "note": "bare device-to-host copy of the same Gamma bytes into the same pinned "
                                        "buffers (one cudaMemcpyAsync per site), timed just before and after the "
                                        "e2e steps; the e2e floor is max(build, bytes / link rate)"},
               "pinned": "torch pin_memory buffers, one per site, touched by two untimed e2e builds"}

    # plain-FP64 path of the same kernels: one untimed build (its first DP
    # launch loads the FP64 kernel), then warm builds timed like the split ones
    fp64 = None
    if not args.no_fp64 and args.precision != "fp64":
        build_mps(sq_dev, d, chi, precision="fp64", out=outs)
        t64s = []
        for _ in range(2):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            build_mps(sq_dev, d, chi, precision="fp64", out=outs)
            e1.record(stream)
            torch.cuda.synchronize()
            t64s.append(e0.elapsed_time(e1))
        t64 = statistics.mean(t64s)
        fp64 = {"build_ms": t64, "sites_per_s": M / (t64 / 1e3), "split_speedup": t64 / ms,
                "note": "mean of 2 warm builds after one untimed build, L2 flushed before each"}
        build_mps(sq_dev, d, chi, precision=args.precision, out=outs)  # restore outputs

    # first build on a fresh handle: partition programs generated, scratch
    # allocated and every table uploaded inside the timed region
    cold = None
    if rank == 0:
        fresh = _lib.Handle(local)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        build_mps(sq_dev, d, chi, precision=args.precision, out=outs, handle=fresh)
        torch.cuda.synchronize()
        cold = {"ms": (time.perf_counter() - t0) * 1e3,
                "note": "one build on a new library handle (empty program cache, no scratch yet), host clock"}
        fresh.close()
        del fresh
        build_mps(sq_dev, d, chi, precision=args.precision, out=outs)

    # roofline of the hafnian DP (the dominant kernel by SM-time: it is
    # ~15k of the ~19k SM-milliseconds of a build; the Williamson / Sigma
    # kernels run one CTA per cut or site on streams that overlap it).  Live
    # CUDA-event timing of every DP launch on its own stream; launches that
    # share the GPU with other groups' kernels are timed as they ran.
    dom = "hafnian_dp"
    peaks = measured_peaks()
    pk64, pk32 = C.c_double(), C.c_double()
    _lib.check(lib.bsg_fma_peak(handle.h, _lib.PREC_FP64, C.byref(pk64), None), "bsg_fma_peak")
    _lib.check(lib.bsg_fma_peak(handle.h, _lib.PREC_FP32, C.byref(pk32), None), "bsg_fma_peak")
    dp_s = prof[dom]["ms"] / 1e3
    achieved = 8.0 * prof[dom]["work"] / dp_s  # 8 real flops per complex multiply-add
    if args.precision == "fp64":
        roof = {"kernel": "dp_kernel<PrecF64> (hafnian DP)", "bound": "fp64-pipe", "achieved": achieved / 1e12,
                "peak": pk64.value / 1e12, "unit": "TFLOP/s", "frac": achieved / pk64.value, "traffic": None}
    else:
        # FP32 operations per complex multiply-add (split: four products of
        # hi/lo pairs, 12 operations each, issued as 24 packed f32x2
        # instructions; plain FP32: 4 FMAs)
        ops = {"split": 48.0, "fp32": 4.0}[args.precision]
        # The arithmetic's own ceiling: the FP32 pipe runs one operation per
        # lane and cycle (half its FMA flop peak), and a complex multiply-add
        # (8 algorithmic flops) costs `ops` of them, so the most this
        # arithmetic can deliver is 8 * (pk32 / 2) / ops algorithmic flop/s.
        ceiling = 8.0 * (pk32.value / 2.0) / ops
        roof = {"kernel": f"dp_kernel<Prec{'Split' if args.precision == 'split' else 'F32'}> (hafnian DP)",
                "bound": "fp32-pipe", "achieved": achieved / 1e12, "peak": pk32.value / 1e12, "unit": "TFLOP/s",
                "frac": achieved / pk32.value, "traffic": (DP_DRAM_BYTES_PER_CMAC * prof[dom]["work"] / max(1, prof[dom]["launches"])
                            if DP_DRAM_BYTES_PER_CMAC else None),
                "fp32_op_busy_frac": achieved / ceiling,
                "fp64_equivalent_frac": achieved / pk64.value,
                "note": ("achieved = 8 algorithmic flops per complex multiply-add of the partition programs over the "
                         "live (CUDA-event) DP launch durations, which overlap the factorisations' kernels; peak = "
                         "the FP32 FMA flop rate measured on this GPU by bsg_fma_peak (MEASURED_PEAKS.json has no "
                         "CUDA-core peak); "
                         f"{'the split arithmetic spends 48 FP32 operations (24 packed f32x2 instructions)' if args.precision == 'split' else 'FP32 arithmetic spends 4 FMAs'} "
                         "per complex multiply-add, so fp32_op_busy_frac = achieved / (8 x half the FMA flop peak / "
                         "those operations) is the FP32 pipe's busy fraction; fp64_equivalent_frac compares the "
                         "FP64-accurate result rate with the FP64 pipe's measured peak; traffic = DRAM bytes per "
                         "DP launch: 2.28 bytes per complex multiply-add measured by ncu on the M=50 build's DP "
                         "launches, times this workload's multiply-adds per launch "
                         "(profiles/dp_kernel_traffic_M50_d6_chi256.md)")}
    roof["peak_source"] = "FMA peak measured on this GPU by bsg_fma_peak (register FMA loop on every SM)"
    roof["launch_ms_mean"] = prof[dom]["ms"] / max(1, prof[dom]["launches"])
    roof["work"] = ("8 flops per complex multiply-add of the repetition-aware partition programs "
                    f"({prof[dom]['work'] / args.steps:.4g} per build)")
    roof["launches_per_build"] = prof[dom]["launches"] / args.steps
    roof["ms_per_build_summed"] = prof[dom]["ms"] / args.steps
    roof["hbm_peak_gbs_measured"] = peaks.get("hbm_gbs")
    launches = int(sum(v["launches"] for v in prof.values()))

    contraction = None
    if rank == 0 and not args.no_contract:
        contraction = measure_contraction(args, lib, handle, peaks)
    sampler = None
    if rank == 0 and not args.no_sampler:
        sampler = measure_sampler(args, lib, handle, peaks)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import cpu_baseline

        mps = build_mps(sq_dev, d, chi, precision=args.precision, out=outs)
        kept = mps.kept
        rs, nm, Ss = mps.res.cpu().numpy(), mps.num.cpu().numpy(), mps.S.cpu().numpy()
        cuts = []
        for c in range(M - 1):
            k = M - 1 - c
            cuts.append((rs[c, : kept[c]], nm[c, : kept[c], :k], Ss[c, : 2 * k, : 2 * k]))
        est = cpu_baseline.estimate_full_build(np.asarray(sq), d, chi, cuts, budget_s=args.cpu_budget)
        cpu = {"value": est["sites_per_s"], "unit": UNIT, "cores": 1, "kind": "port",
               "sample": (f"oracle FP64 restatement of kron_cpu.py + MPS_cpu.py on this host: one middle cut at "
                          f"max_dim=1e5, one williamson(sq_cov) + Bloch-Messiah, ~20 timed A_elem batches fitted "
                          f"to a per-group cost model, applied to the workload's {est['groups']} (j, size) groups "
                          f"({est['items']} items); extrapolated full build {est['build_s']:.0f} s"),
               "extrapolated_build_s": est["build_s"]}

    batch = None
    if rank == 0 and not args.no_batch:
        batch = measure_batch(args, lib, handle)

    decomp = None
    if rank == 0 and not args.no_decomp:
        decomp = measure_decomposition(args)

    largest = None
    if rank == 0 and not args.no_largest:
        del outs
        torch.cuda.empty_cache()
        largest = measure_largest(args, lib, handle)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"split": "fp32x2 (split) hafnian, f64 factorisations",
                                           "fp64": "f64", "fp32": "f32 hafnian, f64 factorisations"}[args.precision],
            "data": "synthetic (seeded lossy GBS covariance; independent instance per rank)",
            "config": {"workload": cfg.label(), "M": M, "d": d, "chi": chi, "precision": args.precision,
                       "gamma_dtype": "complex64", "l2": "flushed between steps (512 MiB write)"},
            "step_ms_all": [round(t, 2) for t in times], "clocks": clk, "gpu_launches": launches, "kernels": {k: {"ms": v["ms"], "launches": v["launches"]}
                                                                 for k, v in prof.items()},
            "host": {k: {"ms": v["ms"], "calls": v["launches"]} for k, v in host_prof.items()},
            "roofline": roof, "fp64_path": fp64, "cold_build": cold, "e2e": e2e, "cpu_baseline": cpu, "contraction": contraction, "sampler": sampler,
            "batch64": batch, "largest": largest, "decomposition": decomp,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
