#!/usr/bin/env python
"""Mattes MI value+derivative throughput on GB300.

Workload (one step = one GetValueAndDerivative of the full-resolution level):
MattesMutualInformationImageToImageMetricv4, 50 histogram bins, affine moving
transform, 256x256x200 float32 blob volumes (moving = fixed under a seeded
affine with the multimodal intensity map), 20 % random sampling
(2,621,440 points), gradient image supplied.  Synthetic seeded inputs stand
in for real volumes.  `--transform bspline` measures the B-spline workload
instead: [affine, BSplineTransform order 3 over an 8x8x8 mesh (11^3 nodes,
3993 parameters)], 192x192x160 volumes whose moving image carries a seeded
smooth displacement (at most 4 mm), 10 % random sampling.

Prints one JSON line.  `value` is device-timed throughput with everything
resident in HBM (CUDA events around each evaluation, L2 flushed between
steps); `e2e` is the same metric through the public call (host parameters in,
value and derivative back to the host each step).  `--impl reference` times
the FP64 CPU port of the reference algorithm (oracle/) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mattes-MI value+deriv Msamples/s"
UNIT = "Msamples/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--transform", default="affine", choices=["affine", "bspline"],
                    help="affine: 256x256x200, 20%% sampling; bspline: [affine, B-spline 8x8x8 mesh], "
                         "192x192x160, 10%% sampling")
    ap.add_argument("--size", default=None)
    ap.add_argument("--fraction", type=float, default=None)
    ap.add_argument("--mesh", type=int, default=8)
    ap.add_argument("--bins", type=int, default=50)
    ap.add_argument("--metric", default="mattes", choices=["mattes", "msq"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    bs = args.transform == "bspline"
    if args.size is None:
        args.size = "192,192,160" if bs else "256,256,200"
    if args.fraction is None:
        args.fraction = 0.1 if bs else 0.2
    return args


def workload(args):
    """The seeded inputs, cached (pickle) under .bench_cache/ in the repository: profiler runs
    re-run the same command."""
    import pickle
    key = f"{args.transform}_{args.metric}_{args.size.replace(',', 'x')}_{args.fraction}_{args.mesh}"
    cache_dir = os.path.join(ROOT, ".bench_cache")
    os.makedirs(cache_dir, exist_ok=True)
    path = os.path.join(cache_dir, f"{key}.pkl")
    if os.path.exists(path):
        try:
            with open(path, "rb") as f:
                return pickle.load(f)
        except Exception:
            pass
    w = make_workload(args)
    tmp = f"{path}.{os.getpid()}"
    with open(tmp, "wb") as f:
        pickle.dump(w, f, protocol=pickle.HIGHEST_PROTOCOL)
    os.replace(tmp, path)
    return w


def make_workload(args):
    from itk_gb300 import BSplineTransform, CompositeTransform, data
    size = tuple(int(s) for s in args.size.split(","))
    if args.transform == "bspline":
        # [affine, B-spline] initialised from the generating affine; the B-spline part mid-optimization
        fixed, moving, A, B = data.pair_bspline(size, (args.mesh,) * 3, instance=0,
                                                multimodal_map=(args.metric == "mattes"))
        grad = data.gradient_image(moving)
        pts = data.random_points(fixed, args.fraction, seed=2001)
        Bm = BSplineTransform()
        Bm.SetFixedParameters(B.GetFixedParameters())
        Bm.SetParameters(0.5 * B.GetParameters())
        U = CompositeTransform()
        U.AddTransform(A)
        U.AddTransform(Bm)
        return fixed, moving, grad, pts, U
    fixed, moving, T = data.pair_affine(size, config=1, multimodal_map=(args.metric == "mattes"))
    grad = data.gradient_image(moving)
    pts = data.random_points(fixed, args.fraction, seed=1001)
    # evaluate at a transform near (not at) the truth, as mid-optimization
    rng = np.random.default_rng(77)
    U = type(T)()
    U.SetCenter(T.GetCenter())
    U.SetMatrix(T.GetMatrix() + rng.uniform(-0.01, 0.01, size=(3, 3)))
    U.SetTranslation(T.GetTranslation() + rng.uniform(-1.0, 1.0, size=3))
    return fixed, moving, grad, pts, U


def config_dict(args, n_samples):
    size = [int(s) for s in args.size.split(",")]
    bs = args.transform == "bspline"
    tname = f"bspline{args.mesh}" if bs else "affine"
    return {
        "workload": f"{args.metric}_{tname}_{'x'.join(map(str, size))}_{int(args.fraction * 100)}pct_{args.bins}bins",
        "volume_xyz": size,
        "samples": int(n_samples),
        "bins": args.bins if args.metric == "mattes" else None,
        "sampling": f"random {args.fraction:.0%} (virtual sampled point set)",
        "transform": (f"CompositeTransform [AffineTransform, BSplineTransform order 3, mesh {args.mesh}^3 "
                      f"({(args.mesh + 3) ** 3} nodes, {3 * (args.mesh + 3) ** 3} parameters)]")
                     if bs else "AffineTransform<double,3>",
        "gradient": "moving gradient image (packed with the moving image)",
        "level": "full resolution (shrink 1, sigma 0)",
        "l2": "flushed between timed steps (256 MiB memset); inputs larger than L2",
    }


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy)"
    return 6800.0, "fallback 6.8 TB/s"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(args, fixed, moving, grad, pts, U, seconds):
    """The FP64 CPU port of the reference path (oracle), all host threads, bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cases import run_oracle
    threads = os.cpu_count() or 1
    kind = "mattes" if args.metric == "mattes" else "msq"
    t0 = time.perf_counter()
    run_oracle(kind, fixed, moving, U, gradient=grad, points=pts, bins=args.bins, nthreads=threads)
    one = time.perf_counter() - t0
    reps = int(max(1, min(20, seconds // max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        run_oracle(kind, fixed, moving, U, gradient=grad, points=pts, bins=args.bins, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": len(pts) * reps / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} full evaluations of the bench workload ({len(pts)} samples each), "
                      f"{dt:.1f} s, FP64 oracle (oracle/itk_oracle.c), {threads} threads"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_GLOO") is None else "gloo")
    return world, rank, local, dist


def run_reference(args):
    world, rank, local, dist = dist_setup()
    if rank != 0:
        return
    fixed, moving, grad, pts, U = workload(args)
    per = cpu_baseline(args, fixed, moving, grad, pts, U, args.cpu_seconds)
    # steps of the reference arm: a bounded number of full evaluations
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cases import run_oracle
    kind = "mattes" if args.metric == "mattes" else "msq"
    threads = os.cpu_count() or 1
    for _ in range(min(args.warmup, 3)):
        run_oracle(kind, fixed, moving, U, gradient=grad, points=pts, bins=args.bins, nthreads=threads)
    steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(steps):
        run_oracle(kind, fixed, moving, U, gradient=grad, points=pts, bins=args.bins, nthreads=threads)
    dt = time.perf_counter() - t0
    value = len(pts) * steps / dt / 1e6
    per["value"] = value
    per["sample"] = f"{steps} full evaluations ({len(pts)} samples each) after {min(args.warmup, 3)} warm-up, " \
                    f"FP64 oracle port of the reference algorithm, {threads} threads"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": min(args.warmup, 3), "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, len(pts)), "impl": "reference", "cpu_baseline": per,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    world, rank, local, dist = dist_setup()
    import torch

    from itk_gb300 import (MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4, context,
                           roofline)
    torch.cuda.set_device(local)
    context(local)
    fixed, moving, grad, pts, U = workload(args)
    cls = MattesMutualInformationImageToImageMetricv4 if args.metric == "mattes" else MeanSquaresImageToImageMetricv4
    m = cls(device=local)
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(U)
    m.SetMovingImageGradientImage(grad)
    if args.metric == "mattes":
        m.SetNumberOfHistogramBins(args.bins)
    m.SetVirtualSampledPointSet(pts)
    m.SetUseSampledPointSet(True)
    t_init = time.perf_counter()
    m.Initialize()
    init_s = time.perf_counter() - t_init
    n = m.GetNumberOfDomainPoints()
    P = U.GetNumberOfParameters()
    ext = torch.cuda.ExternalStream(m.stream(), device=local)
    d_params = torch.tensor(U.GetParameters(), dtype=torch.float64, device=f"cuda:{local}")
    d_out = torch.zeros(2 + P, dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    bs = args.transform == "bspline"

    def one_step(with_events):
        with torch.cuda.stream(ext):
            flush.zero_()
            if with_events:
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(ext)
                m.evaluate_device(d_params.data_ptr(), d_out.data_ptr(), True)
                e.record(ext)
                return s, e
            m.evaluate_device(d_params.data_ptr(), d_out.data_ptr(), True)
            return None

    for _ in range(args.warmup):
        one_step(False)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    events = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            events.append(one_step(True))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        dev_ms = sum(s.elapsed_time(e) for s, e in events)
        status = m.synchronize()
        # end-to-end through the public call: params host->device, value+derivative device->host
        for _ in range(args.warmup):
            m.GetValueAndDerivative()
        e2e_t = 0.0
        for _ in range(args.steps):
            with torch.cuda.stream(ext):
                flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            m.GetValueAndDerivative()
            e2e_t += time.perf_counter() - t1
    clocks = clk.summary()
    if status != 0:
        raise RuntimeError(f"evaluation status {status}")
    if dist:
        t = torch.tensor([dev_ms, e2e_t], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms, e2e_t = float(t[0]), float(t[1])
    if rank != 0:
        return
    value = world * n * args.steps / (dev_ms / 1e3) / 1e6
    e2e_value = world * n * args.steps / e2e_t / 1e6

    # roofline of the dominant kernel: per-kernel CUDA-event times on the launching stream
    m.set_profiling(True)
    ktimes = []
    for _ in range(10):
        with torch.cuda.stream(ext):
            flush.zero_()
        m.evaluate_device(d_params.data_ptr(), d_out.data_ptr(), True)
        ktimes.append(m.kernel_times_ms())
    m.set_profiling(False)
    ktimes = np.mean(np.array(ktimes), axis=0)
    # the affine path's constant kernel runs before the first profiling mark
    kernels_per_eval = len(ktimes) + (0 if bs else 1)
    v_touched = roofline.touched_voxels(pts, U, moving)
    nodes = (args.mesh + 3) ** 3
    if bs:
        # kernel order of the device-resident call: nodes, pass 1 (or MeanSquares), chunks, params
        kidx = 1
        if args.metric == "mattes":
            kbytes = roofline.mattes_pass1_bspline_bytes(n, v_touched, nodes)
            kname = "k_mattes_pass1_bspline"
        else:
            kbytes = roofline.msq_bspline_bytes(n, v_touched, nodes)
            kname = "k_msq_bspline"
    else:
        kidx = 0
        if args.metric == "mattes":
            kbytes = roofline.mattes_pass1_bytes(n, v_touched)
            kname = "k_mattes_pass1_affine"
        else:
            kbytes = roofline.msq_bytes(n, v_touched)
            kname = "k_msq_affine"
    ktime = float(ktimes[kidx])
    peak, peak_src = measured_peak()
    achieved = kbytes / (ktime / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.txt")
    default_size = "192,192,160" if bs else "256,256,200"
    default_fraction = 0.1 if bs else 0.2
    if os.path.exists(tf) and args.size == default_size and abs(args.fraction - default_fraction) < 1e-9:
        for line in open(tf):
            parts = line.split()
            if len(parts) == 2 and parts[0] == kname:
                traffic = int(parts[1])
    b_alg = roofline.evaluation_bytes(n, v_touched, nparams=P)
    eval_ms = dev_ms / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": eval_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args, n),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": int(kbytes), "kernel_ms": ktime,
                     "kernel_ms_all": [float(x) for x in ktimes],
                     "evaluation": {"b_alg_bytes": int(b_alg), "v_touched": v_touched,
                                    "achieved_gbs": b_alg / (eval_ms / 1e3) / 1e9,
                                    "frac": b_alg / (eval_ms / 1e3) / 1e9 / peak}},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * P,
                "d2h_bytes_per_step": 8 * (2 + P) + 4,
                "note": "public GetValueAndDerivative call: parameters in, value/derivative/status out; "
                        "images and samples resident in HBM since Initialize"},
        "gpu_launches": kernels_per_eval * args.steps,
        "clocks": clocks,
        "wall_s_timed_loop": wall,
        "initialize_s": init_s,
    }
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(args, fixed, moving, grad, pts, U, args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
