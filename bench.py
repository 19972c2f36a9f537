#!/usr/bin/env python3
"""Benchmark of the fused image pipeline on one GB300.

Workload (the uniform-batch configuration): 256 float32 RGB images of
1024x1024, values U[0,1) from a seed, Pipeline
    rgb2grey -> gaussian(sigma=3, radius 9) -> rotate(17 deg, bilinear) -> adjust_gamma(0.8)
One step = one pass of the pipeline over the whole batch.

Reported (one JSON line on stdout):
  value        whole-batch Mpix/s of the fused path, inputs resident in HBM,
               CUDA-graph replay of the plan (2 kernel launches per chunk of
               images), CUDA events on the launching stream.  The inputs
               (3.2 GB) exceed L2, so no flush is needed between steps.
  per_op       Mpix/s of the plain per-op path (one kernel per stage and image,
               a fresh pool buffer per stage), same inputs.
  e2e          Mpix/s through the C-ABI host-buffer entry
               (mpk_pipeline_run_host) from page-locked host memory: H2D of
               every input, the kernels, D2H of every output inside the timed
               region.
  roofline     the dominant kernel's algorithmic bytes per launch over its
               average CUDA-event duration, against the measured HBM copy
               bandwidth (MEASURED_PEAKS.json).
  cpu_baseline the FP64 oracle on the host cores for a bounded sample.

`--impl reference` times the reference's CPU implementation of the path --
the oracle port (the reference has no CPU path of its own and its HIP
kernels cannot run here) -- with every host core, on a bounded sample.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mpr
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_IMG, H, W, CH = 256, 1024, 1024, 3
N_IMG_DEFAULT = N_IMG
SIGMA, ANGLE, GAMMA = 3.0, 17.0, 0.8
SEED = 20260303
METRIC = "Mpix/s fused pipeline fwd (grey->gaussian s3->rotate 17->gamma 0.8), 256x1024x1024x3 f32"
CONFIG = {"workload": "uniform batch: 256 x 1024x1024x3 float32 RGB, rgb2grey -> gaussian sigma=3 "
                      "(radius 9) -> rotate 17 deg bilinear -> adjust_gamma 0.8",
          "images": N_IMG, "height": H, "width": W, "channels": CH,
          "l2": "inputs (3.2 GB) larger than L2 (129 MB); no flush between steps"}
ORACLE_OPS = [("rgb2grey",), ("gaussian", SIGMA), ("rotate", ANGLE), ("adjust_gamma", GAMMA)]
CPU_SAMPLE = 64          # images of the workload the cpu_baseline leg times (one bounded sample)
REF_SAMPLE = 16          # images per step of the reference arm (--impl reference)


# ----------------------------------------------------------------- CPU legs
def _cpu_one(seed_i):
    import numpy as np
    from oracle import oracle as O
    rng = np.random.default_rng(seed_i)
    x = rng.random((H, W, CH), dtype=np.float32)
    t = time.perf_counter()
    O.run_ops(x, ORACLE_OPS)
    return time.perf_counter() - t


def cpu_rate(n_images, workers):
    """Mpix/s of the FP64 oracle over n_images, `workers` processes (spawn)."""
    ctx = mpr.get_context("spawn")
    with ctx.Pool(workers) as pool:
        pool.map(_cpu_one, [0] * workers)                  # warm the workers
        t0 = time.perf_counter()
        pool.map(_cpu_one, list(range(1, n_images + 1)))
        dt = time.perf_counter() - t0
    return n_images * H * W / dt / 1e6, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    workers = min(cores, REF_SAMPLE)
    for _ in range(args.warmup):
        cpu_rate(REF_SAMPLE, workers)
    vals, secs = [], []
    for _ in range(args.steps):
        v, dt = cpu_rate(REF_SAMPLE, workers)
        vals.append(v)
        secs.append(dt)
    v = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "Mpix/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * N_IMG * H * W / (v * 1e6), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG,
            "cpu_baseline": {"value": round(v, 3), "unit": "Mpix/s", "cores": workers, "kind": "port",
                             "sample": "%d of the 256 images per step, one process per image "
                                       "(spawn pool of %d), FP64 numpy oracle" % (REF_SAMPLE, workers)},
            "e2e": {"value": round(v, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU legs
class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        # raw samples: $MP_BENCH_CLOCKS_CSV if set, else a per-process temp file
        self.path = os.environ.get("MP_BENCH_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), "mp_bench_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in open(self.path):
            p = [q.strip() for q in row.split(",")]
            if len(p) < 9 or not p[1].isdigit():
                continue
            sm.append(int(p[1]))
            mx = int(p[2])
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic_per_px(kind):
    """DRAM bytes per output pixel measured by ncu for a kernel kind, from the
    committed profile summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(str(kind))
    except (OSError, ValueError):
        return None


def run_ours(args):
    import numpy as np
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from millipyde_gb300 import _abi
    from oracle import oracle as O

    if args.gpus != 1 or int(os.environ.get("WORLD_SIZE", "1")) != 1:
        raise SystemExit("bench.py: this build measures one GPU (replicas only); run with --gpus 1")
    L = _abi.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)

    pitch_in, pitch_out = W * CH * 4, W * 4
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    with torch.cuda.stream(stream):
        x = torch.rand((N_IMG, H, W * CH), device=dev, dtype=torch.float32, generator=gen)
        y = torch.empty((N_IMG, H, W), device=dev, dtype=torch.float32)
    stream.synchronize()
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", SIGMA), _abi.stage("rotate", ANGLE),
                     _abi.stage("adjust_gamma", GAMMA, 1.0))
    ins = _abi.images([_abi.image(x[i].data_ptr(), H, W, CH, pitch_in) for i in range(N_IMG)])
    outs = _abi.images([_abi.image(y[i].data_ptr(), H, W, 1, pitch_out) for i in range(N_IMG)])
    mpix = N_IMG * H * W / 1e6

    # ---- fused plan, captured in a CUDA graph
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(st, 4, ins, outs, N_IMG, 0, 0, sp, C.byref(plan)))
    nlaunch = L.mpk_plan_num_launches(plan)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(max(3, args.warmup)):
        graph.replay()
    torch.cuda.synchronize()
    clocks = Clocks()
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            graph.replay()
        e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = mpix / (ms / 1e3)

    # correctness spot check of the timed outputs against the FP64 oracle
    xs = x[0].view(H, W, CH).cpu().numpy()
    err = float(np.max(np.abs(y[0].cpu().numpy().astype(np.float64) - O.run_ops(xs, ORACLE_OPS))))
    if not err <= 1e-5:
        raise SystemExit("bench.py: fused output differs from the oracle by %.3g" % err)

    # ---- per-launch timing (events around every launch of the plan)
    per_kind = {}
    for rep in range(2):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(nlaunch + 1)]
        with torch.cuda.stream(stream):
            evs[0].record(stream)
            for i in range(nlaunch):
                _abi.check(L.mpk_plan_launch_range(plan, i, 1, sp))
                evs[i + 1].record(stream)
        evs[-1].synchronize()
        if rep == 0:
            continue
        for i in range(nlaunch):
            kind, nj, tiles, byt = C.c_int(), C.c_int(), C.c_int(), C.c_double()
            L.mpk_plan_launch_info(plan, i, C.byref(kind), C.byref(nj), C.byref(tiles), C.byref(byt))
            d = per_kind.setdefault(kind.value, {"ms": 0.0, "launches": 0, "bytes": 0.0, "px": 0.0})
            d["ms"] += evs[i].elapsed_time(evs[i + 1])
            d["launches"] += 1
            d["bytes"] += byt.value
            d["px"] += nj.value * H * W
    dom = max(per_kind, key=lambda k: per_kind[k]["ms"])
    dk = per_kind[dom]
    avg_ms = dk["ms"] / dk["launches"]
    bytes_per_launch = dk["bytes"] / dk["launches"]
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    tpp = ncu_traffic_per_px(dom)
    traffic = tpp * dk["px"] / dk["launches"] if tpp else None
    kind_names = {0: "pointwise", 1: "gaussian tiles", 2: "rotate tiles", 3: "transpose",
                  4: "gaussian strip stream", 5: "rotate footprint (gamma epilogue)",
                  8: "gaussian 1-channel stream (rgb2grey prologue)"}

    per_op = e2e = cpu_v = None
    po_steps = e2e_steps = 0
    cpu_dt = 0.0
    workers = 0
    if args.legs == "all":
        # ---- plain per-op path on the same inputs
        po_steps = max(1, min(3, args.steps))
        with torch.cuda.stream(stream):
            _abi.check(L.mpk_pipeline_run_unfused(st, 4, ins, outs, N_IMG, 0, 0, sp))
        stream.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(po_steps):
                _abi.check(L.mpk_pipeline_run_unfused(st, 4, ins, outs, N_IMG, 0, 0, sp))
            e1.record(stream)
        e1.synchronize()
        per_op = mpix / (e0.elapsed_time(e1) / po_steps / 1e3)

        # ---- end to end from page-locked host buffers through the C-ABI
        hx = torch.empty((N_IMG, H, W * CH), dtype=torch.float32, pin_memory=True)
        hy = torch.empty((N_IMG, H, W), dtype=torch.float32, pin_memory=True)
        hx.copy_(x.cpu())
        hins = _abi.images([_abi.image(hx[i].data_ptr(), H, W, CH, pitch_in) for i in range(N_IMG)])
        houts = _abi.images([_abi.image(hy[i].data_ptr(), H, W, 1, pitch_out) for i in range(N_IMG)])
        _abi.check(L.mpk_pipeline_run_host(st, 4, hins, houts, N_IMG, 0, 0, sp))
        e2e_steps = max(1, min(3, args.steps))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            _abi.check(L.mpk_pipeline_run_host(st, 4, hins, houts, N_IMG, 0, 0, sp))
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        d = float((hy[0] - y[0].cpu()).abs().max())
        if not d <= 1e-6:
            raise SystemExit("bench.py: host-buffer path differs from the device path by %.3g" % d)
        e2e = mpix / e2e_s


        # ---- CPU baseline (FP64 oracle, bounded sample)
        cores = os.cpu_count() or 1
        workers = min(cores, CPU_SAMPLE)
        cpu_v, cpu_dt = cpu_rate(CPU_SAMPLE, workers)

    L.mpk_plan_destroy(plan)
    torch.cuda.synchronize()

    line = {"metric": METRIC, "value": round(value, 1), "unit": "Mpix/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": CONFIG,
            "per_op": None if per_op is None else
                      {"value": round(per_op, 1), "unit": "Mpix/s", "steps": po_steps,
                       "fused_over_per_op": round(value / per_op, 2)},
            "pipeline_hbm": {"algorithmic_bytes_per_step": N_IMG * H * W * 16,
                             "achieved_gbs": round(N_IMG * H * W * 16 / (ms / 1e3) / 1e9, 1),
                             "frac": round(N_IMG * H * W * 16 / (ms / 1e3) / 1e9 / peak, 4)},
            "roofline": {"bound": "hbm", "kernel": kind_names.get(dom, str(dom)),
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "bytes_per_launch": bytes_per_launch, "avg_launch_ms": round(avg_ms, 4),
                         "traffic": traffic,
                         "per_kind_ms": {kind_names.get(k, str(k)): round(v["ms"], 4) for k, v in per_kind.items()}},
            "e2e": None if e2e is None else
                   {"value": round(e2e, 1), "unit": "Mpix/s", "h2d_bytes_per_step": N_IMG * H * pitch_in,
                    "d2h_bytes_per_step": N_IMG * H * pitch_out, "steps": e2e_steps,
                    "path": "mpk_pipeline_run_host, page-locked host buffers"},
            "cpu_baseline": None if cpu_v is None else
                            {"value": round(cpu_v, 3), "unit": "Mpix/s", "cores": workers, "kind": "port",
                             "sample": "%d images of the workload, FP64 numpy oracle, spawn pool of %d "
                                       "(%.1f s)" % (CPU_SAMPLE, workers, cpu_dt)},
            "clocks": clk, "gpu_launches": args.steps * nlaunch,
            "max_abs_err_vs_oracle": err}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- other workloads
def _ragged_sizes(n, seed):
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    lo, hi = math.log(64), math.log(2048)
    return [(int(round(math.exp(rng.uniform(lo, hi)))), int(round(math.exp(rng.uniform(lo, hi)))))
            for _ in range(n)]


def run_ragged(args):
    """1000 RGB images, H and W log-uniform in [64, 2048]; per image rotate
    U(-45,45), gaussian sigma U(0.5,4), gamma U(0.5,2), brightness U(-0.2,0.2),
    fliplr p=0.5 (seeded counter RNG); one fused plan over the ragged batch."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from millipyde_gb300 import _abi
    L = _abi.lib()
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    n = args.images if args.images != N_IMG_DEFAULT else 1000
    sizes = _ragged_sizes(n, SEED)
    px = sum(h * w for h, w in sizes)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    keep, ins, outs = [], [], []
    with torch.cuda.stream(stream):
        for h, w in sizes:
            pitch = (w * 3 * 4 + 15) // 16 * 16
            t = torch.rand((h, pitch // 4), device=dev, generator=gen)
            o = torch.empty((h, pitch // 4), device=dev)
            keep += [t, o]
            ins.append(_abi.image(t.data_ptr(), h, w, 3, pitch))
            outs.append(_abi.image(o.data_ptr(), h, w, 3, pitch))
    stream.synchronize()
    st = _abi.stages(_abi.stage("rotate", random=True, lo=(-45,), hi=(45,)),
                     _abi.stage("gaussian", random=True, lo=(0.5,), hi=(4.0,)),
                     _abi.stage("adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
                     _abi.stage("brightness", random=True, lo=(-0.2,), hi=(0.2,)),
                     _abi.stage("fliplr", probability=0.5))
    ia, oa = _abi.images(ins), _abi.images(outs)
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(st, 5, ia, oa, n, SEED, 0, sp, C.byref(plan)))
    nl = L.mpk_plan_num_launches(plan)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(max(3, args.warmup)):
        g.replay()
    clocks = Clocks()
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            g.replay()
        e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    with torch.cuda.stream(stream):
        e0.record(stream)
        _abi.check(L.mpk_pipeline_run_unfused(st, 5, ia, oa, n, SEED, 0, sp))
        e1.record(stream)
    e1.synchronize()
    po_ms = e0.elapsed_time(e1)
    L.mpk_plan_destroy(plan)
    peak, pk = measured_peaks()
    gbs = px * 24 / (ms / 1e3) / 1e9
    print(json.dumps({"metric": "Mpix/s fused ragged augmentation fwd", "value": round(px / 1e6 / (ms / 1e3), 1),
                      "unit": "Mpix/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "ragged: %d RGB images, H,W log-uniform [64,2048], rotate U(-45,45) "
                                             "-> gaussian U(0.5,4) -> gamma U(0.5,2) -> brightness U(-0.2,0.2) "
                                             "-> fliplr p=0.5" % n, "pixels": px},
                      "per_op": {"value": round(px / 1e6 / (po_ms / 1e3), 1), "unit": "Mpix/s"},
                      "pipeline_hbm": {"bytes_per_px": 24, "achieved_gbs": round(gbs, 1),
                                       "frac": round(gbs / peak, 4), "peak_source": pk},
                      "gpu_launches": args.steps * nl, "clocks": clk}), flush=True)


def run_grad(args, which):
    """Differentiable fwd+bwd.  grad4: 64 x 512x512x3, rotate U(-30,30) ->
    gaussian U(1,3) -> gamma U(0.7,1.5) -> rgb2grey, loss sum(out*W).
    grad5: 16 x 8192x8192x3, gaussian 8 -> rotate U(-45,45) -> brightness
    U(-0.1,0.1); backward recomputes the forward."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from millipyde_gb300.autograd import pipeline
    dev = torch.device("cuda:0")
    torch.manual_seed(SEED)
    if which == "grad4":
        B, Hh, Ww = (args.images if args.images != N_IMG_DEFAULT else 64), 512, 512
        theta = (torch.rand(B, dtype=torch.float64, device=dev) * 60 - 30).requires_grad_()
        sigma = (1 + 2 * torch.rand(B, dtype=torch.float64, device=dev)).requires_grad_()
        gamma = (0.7 + 0.8 * torch.rand(B, dtype=torch.float64, device=dev)).requires_grad_()
        ops = [("rotate", theta), ("gaussian", sigma), ("adjust_gamma", gamma), ("rgb2grey",)]
        params = [theta, sigma, gamma]
        bpp, wshape = 44, (B, Hh, Ww)
        desc = "64 x 512x512x3, rotate U(-30,30) -> gaussian U(1,3) -> gamma U(0.7,1.5) -> rgb2grey"
    else:
        B, Hh, Ww = (args.images if args.images != N_IMG_DEFAULT else 16), 8192, 8192
        theta = (torch.rand(B, dtype=torch.float64, device=dev) * 90 - 45).requires_grad_()
        delta = (torch.rand(B, dtype=torch.float64, device=dev) * 0.2 - 0.1).requires_grad_()
        ops = [("gaussian", 8.0), ("rotate", theta), ("brightness", delta)]
        params = [theta, delta]
        bpp, wshape = 60, (B, Hh, Ww, 3)
        desc = "16 x 8192x8192x3, gaussian 8 -> rotate U(-45,45) -> brightness U(-0.1,0.1)"
    x = torch.rand(B, Hh, Ww, 3, device=dev, requires_grad=True)
    Wt = torch.randn(wshape, device=dev)

    def step():
        for p in [x] + params:
            p.grad = None
        y = pipeline(x, ops)
        y.backward(Wt)          # d(sum(y * W))/dy = W

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    clocks = Clocks()
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    e1.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    px = B * Hh * Ww
    peak, pk = measured_peaks()
    gbs = px * bpp / (ms / 1e3) / 1e9
    print(json.dumps({"metric": "Mpix/s fwd+bwd differentiable chain", "value": round(px / 1e6 / (ms / 1e3), 1),
                      "unit": "Mpix/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": desc, "loss": "sum(out * W), W ~ N(0,1)"},
                      "pipeline_hbm": {"bytes_per_px": bpp, "achieved_gbs": round(gbs, 1),
                                       "frac": round(gbs / peak, 4), "peak_source": pk},
                      "torch_peak_memory_gb": round(torch.cuda.max_memory_allocated() / 1e9, 2),
                      "clocks": clk}), flush=True)


def main():
    global N_IMG
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--images", type=int, default=N_IMG,
                    help="batch size (profiling runs use a smaller batch)")
    ap.add_argument("--legs", default="all", choices=["all", "fused"],
                    help="'fused' times only the fused plan (profiling runs)")
    ap.add_argument("--workload", default="uniform", choices=["uniform", "ragged", "grad4", "grad5"],
                    help="uniform: the headline batch; the others are the ragged, "
                         "differentiable and large-image configurations")
    args = ap.parse_args()
    N_IMG = args.images
    CONFIG["images"] = N_IMG
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ragged":
        run_ragged(args)
    elif args.workload in ("grad4", "grad5"):
        run_grad(args, args.workload)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
