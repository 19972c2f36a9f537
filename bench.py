#!/usr/bin/env python3
"""Benchmark of the fused image pipeline on one GB300.

Headline workload (the ragged random-augmentation configuration): 1000
float32 RGB images whose height and width are each drawn log-uniformly in
[64, 2048] from a seed; per image, counter-RNG parameters: rotate U(-45,45)
deg (bilinear, zero fill) -> gaussian sigma U(0.5,4) (radius ceil(3 sigma))
-> adjust_gamma U(0.5,2) -> brightness U(-0.2,0.2) -> fliplr p=0.5.  One step
= one pass of the pipeline over the whole batch, replayed as a CUDA graph of
the fused plan (one launch per segment kind and compiled radius).

Reported (one JSON line on stdout):
  value        whole-batch Mpix/s of the fused ragged forward, inputs resident
               in HBM (4.0 GB, larger than L2: no flush between steps), CUDA
               events on the launching stream.
  per_op       Mpix/s of the plain per-op path on the same batch (one kernel
               per stage and image).
  e2e          the same metric through the C-ABI host-buffer entry
               (mpk_pipeline_run_host) from page-locked host memory: H2D of
               every input, the kernels and D2H of every output per step.
  roofline     the dominant kernel's algorithmic bytes per launch over its
               average CUDA-event duration, against the measured HBM copy
               bandwidth (MEASURED_PEAKS.json); traffic = ncu DRAM bytes.
  cpu_baseline the FP64 oracle port on the host cores for a bounded sample.
  fwd_bwd      the differentiable chains: 64 x 512x512x3 and 16 x 8192x8192x3
               forward + backward (with recomputation), Mpix/s, %HBM, peak
               memory.
  uniform      256 x 1024x1024x3, rgb2grey -> gaussian 3 -> rotate 17 ->
               adjust_gamma 0.8: fused vs per-op.
  plain_ops    each op alone on one 512x512x3 image: GPU per-op kernel and
               numpy/scipy on one host core, with the max-abs error of the
               GPU result against the FP64 oracle.
  max_abs_err  max-abs error against the FP64 oracle, per op and per workload.

`--impl reference` times the reference's CPU implementation of the path --
the oracle port (the reference has no CPU path of its own and its HIP
kernels cannot run here) -- with every host core, on a bounded sample of the
same ragged batch (every 8th image); its ms_per_step is the measured time of
that sample.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import multiprocessing as mpr
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20260303
METRIC = "Mpix/s fwd and fwd+bwd: fused ragged batch vs per-op kernels, 1 GB300, %HBM peak"
VALUE_IS = "fused ragged batch forward, Mpix/s (fwd+bwd under fwd_bwd)"

# ragged batch
N_RAGGED = 1000
RAGGED_SPEC = [dict(op="rotate", random=True, lo=(-45.0,), hi=(45.0,)),
               dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
               dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
               dict(op="brightness", random=True, lo=(-0.2,), hi=(0.2,)),
               dict(op="fliplr", probability=0.5)]
RAGGED_DESC = ("ragged: %d float32 RGB images, H and W log-uniform in [64, 2048], per-image rotate U(-45,45) "
               "-> gaussian sigma U(0.5,4) -> adjust_gamma U(0.5,2) -> brightness U(-0.2,0.2) -> fliplr p=0.5")
REF_EVERY = 8            # the CPU legs time every 8th image of the ragged batch

# uniform batch
N_UNI, H_UNI, W_UNI = 256, 1024, 1024
UNI_OPS = [("rgb2grey",), ("gaussian", 3.0), ("rotate", 17.0), ("adjust_gamma", 0.8)]


def ragged_sizes(n, seed=SEED):
    import numpy as np
    rng = np.random.default_rng(seed)
    lo, hi = math.log(64), math.log(2048)
    return [(int(round(math.exp(rng.uniform(lo, hi)))), int(round(math.exp(rng.uniform(lo, hi)))))
            for _ in range(n)]


def resolved_ops(spec, seed, index):
    """The ops image `index` runs, with its drawn parameters (oracle form)."""
    from oracle import oracle as O
    ops = []
    for s, d in enumerate(spec):
        run, p = O.resolve_stage(d, seed, index, s)
        if run:
            nargs = {"gaussian": 1, "rotate": 1, "brightness": 1, "adjust_gamma": 2, "colorize": 3}.get(d["op"], 0)
            ops.append((d["op"],) + tuple(p[:nargs]))
    return ops


def _stage(d):
    from millipyde_gb300 import _abi
    if d.get("random"):
        return _abi.stage(d["op"], random=True, lo=d["lo"], hi=d["hi"], probability=d.get("probability", -1.0))
    return _abi.stage(d["op"], *d.get("lo", ()), probability=d.get("probability", -1.0))


# ----------------------------------------------------------------- CPU legs
def _cpu_ragged_one(args):
    """FP64 oracle of image i of the ragged batch (seeded input); seconds."""
    import numpy as np
    from oracle import oracle as O
    i, h, w = args
    x = np.random.default_rng(SEED + i).random((h, w, 3), dtype=np.float32)
    t = time.perf_counter()
    O.run_ops(x, resolved_ops(RAGGED_SPEC, SEED, i))
    return time.perf_counter() - t


class CpuPool:
    """One spawn pool of host processes, created before any GPU work."""

    def __init__(self, workers):
        self.workers = workers
        self.pool = mpr.get_context("spawn").Pool(workers)

    def ragged_sample(self, n_images):
        sizes = ragged_sizes(n_images)
        items = [(i, h, w) for i, (h, w) in enumerate(sizes) if i % REF_EVERY == 0]
        items.sort(key=lambda t: -t[1] * t[2])            # largest first: balanced finish
        px = sum(h * w for _, h, w in items)
        t0 = time.perf_counter()
        self.pool.map(_cpu_ragged_one, items, chunksize=1)
        return px, len(items), time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    cp = CpuPool(workers)
    n = args.images or N_RAGGED
    cp.pool.map(_cpu_ragged_one, [(0, 64, 64)] * workers)           # start the workers
    for _ in range(args.warmup):
        cp.ragged_sample(n)
    secs, px, nimg = [], 0, 0
    for _ in range(args.steps):
        px, nimg, dt = cp.ragged_sample(n)
        secs.append(dt)
    cp.close()
    ms = 1000.0 * statistics.mean(secs)
    v = px / 1e6 / (ms / 1e3)
    sample = ("every %dth image of the ragged batch per step (%d images, %d px of %d), FP64 numpy oracle, "
              "one process per image (spawn pool of %d)" % (REF_EVERY, nimg, px, sum(h * w for h, w in ragged_sizes(n)),
                                                            workers))
    line = {"impl": "reference", "metric": METRIC, "value_is": VALUE_IS, "value": round(v, 3), "unit": "Mpix/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "ms_per_step_is": "measured time of the sample processed in one step",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": RAGGED_DESC % n, "images": n, "sample_images": nimg, "sample_pixels": px},
            "cpu_baseline": {"value": round(v, 3), "unit": "Mpix/s", "cores": workers, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU helpers
class Clocks:
    """nvidia-smi sampler running during a timed region (rows of the
    benchmarked GPU only, matched by UUID)."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.proc = None
        self.uuid = uuid
        self.path = os.environ.get("MP_BENCH_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), "mp_bench_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            d = os.path.dirname(self.path)
            if d:
                os.makedirs(d, exist_ok=True)
            self.f = open(self.path, "a")
            self.pos = self.f.tell()
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
        with open(self.path) as f:
            f.seek(self.pos)
            rows = f.read().splitlines()
        for row in rows:
            p = [q.strip() for q in row.split(",")]
            if len(p) < 9 or not p[1].isdigit():
                continue
            if self.uuid and p[0].lower().replace("gpu-", "") != self.uuid:
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


def gpu_uuid(torch):
    try:
        return str(torch.cuda.get_device_properties(0).uuid).lower().replace("gpu-", "")
    except Exception:  # noqa: BLE001 -- older torch without the field: sample every row
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic_per_px(workload, kind):
    """DRAM bytes per pixel ncu measured for a kernel kind of a workload
    (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(workload, {}).get(str(kind))
    except (OSError, ValueError, AttributeError):
        return None


KIND_NAMES = {0: "pointwise", 1: "gaussian tiles", 2: "rotate tiles", 3: "transpose",
              4: "gaussian strip stream", 5: "rotate footprint", 8: "gaussian stream (mp_vh family)",
              9: "gaussian + rotate fused (blur kept in shared memory)"}


def time_graph(torch, graph, stream, steps, uuid):
    """ms per replay over `steps` replays (CUDA events), clocks sampled."""
    clocks = Clocks(uuid)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(steps):
            graph.replay()
        e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    return e0.elapsed_time(e1) / steps, clk


def per_kind_timing(torch, L, plan, stream):
    """Per kernel kind: total ms (events around every launch of the plan),
    launches, algorithmic bytes, pixels."""
    from millipyde_gb300 import _abi
    sp = C.c_void_p(stream.cuda_stream)
    n = L.mpk_plan_num_launches(plan)
    per = {}
    for rep in range(2):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
        with torch.cuda.stream(stream):
            evs[0].record(stream)
            for i in range(n):
                _abi.check(L.mpk_plan_launch_range(plan, i, 1, sp))
                evs[i + 1].record(stream)
        evs[-1].synchronize()
        if rep == 0:
            continue
        for i in range(n):
            kind, nj, tiles, byt = C.c_int(), C.c_int(), C.c_int(), C.c_double()
            L.mpk_plan_launch_info(plan, i, C.byref(kind), C.byref(nj), C.byref(tiles), C.byref(byt))
            d = per.setdefault(kind.value, {"ms": 0.0, "launches": 0, "bytes": 0.0})
            d["ms"] += evs[i].elapsed_time(evs[i + 1])
            d["launches"] += 1
            d["bytes"] += byt.value
    return per


def roofline(per, workload):
    """Roofline object of the dominant kernel kind of a plan."""
    peak, pk = measured_peaks()
    dom = max(per, key=lambda k: per[k]["ms"])
    d = per[dom]
    avg_ms = d["ms"] / d["launches"]
    bpl = d["bytes"] / d["launches"]
    achieved = bpl / (avg_ms / 1e3) / 1e9
    tpp = ncu_traffic_per_px(workload, dom)
    # traffic per launch: ncu DRAM bytes per algorithmic byte x algorithmic bytes
    traffic = tpp * bpl if tpp else None
    return {"bound": "hbm", "kernel": KIND_NAMES.get(dom, str(dom)), "achieved": round(achieved, 1),
            "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": pk,
            "bytes_per_launch": bpl, "avg_launch_ms": round(avg_ms, 4),
            "traffic": None if traffic is None else round(traffic, 1),
            "per_kind_ms": {KIND_NAMES.get(k, str(k)): round(v["ms"], 4) for k, v in per.items()},
            "per_kind_launches": {KIND_NAMES.get(k, str(k)): v["launches"] for k, v in per.items()}}


def _maxerr(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.max(np.abs(a - b))) if a.size else 0.0


# ----------------------------------------------------------------- ragged (headline)
def bench_ragged(args, torch, L, uuid, cpu_pool):
    import numpy as np
    from millipyde_gb300 import _abi
    from oracle import oracle as O
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    n = args.images or N_RAGGED
    sizes = ragged_sizes(n)
    px = sum(h * w for h, w in sizes)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    keep, ins, outs = [], [], []
    st = _abi.stages(*[_stage(d) for d in RAGGED_SPEC])
    with torch.cuda.stream(stream):
        for h, w in sizes:
            pitch = (w * 3 * 4 + 15) // 16 * 16
            t = torch.rand((h, pitch // 4), device=dev, generator=gen)
            o = torch.empty((h, pitch // 4), device=dev)
            keep += [t, o]
            ins.append(_abi.image(t.data_ptr(), h, w, 3, pitch))
            outs.append(_abi.image(o.data_ptr(), h, w, 3, pitch))
    stream.synchronize()
    ia, oa = _abi.images(ins), _abi.images(outs)
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(st, len(RAGGED_SPEC), ia, oa, n, SEED, 0, sp, C.byref(plan)))
    nl = L.mpk_plan_num_launches(plan)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(max(3, args.warmup)):
        g.replay()
    ms, clk = time_graph(torch, g, stream, args.steps, uuid)
    value = px / 1e6 / (ms / 1e3)

    # oracle check of the timed outputs: the largest image and every 97th
    err = 0.0
    check = sorted(set([max(range(n), key=lambda i: sizes[i][0] * sizes[i][1])] + list(range(0, n, 97))))
    for i in check:
        h, w = sizes[i]
        x = keep[2 * i][:, : w * 3].cpu().numpy().reshape(h, w, 3)
        y = keep[2 * i + 1][:, : w * 3].cpu().numpy().reshape(h, w, 3)
        err = max(err, _maxerr(y, O.run_ops(x, resolved_ops(RAGGED_SPEC, SEED, i))))
    if not err <= 1e-5:
        raise SystemExit("bench.py: ragged output differs from the oracle by %.3g" % err)

    per = per_kind_timing(torch, L, plan, stream)
    rl = roofline(per, "ragged")
    L.mpk_plan_destroy(plan)

    out = {"value": value, "ms": ms, "clocks": clk, "launches": nl, "pixels": px, "err": err,
           "errs_checked": len(check), "roofline": rl}
    if args.legs == "all":
        # plain per-op path on the same batch
        po_steps = max(1, min(3, args.steps))
        _abi.check(L.mpk_pipeline_run_unfused(st, len(RAGGED_SPEC), ia, oa, n, SEED, 0, sp))
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(po_steps):
                _abi.check(L.mpk_pipeline_run_unfused(st, len(RAGGED_SPEC), ia, oa, n, SEED, 0, sp))
            e1.record(stream)
        e1.synchronize()
        out["per_op"] = px / 1e6 / (e0.elapsed_time(e1) / po_steps / 1e3)
        out["per_op_steps"] = po_steps

        # end to end from page-locked host buffers through the C-ABI
        hkeep, hins, houts = [], [], []
        h2d = d2h = 0
        for i, (h, w) in enumerate(sizes):
            hx = torch.empty((h, w * 3), dtype=torch.float32, pin_memory=True)
            hx.copy_(keep[2 * i][:, : w * 3])
            hy = torch.empty((h, w * 3), dtype=torch.float32, pin_memory=True)
            hkeep += [hx, hy]
            hins.append(_abi.image(hx.data_ptr(), h, w, 3, w * 12))
            houts.append(_abi.image(hy.data_ptr(), h, w, 3, w * 12))
            h2d += h * w * 12
            d2h += h * w * 12
        hia, hoa = _abi.images(hins), _abi.images(houts)
        # the first calls of the host path are slower (first DMA from fresh
        # page-locked pages, pool growth): three warm-up calls
        for _ in range(3):
            _abi.check(L.mpk_pipeline_run_host(st, len(RAGGED_SPEC), hia, hoa, n, SEED, 0, sp))
        # each step timed on its own: the median is the value, every step's
        # time is listed (occasional steps several times slower than the rest
        # come from the host: bare copies of the same bytes show them too)
        e2e_steps = max(1, min(7, args.steps))
        step_s = []
        for _ in range(e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _abi.check(L.mpk_pipeline_run_host(st, len(RAGGED_SPEC), hia, hoa, n, SEED, 0, sp))
            step_s.append(time.perf_counter() - t0)
        e2e_s = statistics.median(step_s)
        i0 = check[0]
        h, w = sizes[i0]
        d = float((hkeep[2 * i0 + 1] - keep[2 * i0 + 1][:, : w * 3].cpu()).abs().max())
        if not d <= 1e-6:
            raise SystemExit("bench.py: host-buffer path differs from the device path by %.3g" % d)
        out["e2e"] = {"value": round(px / 1e6 / e2e_s, 1), "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "steps": e2e_steps, "statistic": "median step",
                      "steps_ms": [round(1e3 * t, 2) for t in step_s],
                      "mean_value": round(px / 1e6 / statistics.mean(step_s), 1),
                      "path": "mpk_pipeline_run_host, page-locked host buffers"}
        del hkeep
        # CPU baseline: the oracle port on the host cores, every 8th image
        cpx, cn, cdt = cpu_pool.ragged_sample(n)
        out["cpu_baseline"] = {"value": round(cpx / 1e6 / cdt, 3), "unit": "Mpix/s", "cores": cpu_pool.workers,
                               "kind": "port",
                               "sample": "every %dth image of the ragged batch (%d images, %d px), FP64 numpy "
                                         "oracle, spawn pool of %d (%.1f s)" % (REF_EVERY, cn, cpx,
                                                                                cpu_pool.workers, cdt)}
    del keep
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------- uniform batch
def bench_uniform(args, torch, L, uuid):
    import numpy as np
    from millipyde_gb300 import _abi
    from oracle import oracle as O
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    n, H, W = (args.images if args.workload == "uniform" and args.images else N_UNI), H_UNI, W_UNI
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    with torch.cuda.stream(stream):
        x = torch.rand((n, H, W * 3), device=dev, dtype=torch.float32, generator=gen)
        y = torch.empty((n, H, W), device=dev, dtype=torch.float32)
    stream.synchronize()
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 17.0),
                     _abi.stage("adjust_gamma", 0.8, 1.0))
    ins = _abi.images([_abi.image(x[i].data_ptr(), H, W, 3, W * 12) for i in range(n)])
    outs = _abi.images([_abi.image(y[i].data_ptr(), H, W, 1, W * 4) for i in range(n)])
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(st, 4, ins, outs, n, 0, 0, sp, C.byref(plan)))
    nl = L.mpk_plan_num_launches(plan)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(max(3, args.warmup)):
        g.replay()
    steps = min(args.steps, 50)
    ms, clk = time_graph(torch, g, stream, steps, uuid)
    err = 0.0
    for i in (0, n - 1):
        err = max(err, _maxerr(y[i].cpu().numpy(), O.run_ops(x[i].view(H, W, 3).cpu().numpy(), UNI_OPS)))
    if not err <= 1e-5:
        raise SystemExit("bench.py: uniform output differs from the oracle by %.3g" % err)
    per = per_kind_timing(torch, L, plan, stream)
    L.mpk_plan_destroy(plan)
    px = n * H * W
    value = px / 1e6 / (ms / 1e3)
    peak, pk = measured_peaks()
    res = {"workload": "uniform batch: %d x 1024x1024x3 float32 RGB, rgb2grey -> gaussian sigma=3 (radius 9) "
                       "-> rotate 17 deg bilinear -> adjust_gamma 0.8" % n,
           "value": round(value, 1), "unit": "Mpix/s", "ms_per_step": round(ms, 4), "steps": steps,
           "gpu_launches_per_step": nl, "clocks": clk,
           "pipeline_hbm": {"bytes_per_px": 16, "achieved_gbs": round(px * 16 / (ms / 1e3) / 1e9, 1),
                            "frac": round(px * 16 / (ms / 1e3) / 1e9 / peak, 4), "peak_source": pk},
           "roofline": roofline(per, "uniform"), "max_abs_err": err}
    if args.legs == "all":
        po_steps = max(1, min(3, args.steps))
        _abi.check(L.mpk_pipeline_run_unfused(st, 4, ins, outs, n, 0, 0, sp))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(po_steps):
                _abi.check(L.mpk_pipeline_run_unfused(st, 4, ins, outs, n, 0, 0, sp))
            e1.record(stream)
        e1.synchronize()
        po = px / 1e6 / (e0.elapsed_time(e1) / po_steps / 1e3)
        res["per_op"] = {"value": round(po, 1), "unit": "Mpix/s", "steps": po_steps,
                         "fused_over_per_op": round(value / po, 2)}
    del x, y
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return res


# ----------------------------------------------------------------- fwd + bwd
def bench_grad(args, torch, L, uuid, which):
    """grad4: 64 x 512x512x3, rotate U(-30,30) -> gaussian U(1,3) -> gamma
    U(0.7,1.5) -> rgb2grey, loss sum(out*W).  grad5: 16 x 8192x8192x3,
    gaussian 8 -> rotate U(-45,45) -> brightness U(-0.1,0.1); the forward
    keeps its segment-boundary intermediates for the backward."""
    from millipyde_gb300.autograd import pipeline
    from oracle import oracle as O
    dev = torch.device("cuda:0")
    torch.manual_seed(SEED)
    if which == "grad4":
        B, Hh, Ww = (args.images if args.workload == which and args.images else 64), 512, 512
        theta = (torch.rand(B, dtype=torch.float64, device=dev) * 60 - 30).requires_grad_()
        sigma = (1 + 2 * torch.rand(B, dtype=torch.float64, device=dev)).requires_grad_()
        gamma = (0.7 + 0.8 * torch.rand(B, dtype=torch.float64, device=dev)).requires_grad_()
        ops = [("rotate", theta), ("gaussian", sigma), ("adjust_gamma", gamma), ("rgb2grey",)]
        params = [theta, sigma, gamma]
        bpp, wshape = 44, (B, Hh, Ww)
        desc = "%d x 512x512x3, rotate U(-30,30) -> gaussian U(1,3) -> gamma U(0.7,1.5) -> rgb2grey" % B
    else:
        B, Hh, Ww = (args.images if args.workload == which and args.images else 16), 8192, 8192
        theta = (torch.rand(B, dtype=torch.float64, device=dev) * 90 - 45).requires_grad_()
        delta = (torch.rand(B, dtype=torch.float64, device=dev) * 0.2 - 0.1).requires_grad_()
        ops = [("gaussian", 8.0), ("rotate", theta), ("brightness", delta)]
        params = [theta, delta]
        bpp, wshape = 60, (B, Hh, Ww, 3)
        desc = ("%d x 8192x8192x3, gaussian 8 -> rotate U(-45,45) -> brightness U(-0.1,0.1); the backward " % B +
                "reads the forward's saved blur and back-propagates the brightness from the output")
    x = torch.rand(B, Hh, Ww, 3, device=dev, requires_grad=True)
    Wt = torch.randn(wshape, device=dev)

    def step():
        for p in [x] + params:
            p.grad = None
        y = pipeline(x, ops)
        y.backward(Wt)          # d(sum(y * W))/dy = W
        return y

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    _abi_pool_reset(L)
    steps = min(args.steps, 20)
    clocks = Clocks(uuid)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        y = step()
    e1.record()
    e1.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / steps
    px = B * Hh * Ww
    peak, pk = measured_peaks()
    gbs = px * bpp / (ms / 1e3) / 1e9
    res = {"workload": desc, "loss": "sum(out * W), W ~ N(0,1)", "value": round(px / 1e6 / (ms / 1e3), 1),
           "unit": "Mpix/s", "ms_per_step": round(ms, 3), "steps": steps,
           "pipeline_hbm": {"bytes_per_px": bpp, "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                            "peak_source": pk},
           "peak_memory_gb": {"torch": round(torch.cuda.max_memory_allocated() / 1e9, 2),
                              "library_pool": round(_abi_pool_peak(L) / 1e9, 2)},
           "clocks": clk}
    if which == "grad4":
        # forward of two images against the oracle (the gradients are checked
        # against FD and a torch-composed reference in the tests)
        err = 0.0
        for b in (0, B - 1):
            ob = [("rotate", float(theta[b])), ("gaussian", float(sigma[b])), ("adjust_gamma", float(gamma[b])),
                  ("rgb2grey",)]
            err = max(err, _maxerr(y[b].detach().cpu().numpy().reshape(Hh, Ww),
                                   O.run_ops(x[b].detach().cpu().numpy(), ob)))
        res["max_abs_err_fwd"] = err
    del x, Wt, y
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return res


def _abi_pool_reset(L):
    L.mpdev_pool_reset_peak(0)


def _abi_pool_peak(L):
    r, u, h = C.c_uint64(), C.c_uint64(), C.c_uint64()
    if L.mpdev_pool_usage(0, C.byref(r), C.byref(u), C.byref(h)) != 0:
        return 0
    return h.value


# ----------------------------------------------------------------- plain ops
PLAIN_OPS = [("rgb2grey", ()), ("transpose", ()), ("fliplr", ()), ("gaussian", (2.0,)), ("rotate", (30.0,)),
             ("adjust_gamma", (2.2, 1.0)), ("brightness", (0.1,))]


def _cpu_op(name, p, x):
    """The op on one host core with numpy / scipy (the CPU counterpart the
    reference's tests compare with)."""
    import numpy as np
    from scipy import ndimage
    if name == "rgb2grey":
        return np.minimum(1.0, x[..., 0] * 0.2125 + x[..., 1] * 0.7154 + x[..., 2] * 0.0721)
    if name == "transpose":
        return np.ascontiguousarray(x.transpose(1, 0, 2))
    if name == "fliplr":
        return np.ascontiguousarray(x[:, ::-1])
    if name == "gaussian":
        r = int(math.ceil(3 * p[0]))
        k = np.exp(-np.arange(-r, r + 1) ** 2 / (2 * p[0] ** 2))
        k = (k / k.sum()).astype(np.float32)
        t = ndimage.correlate1d(x, k, axis=0, mode="constant")
        return ndimage.correlate1d(t, k, axis=1, mode="constant")
    if name == "rotate":
        h, w = x.shape[:2]
        th = math.radians(p[0])
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
        sx = math.cos(th) * (xx - w / 2) - math.sin(th) * (yy - h / 2) + w / 2
        sy = math.sin(th) * (xx - w / 2) + math.cos(th) * (yy - h / 2) + h / 2
        return np.stack([ndimage.map_coordinates(x[..., c], [sy, sx], order=1, mode="grid-constant")
                         for c in range(x.shape[2])], axis=-1)
    if name == "adjust_gamma":
        return np.clip(p[1] * np.power(x, p[0]), 0, 1)
    if name == "brightness":
        return np.clip(x + p[0], 0, 1)
    raise ValueError(name)


def bench_plain_ops(args, torch, L):
    """Each op alone on one 512x512x3 image (the reference's per-op
    methods): GPU per-op kernel (plain path, CUDA events over 200 calls),
    numpy/scipy on one host core, and the GPU result's max-abs error against
    the FP64 oracle.  512x512x3 fits in L2: launch-bound, not a roofline
    figure."""
    import numpy as np
    from millipyde_gb300 import _abi
    from oracle import oracle as O
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    H = W = 512
    xh = np.random.default_rng(SEED).random((H, W, 3), dtype=np.float32)
    x = torch.from_numpy(xh.reshape(H, W * 3)).to(dev)
    table = {}
    for name, p in PLAIN_OPS:
        st = _abi.stages(_abi.stage(name, *p))
        ins = _abi.images([_abi.image(x.data_ptr(), H, W, 3, W * 12)])
        outs = _abi.images([_abi.MPImage()])
        _abi.check(L.mpk_pipeline_shapes(st, 1, ins, outs, 1, 0, 0))
        m = outs[0]
        y = torch.empty((m.height, m.pitch // 4), device=dev)
        m.data = y.data_ptr()
        outs[0] = m
        reps = 200
        _abi.check(L.mpk_pipeline_run_unfused(st, 1, ins, outs, 1, 0, 0, sp))
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                _abi.check(L.mpk_pipeline_run_unfused(st, 1, ins, outs, 1, 0, 0, sp))
            e1.record(stream)
        e1.synchronize()
        us = 1000.0 * e0.elapsed_time(e1) / reps
        got = y[:, : m.width * m.channels].cpu().numpy().reshape(m.height, m.width, m.channels)
        if m.channels == 1:
            got = got[..., 0]
        ref = O.run_ops(xh, [(name,) + tuple(p)])
        err = _maxerr(got, ref)
        exact = name in ("transpose", "fliplr")
        if exact and not np.array_equal(got, ref):
            raise SystemExit("bench.py: %s is not bit-exact" % name)
        _cpu_op(name, p, xh)
        t0 = time.perf_counter()
        nrep = 3
        for _ in range(nrep):
            _cpu_op(name, p, xh)
        cpu_us = 1e6 * (time.perf_counter() - t0) / nrep
        table[name] = {"gpu_us": round(us, 2), "gpu_mpix_s": round(H * W / us, 1),
                       "cpu_us": round(cpu_us, 1), "cpu_mpix_s": round(H * W / cpu_us, 2),
                       "max_abs_err": err, "bit_exact": exact}
    return {"workload": "one 512x512x3 float32 image, U[0,1], each op alone through the plain per-op path "
                        "(mpk_pipeline_run_unfused, one stage); CPU: numpy/scipy.ndimage on one host core",
            "cpu_cores": 1, "ops": table}


# ----------------------------------------------------------------- host transfers
def bench_ingest(torch):
    """Host <-> device object transfers (gpuimage(ndarray), np.array(img)) of
    a 108 MB float32 RGB image with pitched rows, best of 3, against torch's
    pageable and page-locked host->device copies of the same bytes."""
    import numpy as np
    import millipyde_gb300 as mp
    x = np.random.default_rng(1).random((3000, 3001, 3), dtype=np.float32)
    nb = x.nbytes

    def best(fn):
        fn()
        ts = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return nb / min(ts) / 1e9

    img = mp.gpuimage(x)
    h2d = best(lambda: mp.gpuimage(x))
    d2h = best(lambda: np.array(img))
    if not np.array_equal(np.array(img), x):
        raise SystemExit("bench.py: gpuimage round trip differs")
    tx = torch.from_numpy(x)
    pageable = best(lambda: tx.to("cuda"))
    px = tx.pin_memory()
    pinned = best(lambda: px.to("cuda", non_blocking=True))
    return {"bytes": nb, "gpuimage_from_ndarray_gbs": round(h2d, 1), "ndarray_from_gpuimage_gbs": round(d2h, 1),
            "torch_pageable_h2d_gbs": round(pageable, 1), "torch_pinned_h2d_gbs": round(pinned, 1),
            "path": "library objects: one copy straight from pageable memory (2-D for pitched rows)"}


# ----------------------------------------------------------------- main GPU run
def run_ours(args):
    import torch
    # the CPU pool starts before any GPU work (a pool forked later would hang)
    cpu_pool = CpuPool(os.cpu_count() or 1) if args.legs == "all" else None

    import __graft_entry__
    __graft_entry__.build()
    from millipyde_gb300 import _abi

    if args.gpus != 1 or int(os.environ.get("WORLD_SIZE", "1")) != 1:
        raise SystemExit("bench.py: this build measures one GPU (replicas only); run with --gpus 1")
    L = _abi.lib()
    torch.cuda.set_device(0)
    uuid = gpu_uuid(torch)
    if args.fuse != "auto":
        _abi.check(L.mpk_tune_set_fuse(1 if args.fuse == "on" else 0))

    if args.workload in ("grad4", "grad5"):
        print(json.dumps(bench_grad(args, torch, L, uuid, args.workload)), flush=True)
        return
    if args.workload == "uniform":
        print(json.dumps(bench_uniform(args, torch, L, uuid)), flush=True)
        return

    rg = bench_ragged(args, torch, L, uuid, cpu_pool)
    peak, pk = measured_peaks()
    px = rg["pixels"]
    gbs = px * 24 / (rg["ms"] / 1e3) / 1e9
    line = {"metric": METRIC, "value_is": VALUE_IS, "value": round(rg["value"], 1), "unit": "Mpix/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(rg["ms"], 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": RAGGED_DESC % (args.images or N_RAGGED), "images": args.images or N_RAGGED,
                       "pixels": px, "seed": SEED,
                       "l2": "inputs (%.1f GB) larger than L2 (129 MB); no flush between steps" % (px * 12 / 1e9)},
            "pipeline_hbm": {"bytes_per_px": 24, "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                             "peak_source": pk},
            "roofline": rg["roofline"], "clocks": rg["clocks"], "gpu_launches": args.steps * rg["launches"]}
    if args.legs == "all":
        line["per_op"] = {"value": round(rg["per_op"], 1), "unit": "Mpix/s", "steps": rg["per_op_steps"],
                          "fused_over_per_op": round(rg["value"] / rg["per_op"], 2)}
        line["e2e"] = rg["e2e"]
        line["cpu_baseline"] = rg["cpu_baseline"]
        cpu_pool.close()
        uni = bench_uniform(args, torch, L, uuid)
        g4 = bench_grad(args, torch, L, uuid, "grad4")
        g5 = bench_grad(args, torch, L, uuid, "grad5")
        plain = bench_plain_ops(args, torch, L)
        line["ingest"] = bench_ingest(torch)
        line["fwd_bwd"] = {"grad4": g4, "grad5": g5}
        line["uniform"] = uni
        line["plain_ops"] = plain
        line["max_abs_err"] = {
            "tolerance": 1e-5,
            "per_op_512x512x3": {k: v["max_abs_err"] for k, v in plain["ops"].items()},
            "ragged": {"max": rg["err"], "images_checked": rg["errs_checked"]},
            "uniform": {"max": uni["max_abs_err"], "images_checked": 2},
            "grad4_forward": {"max": g4["max_abs_err_fwd"], "images_checked": 2}}
    else:
        line["max_abs_err"] = {"ragged": {"max": rg["err"], "images_checked": rg["errs_checked"]}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--images", type=int, default=0,
                    help="batch size of the selected --workload (default: ragged 1000, uniform 256, "
                         "grad4 64, grad5 16; profiling runs use a smaller batch)")
    ap.add_argument("--legs", default="all", choices=["all", "fused"],
                    help="'fused' times only the fused plan (profiling runs)")
    ap.add_argument("--fuse", default="auto", choices=["auto", "on", "off"],
                    help="gaussian + rotate fusion: the tuned/default choice, or forced (comparison runs)")
    ap.add_argument("--workload", default="ragged", choices=["ragged", "uniform", "grad4", "grad5"],
                    help="ragged: the headline line with every other configuration as extra keys; "
                         "the others print one configuration alone")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
