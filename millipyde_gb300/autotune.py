"""Autotuner: the gaussian tile kernel's tile shape, the persistent
kernels' geometry and the gaussian -> rotate fusion split.

The gaussian segment kernel processes tw x th output pixels per CTA; the best
shape depends on the channel variant (source channels, channels after the
prologue), whether a prologue runs, and the radius (halo size versus shared
memory and CTAs per SM).  tune_gaussian() times every candidate tile on the
device -- a plan over a batch of synthetic images, CUDA events around its
launch -- and records the fastest with mpk_tune_set_gauss_tile; the planner
then uses it for every batch and per-op call in that radius range.

tune_kernels() does the same for the hot kernels' launch geometry
(mpk_tune_set_kernel: work items per CTA, CTAs per SM and strip width of the
streaming gaussian, CTAs per SM of the footprint rotate and of the fused
gaussian + rotate) on a ragged and a uniform synthetic batch, coordinate by
coordinate, and decides the fusion split (mpk_tune_set_fuse) by timing the
uniform chain fused and split.

Results persist in a JSON table keyed by GPU name: the package ships one for
GB300 (tune_gb300.json, produced by tune_defaults() on a GB300), applied at
import; MILLIPYDE_GB300_TUNE names an alternative file.
"""
from __future__ import annotations

import ctypes as C
import json
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
SHIPPED = os.path.join(HERE, "tune_gb300.json")

CANDIDATES = [(128, 32), (96, 32), (64, 64), (64, 32), (64, 16), (128, 16), (48, 32), (32, 32),
              (32, 16), (128, 8), (64, 8), (16, 16), (16, 8), (8, 8)]


def _sigma_for_radius(r):
    # radius = ceil(3 sigma): (r - 0.5) / 3 lands strictly inside (r-1, r]
    return (r - 0.5) / 3.0


def time_gaussian(cin, cmid, has_pro, radius, tw, th, n_img=24, height=1024, width=1024, reps=5):
    """Milliseconds per launch of the gaussian segment with tile (tw, th)."""
    import torch

    L = _abi.lib()
    if L.mpk_tune_set_gauss_tile(cin, cmid, int(has_pro), radius, radius, tw, th) != 0:
        return None
    stages = []
    if has_pro and cmid == 1:
        stages.append(_abi.stage("rgb2grey"))
    elif has_pro:
        stages.append(_abi.stage("brightness", 0.01))
    stages.append(_abi.stage("gaussian", _sigma_for_radius(radius)))
    st = _abi.stages(*stages)
    pitch_in = (width * cin * 4 + 15) // 16 * 16
    pitch_out = (width * cmid * 4 + 15) // 16 * 16
    x = torch.rand((n_img, height, pitch_in // 4), device="cuda")
    y = torch.empty((n_img, height, pitch_out // 4), device="cuda")
    ins = _abi.images([_abi.image(x[i].data_ptr(), height, width, cin, pitch_in) for i in range(n_img)])
    outs = _abi.images([_abi.image(y[i].data_ptr(), height, width, cmid, pitch_out) for i in range(n_img)])
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    plan = C.c_void_p()
    if L.mpk_plan_create(st, len(stages), ins, outs, n_img, 0, 0, sp, C.byref(plan)) != 0:
        return None
    try:
        _abi.check(L.mpk_plan_launch(plan, sp))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _abi.check(L.mpk_plan_launch(plan, sp))
        e1.record()
        e1.synchronize()
        nl = L.mpk_plan_num_launches(plan)
        return e0.elapsed_time(e1) / reps / max(1, nl) * nl
    finally:
        L.mpk_plan_destroy(plan)
        torch.cuda.synchronize()


def tune_gaussian(cin, cmid, has_pro, radius, radius_range=None, candidates=None, apply=True, **kw):
    """Times the candidates, records the fastest for radius_range (default
    (radius, radius)), returns {"tile": (tw, th), "ms": {...}}."""
    L = _abi.lib()
    times = {}
    for tw, th in candidates or CANDIDATES:
        t = time_gaussian(cin, cmid, has_pro, radius, tw, th, **kw)
        if t is not None:
            times["%dx%d" % (tw, th)] = round(t, 5)
    L.mpk_tune_clear()
    load()   # restore the table the timing runs overwrote
    if not times:
        return None
    best = min(times, key=times.get)
    tw, th = (int(v) for v in best.split("x"))
    lo, hi = radius_range or (radius, radius)
    if apply:
        _abi.check(L.mpk_tune_set_gauss_tile(cin, cmid, int(has_pro), lo, hi, tw, th))
    return {"cin": cin, "cmid": cmid, "has_pro": int(has_pro), "radius_lo": lo, "radius_hi": hi,
            "tile": [tw, th], "ms": times}


# (cin, cmid, has_pro, radius tuned at, radius range)
DEFAULT_CASES = [
    (3, 1, 1, 9, (1, 16)), (4, 1, 1, 9, (1, 16)),
    (1, 1, 0, 9, (1, 16)), (1, 1, 0, 24, (17, 48)),
    (3, 3, 0, 3, (1, 4)), (3, 3, 0, 6, (5, 8)), (3, 3, 0, 12, (9, 16)), (3, 3, 0, 24, (17, 48)),
    (4, 4, 0, 6, (1, 16)),
]


def tune_defaults(path=None, cases=DEFAULT_CASES, kernels=True, **kw):
    """Tunes the common cases (gaussian tiles, then the kernel geometry and
    the fusion split) and writes the JSON table."""
    entries = []
    for cin, cmid, pro, r, rr in cases:
        res = tune_gaussian(cin, cmid, pro, r, radius_range=rr, apply=False, **kw)
        if res:
            entries.append(res)
    if kernels:
        entries += tune_kernels()
    save(entries, path)
    load(path)
    return entries


# Launch kinds of mpk_plan_launch_info and mpk_tune_set_kernel.
KIND_ROTATE, KIND_GAUSS_STREAM, KIND_FUSED = 5, 8, 9
PARAM_ITEMS, PARAM_CTAS, PARAM_STRIP = 0, 1, 2
# (kind, param, candidate values; 0 = the built-in choice)
KERNEL_CANDIDATES = [
    (KIND_GAUSS_STREAM, PARAM_ITEMS, [0, 2, 8, 16]),
    (KIND_GAUSS_STREAM, PARAM_CTAS, [0, 2]),
    (KIND_GAUSS_STREAM, PARAM_STRIP, [0, 128]),
    (KIND_ROTATE, PARAM_CTAS, [0, 2, 3]),
    (KIND_FUSED, PARAM_CTAS, [0, 1]),
]


class _Batch:
    """A synthetic batch and its chain on the device, timed as one plan."""

    def __init__(self, kind, n):
        import math

        import numpy as np
        import torch

        rng = np.random.default_rng(7)
        if kind == "ragged":
            lo, hi = math.log(64), math.log(2048)
            sizes = [(int(round(math.exp(rng.uniform(lo, hi)))), int(round(math.exp(rng.uniform(lo, hi)))))
                     for _ in range(n)]
            self.stages = _abi.stages(
                _abi.stage("rotate", random=True, lo=(-45,), hi=(45,)),
                _abi.stage("gaussian", random=True, lo=(0.5,), hi=(4.0,)),
                _abi.stage("adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
                _abi.stage("brightness", random=True, lo=(-0.2,), hi=(0.2,)),
                _abi.stage("fliplr", probability=0.5))
            self.nst, cout = 5, 3
        else:
            sizes = [(1024, 1024)] * n
            self.stages = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0),
                                      _abi.stage("rotate", 17.0), _abi.stage("adjust_gamma", 0.8, 1.0))
            self.nst, cout = 4, 1
        self.keep, ins, outs = [], [], []
        for h, w in sizes:
            pi, po = (w * 12 + 15) // 16 * 16, (w * cout * 4 + 15) // 16 * 16
            x = torch.rand((h, pi // 4), device="cuda")
            y = torch.empty((h, po // 4), device="cuda")
            self.keep += [x, y]
            ins.append(_abi.image(x.data_ptr(), h, w, 3, pi))
            outs.append(_abi.image(y.data_ptr(), h, w, cout, po))
        self.ins, self.outs, self.n = _abi.images(ins), _abi.images(outs), n

    def time(self, reps=5):
        """Milliseconds per pass of the plan (CUDA events), or None."""
        import torch

        L = _abi.lib()
        sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        plan = C.c_void_p()
        if L.mpk_plan_create(self.stages, self.nst, self.ins, self.outs, self.n, 1, 0, sp, C.byref(plan)) != 0:
            return None
        try:
            _abi.check(L.mpk_plan_launch(plan, sp))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                _abi.check(L.mpk_plan_launch(plan, sp))
            e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) / reps
        finally:
            L.mpk_plan_destroy(plan)
            torch.cuda.synchronize()


def tune_kernels(ragged_images=150, uniform_images=24, candidates=KERNEL_CANDIDATES, apply=True):
    """Coordinate search over the kernel geometry knobs (each timed on the
    batch whose launches it affects) and the fusion split; returns the
    entries (recorded with mpk_tune_set_kernel / mpk_tune_set_fuse when
    apply)."""
    L = _abi.lib()
    batches = {"ragged": _Batch("ragged", ragged_images), "uniform": _Batch("uniform", uniform_images)}
    entries = []
    # fusion split on the uniform chain
    times = {}
    for mode, name in ((1, "fused"), (0, "split")):
        _abi.check(L.mpk_tune_set_fuse(mode))
        times[name] = batches["uniform"].time()
    fuse = 1 if (times["fused"] or 1e30) <= (times["split"] or 1e30) else 0
    _abi.check(L.mpk_tune_set_fuse(fuse))
    entries.append({"fuse": fuse, "ms": {k: round(v, 5) for k, v in times.items() if v}})
    for kind, param, values in candidates:
        batch = batches["uniform" if kind == KIND_FUSED else "ragged"]
        times = {}
        for v in values:
            if L.mpk_tune_set_kernel(kind, param, v) != 0:
                continue
            t = batch.time()
            if t is not None:
                times[v] = t
        best = min(times, key=times.get) if times else 0
        _abi.check(L.mpk_tune_set_kernel(kind, param, best))
        entries.append({"kernel_kind": kind, "param": param, "value": best,
                        "ms": {str(k): round(t, 5) for k, t in times.items()}})
    if not apply:
        _apply(entries, clear=False, undo=True)
    return entries


def _apply(entries, clear=False, undo=False):
    L = _abi.lib()
    n = 0
    for e in entries:
        if "fuse" in e:
            n += L.mpk_tune_set_fuse(0 if undo else e["fuse"]) == 0
        elif "kernel_kind" in e:
            n += L.mpk_tune_set_kernel(e["kernel_kind"], e["param"], 0 if undo else e["value"]) == 0
        elif not undo and L.mpk_tune_set_gauss_tile(e["cin"], e["cmid"], e["has_pro"], e["radius_lo"],
                                                    e["radius_hi"], e["tile"][0], e["tile"][1]) == 0:
            n += 1
    return n


def _device_name():
    L = _abi.lib()
    if L.mpdev_get_device_count() <= 0:
        return None
    buf = C.create_string_buffer(256)
    if L.mpdev_get_device_name(0, buf, 256) != 0:
        return None
    return buf.value.decode()


def save(entries, path=None):
    path = path or os.environ.get("MILLIPYDE_GB300_TUNE") or SHIPPED
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[_device_name() or "unknown"] = entries
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)


def load(path=None):
    """Applies the table for this GPU (by name) from path or the shipped file;
    returns the number of entries applied."""
    path = path or os.environ.get("MILLIPYDE_GB300_TUNE") or SHIPPED
    if not os.path.exists(path):
        return 0
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return 0
    return _apply(data.get(_device_name(), []))
