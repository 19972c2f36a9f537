"""Autotuner for the gaussian kernel's tile shape.

The gaussian segment kernel processes tw x th output pixels per CTA; the best
shape depends on the channel variant (source channels, channels after the
prologue), whether a prologue runs, and the radius (halo size versus shared
memory and CTAs per SM).  tune_gaussian() times every candidate tile on the
device -- a plan over a batch of synthetic images, CUDA events around its
launch -- and records the fastest with mpk_tune_set_gauss_tile; the planner
then uses it for every batch and per-op call in that radius range.

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


def tune_defaults(path=None, cases=DEFAULT_CASES, **kw):
    """Tunes the common cases and writes the JSON table."""
    entries = []
    for cin, cmid, pro, r, rr in cases:
        res = tune_gaussian(cin, cmid, pro, r, radius_range=rr, apply=False, **kw)
        if res:
            entries.append(res)
    save(entries, path)
    load(path)
    return entries


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
    L = _abi.lib()
    name = _device_name()
    n = 0
    for e in data.get(name, []):
        if L.mpk_tune_set_gauss_tile(e["cin"], e["cmid"], e["has_pro"], e["radius_lo"], e["radius_hi"],
                                     e["tile"][0], e["tile"][1]) == 0:
            n += 1
    return n
