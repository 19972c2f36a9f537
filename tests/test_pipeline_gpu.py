"""GPU parity of the fused batch path (mpk_pipeline_run / plans) through the
C-ABI: fused == oracle, fused == unfused per-op kernels, ragged batches with
seeded per-image random parameters, shape-changing probabilistic stages,
L2 chunking, and CUDA-graph replay of a plan."""
import ctypes as C
import math

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pitch(w, c):
    return (w * c * 4 + 15) // 16 * 16


def dev_image(x):
    h, w = x.shape[:2]
    c = 1 if x.ndim == 2 else x.shape[2]
    pitch = _pitch(w, c)
    t = torch.zeros(max(1, h), pitch // 4, device="cuda", dtype=torch.float32)
    if h and w:
        t[:h, : w * c] = torch.from_numpy(np.ascontiguousarray(x).reshape(h, w * c)).cuda()
    return t, _abi.image(t.data_ptr(), h, w, c, pitch)


def alloc_like(m):
    t = torch.full((max(1, m.height), m.pitch // 4), float("nan"), device="cuda", dtype=torch.float32)
    m.data = t.data_ptr()
    return t


def host(t, m):
    a = t[: m.height, : m.width * m.channels].cpu().numpy()
    return a.reshape(m.height, m.width) if m.channels == 1 else a.reshape(m.height, m.width, m.channels)


def run_batch(stage_list, xs, seed=0, index0=0, fused=True):
    L = _abi.lib()
    st = _abi.stages(*stage_list)
    keep, ins = [], []
    for x in xs:
        t, m = dev_image(x)
        keep.append(t)
        ins.append(m)
    ins_a = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(st, len(stage_list), ins_a, outs, len(xs), seed, index0))
    obufs = [alloc_like(outs[i]) for i in range(len(xs))]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    fn = L.mpk_pipeline_run if fused else L.mpk_pipeline_run_unfused
    _abi.check(fn(st, len(stage_list), ins_a, outs, len(xs), seed, index0, stream))
    torch.cuda.synchronize()
    return [host(obufs[i], outs[i]) for i in range(len(xs))]


def oracle_batch(spec, xs, seed=0, index0=0):
    res = []
    for i, x in enumerate(xs):
        ops = []
        for s, d in enumerate(spec):
            run, p = O.resolve_stage(d, seed, index0 + i, s)
            if not run:
                continue
            name = d["op"]
            nargs = {"gaussian": 1, "rotate": 1, "brightness": 1, "adjust_gamma": 2, "colorize": 3}.get(name, 0)
            ops.append((name,) + tuple(p[:nargs]))
        res.append(O.run_ops(x, ops))
    return res


def to_stage(d):
    if d.get("random"):
        return _abi.stage(d["op"], random=True, lo=d["lo"], hi=d["hi"], probability=d.get("probability", -1.0))
    return _abi.stage(d["op"], *d.get("lo", ()), probability=d.get("probability", -1.0))


@pytest.fixture
def rng():
    return np.random.default_rng(7)


def check_spec(spec, xs, seed=0, index0=0, tol=TOL):
    stages = [to_stage(d) for d in spec]
    ref = oracle_batch(spec, xs, seed, index0)
    fused = run_batch(stages, xs, seed, index0, fused=True)
    unfused = run_batch(stages, xs, seed, index0, fused=False)
    for a, b, r in zip(fused, unfused, ref):
        assert a.shape == r.shape
        assert maxabs(a, r) <= tol
        assert maxabs(b, r) <= tol
    return fused


def test_uniform_batch_grey_gauss_rotate_gamma(gpu, rng):
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(3.0,)), dict(op="rotate", lo=(17.0,)),
            dict(op="adjust_gamma", lo=(0.8, 1.0))]
    xs = [rng.random((96, 128, 3), dtype=np.float32) for _ in range(4)]
    check_spec(spec, xs)


def test_ragged_random_augmentation(gpu, rng):
    spec = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
            dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
            dict(op="brightness", random=True, lo=(-0.2,), hi=(0.2,)),
            dict(op="fliplr", probability=0.5)]
    xs = []
    for _ in range(24):
        h, w = (int(round(math.exp(rng.uniform(math.log(8), math.log(300))))) for _ in range(2))
        xs.append(rng.random((h, w, 3), dtype=np.float32))
    check_spec(spec, xs, seed=99, index0=5)


def test_differentiable_chain_forward(gpu, rng):
    spec = [dict(op="rotate", random=True, lo=(-30,), hi=(30,)),
            dict(op="gaussian", random=True, lo=(1.0,), hi=(3.0,)),
            dict(op="adjust_gamma", random=True, lo=(0.7, 1.0), hi=(1.5, 1.0)),
            dict(op="rgb2grey")]
    xs = [rng.random((64, 64, 3), dtype=np.float32) for _ in range(6)]
    check_spec(spec, xs, seed=3)


def test_large_radius_chain(gpu, rng):
    spec = [dict(op="gaussian", lo=(8.0,)), dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="brightness", random=True, lo=(-0.1,), hi=(0.1,))]
    xs = [rng.random((200, 180, 3), dtype=np.float32) for _ in range(3)]
    check_spec(spec, xs, seed=11)


def test_shape_changing_probabilistic_stages(gpu, rng):
    spec = [dict(op="transpose", probability=0.5), dict(op="fliplr", probability=0.5),
            dict(op="rgb2grey", probability=0.5), dict(op="colorize", random=True, lo=(0.5, 0.5, 0.5),
                                                      hi=(1.5, 1.5, 1.5), probability=0.7),
            dict(op="gaussian", lo=(1.0,)), dict(op="transpose")]
    xs = [rng.random((30 + i, 50 - i, 3), dtype=np.float32) for i in range(16)]
    check_spec(spec, xs, seed=1234)


def test_every_op_alone_and_rgba(gpu, rng):
    for spec in ([dict(op="fliplr")], [dict(op="transpose")], [dict(op="rgb2grey")],
                 [dict(op="brightness", lo=(0.3,))], [dict(op="colorize", lo=(1.2, 0.7, 0.0))],
                 [dict(op="adjust_gamma", lo=(2.2, 1.0))], [], [dict(op="fliplr"), dict(op="fliplr")]):
        xs = [rng.random((17, 29, 4), dtype=np.float32), rng.random((5, 3), dtype=np.float32)]
        out = check_spec(spec, xs)
        if spec and all(d["op"] in ("fliplr", "transpose") for d in spec):
            for o, r in zip(out, oracle_batch(spec, xs)):
                assert np.array_equal(o, r)


def test_pointwise_before_rotate_runs_per_neighbour(gpu, rng):
    spec = [dict(op="adjust_gamma", lo=(2.0, 1.0)), dict(op="brightness", lo=(0.1,)),
            dict(op="rotate", lo=(33.0,)), dict(op="adjust_gamma", lo=(0.5, 1.0))]
    xs = [rng.random((40, 44, 3), dtype=np.float32)]
    check_spec(spec, xs)


def test_pointwise_before_gaussian_keeps_zero_padding(gpu, rng):
    # brightness(+0.5) before the blur must not leak into the padding
    spec = [dict(op="brightness", lo=(0.5,)), dict(op="gaussian", lo=(2.0,))]
    xs = [rng.random((33, 47, 3), dtype=np.float32), rng.random((33, 47), dtype=np.float32)]
    check_spec(spec, xs)


def test_channel_preserving_gaussian_strips_and_mirror(gpu, rng):
    # 1-channel / RGB / RGBA blur across several strips, a per-channel
    # prologue and epilogue, a mirrored output; radii 2, 4 and 12 (compiled
    # one by one), 14, 20 and 24 (the buckets 16, 20, 24)
    for c in (1, 3, 4):
        for sigma in (0.4, 1.3, 4.0, 4.4, 6.5, 8.0):
            spec = [dict(op="colorize", lo=(1.2, 0.7, 0.9)), dict(op="gaussian", lo=(sigma,)),
                    dict(op="adjust_gamma", lo=(0.8, 1.0)), dict(op="fliplr")]
            shape = (70, 301) if c == 1 else (70, 301, c)
            small = (9, 5) if c == 1 else (9, 5, c)
            xs = [rng.random(shape, dtype=np.float32), rng.random(small, dtype=np.float32)]
            check_spec(spec, xs)
            check_spec(spec[1:2], xs[:1])


def test_gaussian_launch_mixing_radius_buckets(gpu, rng):
    # one batch whose radii fall on both sides of 12: two launches of the
    # streaming kernels, images in radius order
    spec = [dict(op="gaussian", random=True, lo=(0.5,), hi=(7.5,))]
    xs = [rng.random((40 + 3 * i, 90 - 2 * i, 3), dtype=np.float32) for i in range(12)]
    check_spec(spec, xs, seed=5)


def test_chunking_over_l2_budget(gpu, rng):
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(2.0,)), dict(op="rotate", lo=(10.0,))]
    xs = [rng.random((640, 640, 3), dtype=np.float32) for _ in range(40)]   # > 48 MB of intermediates
    check_spec(spec, xs[:3] + xs[3:], tol=TOL)


def test_empty_and_zero_size(gpu, rng):
    assert run_batch([_abi.stage("rotate", 5.0)], []) == []
    out = run_batch([_abi.stage("gaussian", 1.0)], [np.zeros((0, 7, 3), np.float32)])
    assert out[0].size == 0


def test_plan_replay_and_cuda_graph(gpu, rng):
    L = _abi.lib()
    stages = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 17.0),
                         _abi.stage("adjust_gamma", 0.8, 1.0))
    xs = [rng.random((128, 160, 3), dtype=np.float32) for _ in range(5)]
    keep, ins = [], []
    for x in xs:
        t, m = dev_image(x)
        keep.append(t)
        ins.append(m)
    ins_a = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(stages, 4, ins_a, outs, len(xs), 0, 0))
    obufs = [alloc_like(outs[i]) for i in range(len(xs))]
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    plan = C.c_void_p()
    with torch.cuda.stream(s):
        _abi.check(L.mpk_plan_create(stages, 4, ins_a, outs, len(xs), 0, 0, sp, C.byref(plan)))
        # launches per plan do not grow with the batch: gaussian (with the
        # rgb2grey prologue), rotate (with the adjust_gamma epilogue); one
        # launch when the two are fused
        fused = L.mpk_plan_num_launches(plan)
        assert fused in (1, 2)
        _abi.check(L.mpk_plan_launch(plan, sp))
        s.synchronize()
        first = [host(obufs[i], outs[i]).copy() for i in range(len(xs))]
        for t in obufs:
            t.fill_(-1.0)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        g.replay()
        g.replay()
        torch.cuda.synchronize()
    again = [host(obufs[i], outs[i]) for i in range(len(xs))]
    for a, b, x in zip(first, again, xs):
        assert np.array_equal(a, b)
        ref = O.run_ops(x, [("rgb2grey",), ("gaussian", 3.0), ("rotate", 17.0), ("adjust_gamma", 0.8, 1.0)])
        assert maxabs(a, ref) <= TOL
    _abi.check(L.mpk_plan_destroy(plan))
    torch.cuda.synchronize()


_FRESH_CAPTURE = r"""
import ctypes as C, sys
sys.path.insert(0, sys.argv[1])
import torch
from millipyde_gb300 import _abi
L = _abi.lib()
x = torch.rand(2, 64, 64 * 3, device="cuda")
y = torch.empty(2, 64, 64, device="cuda")
st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 9.0))
ins = _abi.images([_abi.image(x[i].data_ptr(), 64, 64, 3, 768) for i in range(2)])
outs = _abi.images([_abi.image(y[i].data_ptr(), 64, 64, 1, 256) for i in range(2)])
s = torch.cuda.Stream()
plan = C.c_void_p()
_abi.check(L.mpk_plan_create(st, 3, ins, outs, 2, 0, 0, C.c_void_p(s.cuda_stream), C.byref(plan)))
s.synchronize()
g = torch.cuda.CUDAGraph()
with torch.cuda.graph(g, stream=s):
    _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
g.replay()
torch.cuda.synchronize()
print("ok", float(y.sum()))
"""


def test_plan_capture_in_fresh_process(gpu):
    """The first library call of a process may be a plan whose launch is
    captured: all device set-up must happen at plan creation."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH_CAPTURE, root], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("ok")


def _launch_kinds(spec_stages, nst, xs):
    L = _abi.lib()
    keep, ins = [], []
    for x in xs:
        t, m = dev_image(x)
        keep.append(t)
        ins.append(m)
    ia = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(spec_stages, nst, ia, outs, len(xs), 0, 0))
    keep += [alloc_like(outs[i]) for i in range(len(xs))]
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(spec_stages, nst, ia, outs, len(xs), 0, 0, None, C.byref(plan)))
    kinds = []
    for i in range(L.mpk_plan_num_launches(plan)):
        k = C.c_int()
        L.mpk_plan_launch_info(plan, i, C.byref(k), None, None, None)
        kinds.append(k.value)
    _abi.check(L.mpk_plan_destroy(plan))
    torch.cuda.synchronize()
    return kinds


@pytest.mark.parametrize("sigma", [1.3, 3.0, 6.0])
def test_grey_after_colour_gaussian_is_split(gpu, rng, sigma):
    """rgb2grey after a colour gaussian (no spatial op after it) runs as a
    pointwise pass after the channel-preserving streaming blur; with a
    rotate after it the grey stays the blur's epilogue."""
    xs = [rng.random((h, w, 3), dtype=np.float32) for h, w in ((96, 128), (61, 203), (300, 40))]
    spec = [dict(op="gaussian", lo=(sigma,)), dict(op="adjust_gamma", lo=(0.7, 1.0)), dict(op="rgb2grey"),
            dict(op="brightness", lo=(0.05,))]
    check_spec(spec, xs)
    kinds = _launch_kinds(_abi.stages(*[to_stage(d) for d in spec]), len(spec), xs)
    assert kinds[-1] == 0                       # MPK_POINT last: the grey split off the blur
    spec2 = [dict(op="gaussian", lo=(sigma,)), dict(op="rgb2grey"), dict(op="rotate", lo=(12.0,))]
    check_spec(spec2, xs)
    assert 0 not in _launch_kinds(_abi.stages(*[to_stage(d) for d in spec2]), len(spec2), xs)
