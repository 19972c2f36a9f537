"""GPU: the allocation-free entry point, mpk_pipeline_run_noalloc.

It exists for callers that cannot allocate device memory (an application
whose GPU memory belongs to its own allocator, or a loop where a cudaMalloc
would stall the device): it keeps its intermediates in a fixed 32 MB device
array compiled into the library.  Its results must match the regular entry
point, mpk_pipeline_run, call after call, even though every call reuses the
same array.  This file is collected last so a failure here comes after every
other test has run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pitch(w, c):
    return (w * c * 4 + 15) // 16 * 16


def _upload(xs):
    keep, ims = [], []
    for x in xs:
        h, w = x.shape[:2]
        c = 1 if x.ndim == 2 else x.shape[2]
        p = _pitch(w, c)
        t = torch.zeros(max(1, h), p // 4, device="cuda")
        t[:h, : w * c] = torch.from_numpy(x.reshape(h, w * c)).cuda()
        keep.append(t)
        ims.append(_abi.image(t.data_ptr(), h, w, c, p))
    return keep, _abi.images(ims)


def _outputs(st, nst, ins, n, seed, index0):
    L = _abi.lib()
    outs = _abi.images([_abi.MPImage() for _ in range(n)])
    _abi.check(L.mpk_pipeline_shapes(st, nst, ins, outs, n, seed, index0))
    keep = []
    for i in range(n):
        t = torch.full((max(1, outs[i].height), outs[i].pitch // 4), float("nan"), device="cuda")
        keep.append(t)
        outs[i].data = t.data_ptr()
    return keep, outs


def _host(t, m):
    a = t[: m.height, : m.width * m.channels].cpu().numpy()
    return a.reshape(m.height, m.width, m.channels)


def _run_both(st, nst, xs, seed, index0):
    """Outputs of the regular entry point and of the allocation-free one."""
    L = _abi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _kin, ins = _upload(xs)
    ref_keep, ref_outs = _outputs(st, nst, ins, len(xs), seed, index0)
    _abi.check(L.mpk_pipeline_run(st, nst, ins, ref_outs, len(xs), seed, index0, stream))
    na_keep, na_outs = _outputs(st, nst, ins, len(xs), seed, index0)
    _abi.check(L.mpk_pipeline_run_noalloc(st, nst, ins, na_outs, len(xs), seed, index0, stream))
    torch.cuda.synchronize()
    return ([_host(ref_keep[i], ref_outs[i]) for i in range(len(xs))],
            [_host(na_keep[i], na_outs[i]) for i in range(len(xs))])


def _oracle(spec, xs, seed, index0):
    """The FP64 oracle of the same stages, with the same per-image draws."""
    res = []
    for i, x in enumerate(xs):
        ops = []
        for s, d in enumerate(spec):
            run, p = O.resolve_stage(d, seed, index0 + i, s)
            if run:
                nargs = {"gaussian": 1, "rotate": 1, "brightness": 1, "adjust_gamma": 2}.get(d["op"], 0)
                ops.append((d["op"],) + tuple(p[:nargs]))
        res.append(O.run_ops(x, ops))
    return res


def test_noalloc_matches_regular_entry_point_twice(gpu):
    rng = np.random.default_rng(11)
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(3.0,)), dict(op="rotate", lo=(17.0,)),
            dict(op="adjust_gamma", lo=(0.8, 1.0))]
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 17.0),
                     _abi.stage("adjust_gamma", 0.8, 1.0))
    for call in range(2):   # two calls in a row: the shared array holds the previous call's data
        xs = [rng.random((150 + 7 * i, 210 - 5 * i, 3), dtype=np.float32) for i in range(3)]
        ref, got = _run_both(st, 4, xs, 0, 0)
        for a, b, o in zip(ref, got, _oracle(spec, xs, 0, 0)):
            assert a.shape == b.shape
            assert maxabs(a, b) <= TOL, call
            assert maxabs(b[..., 0], o) <= TOL, call


def test_noalloc_ragged_random_stages_twice(gpu):
    rng = np.random.default_rng(12)
    spec = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
            dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
            dict(op="transpose", probability=0.5),
            dict(op="fliplr", probability=0.5)]
    st = _abi.stages(_abi.stage("rotate", random=True, lo=(-45,), hi=(45,)),
                     _abi.stage("gaussian", random=True, lo=(0.5,), hi=(4.0,)),
                     _abi.stage("adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
                     _abi.stage("transpose", probability=0.5),
                     _abi.stage("fliplr", probability=0.5))
    for call in range(2):
        xs = [rng.random((int(rng.integers(20, 300)), int(rng.integers(20, 300)), 3), dtype=np.float32)
              for _ in range(5)]
        ref, got = _run_both(st, 5, xs, 99 + call, 10 * call)
        for a, b, o in zip(ref, got, _oracle(spec, xs, 99 + call, 10 * call)):
            assert a.shape == b.shape == o.shape
            assert maxabs(a, b) <= TOL, call
            assert maxabs(b, o) <= TOL, call


def _pool():
    r, u = C.c_uint64(), C.c_uint64()
    _abi.check(_abi.lib().mpdev_pool_usage(torch.cuda.current_device(), C.byref(r), C.byref(u), None))
    return r.value, u.value


def test_noalloc_allocates_no_device_memory(gpu):
    """Neither the library's memory pool nor the device's free memory moves
    across calls of the allocation-free entry point (after a first call,
    which may load the library's kernels)."""
    L = _abi.lib()
    rng = np.random.default_rng(13)
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 2.0), _abi.stage("rotate", 21.0))
    xs = [rng.random((300, 400, 3), dtype=np.float32) for _ in range(2)]
    _kin, ins = _upload(xs)
    _kout, outs = _outputs(st, 3, ins, 2, 0, 0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(L.mpk_pipeline_run_noalloc(st, 3, ins, outs, 2, 0, 0, stream))
    torch.cuda.synchronize()
    pool0, free0 = _pool(), torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _abi.check(L.mpk_pipeline_run_noalloc(st, 3, ins, outs, 2, 0, 0, stream))
    torch.cuda.synchronize()
    assert _pool() == pool0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_a_batch_before_any_launch(gpu):
    """A small first image and an oversize second one: the call is rejected
    during validation, so the first image's output is never written."""
    L = _abi.lib()
    st = _abi.stages(_abi.stage("gaussian", 1.0), _abi.stage("rotate", 5.0))
    x0 = torch.rand(40, 50 * 3, device="cuda")
    y0 = torch.full((40, 50 * 3), 7.0, device="cuda")
    x1 = torch.zeros(2100, 2100 * 3, device="cuda")
    y1 = torch.full((2100, 2100 * 3), 7.0, device="cuda")
    ins = _abi.images([_abi.image(x0.data_ptr(), 40, 50, 3, 600), _abi.image(x1.data_ptr(), 2100, 2100, 3, 25200)])
    outs = _abi.images([_abi.image(y0.data_ptr(), 40, 50, 3, 600), _abi.image(y1.data_ptr(), 2100, 2100, 3, 25200)])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.mpk_pipeline_run_noalloc(st, 2, ins, outs, 2, 0, 0, stream) == _abi.MP_ERROR_TOO_LARGE
    torch.cuda.synchronize()
    assert bool((y0 == 7.0).all()) and bool((y1 == 7.0).all())
    # the same first image alone still runs
    _abi.check(L.mpk_pipeline_run_noalloc(st, 2, ins, outs, 1, 0, 0, stream))
    torch.cuda.synchronize()
    assert not bool((y0 == 7.0).all())


def test_noalloc_rejects_intermediates_above_its_limit(gpu):
    """A 2100 x 2100 RGB intermediate (53 MB) exceeds the 16 MB half."""
    L = _abi.lib()
    st = _abi.stages(_abi.stage("gaussian", 1.0), _abi.stage("rotate", 5.0))
    x = torch.zeros(2100, 2100 * 3, device="cuda")
    y = torch.full((2100, 2100 * 3), 7.0, device="cuda")
    ins = _abi.images([_abi.image(x.data_ptr(), 2100, 2100, 3, 2100 * 12)])
    outs = _abi.images([_abi.image(y.data_ptr(), 2100, 2100, 3, 2100 * 12)])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.mpk_pipeline_run_noalloc(st, 2, ins, outs, 1, 0, 0, stream) == _abi.MP_ERROR_TOO_LARGE
    torch.cuda.synchronize()
    assert bool((y == 7.0).all())   # nothing was launched
