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


def test_noalloc_matches_regular_entry_point_twice(gpu):
    rng = np.random.default_rng(11)
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 17.0),
                     _abi.stage("adjust_gamma", 0.8, 1.0))
    for call in range(2):   # two calls in a row: the shared array holds the previous call's data
        xs = [rng.random((150 + 7 * i, 210 - 5 * i, 3), dtype=np.float32) for i in range(3)]
        ref, got = _run_both(st, 4, xs, 0, 0)
        for a, b in zip(ref, got):
            assert a.shape == b.shape
            assert maxabs(a, b) <= TOL, call


def test_noalloc_ragged_random_stages_twice(gpu):
    rng = np.random.default_rng(12)
    st = _abi.stages(_abi.stage("rotate", random=True, lo=(-45,), hi=(45,)),
                     _abi.stage("gaussian", random=True, lo=(0.5,), hi=(4.0,)),
                     _abi.stage("adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
                     _abi.stage("transpose", probability=0.5),
                     _abi.stage("fliplr", probability=0.5))
    for call in range(2):
        xs = [rng.random((int(rng.integers(20, 300)), int(rng.integers(20, 300)), 3), dtype=np.float32)
              for _ in range(5)]
        ref, got = _run_both(st, 5, xs, 99 + call, 10 * call)
        for a, b in zip(ref, got):
            assert a.shape == b.shape
            assert maxabs(a, b) <= TOL, call


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
