"""GPU: the host-buffer batch entry (mpk_pipeline_run_host) -- copies in,
kernels, copies out, chunked and overlapped on three streams -- returns the
device path's results for every host layout: packed rows whose width makes
the device pitch differ (a 1-D landing copy re-pitched on the device),
packed rows equal to the device pitch (one copy), padded host rows (2-D
copies), pageable and page-locked memory, several chunks, empty images."""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi

from helpers import TOL, maxabs
from test_pipeline_gpu import run_batch, oracle_batch, to_stage

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SPEC = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
        dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
        dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
        dict(op="fliplr", probability=0.5)]


def _host_images(xs, pad, pinned):
    keep, ims = [], []
    for x in xs:
        h, w, c = x.shape
        p = w * c * 4 + pad
        t = torch.zeros((h, p // 4), dtype=torch.float32)
        if pinned:
            t = t.pin_memory()
        t[:, : w * c] = torch.from_numpy(x.reshape(h, w * c))
        keep.append(t)
        ims.append(_abi.image(t.data_ptr(), h, w, c, p))
    return keep, ims


@pytest.mark.parametrize("pad,pinned", [(0, True), (0, False), (16, True)])
def test_host_path_matches_device_path(gpu, pad, pinned):
    L = _abi.lib()
    rng = np.random.default_rng(51 + pad)
    shapes = [(2048, 2048), (2048, 2047), (1500, 37), (37, 1500), (300, 301), (64, 64), (0, 5),
              (777, 1999), (1800, 2044), (1600, 1601), (1, 1), (2048, 1024)]
    xs = [rng.random((h, w, 3), dtype=np.float32) for h, w in shapes]
    stages = _abi.stages(*[to_stage(d) for d in SPEC])
    kin, ins = _host_images(xs, pad, pinned)
    ia = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(stages, len(SPEC), ia, outs, len(xs), 9, 0))
    kout = []
    for i in range(len(xs)):
        m = outs[i]
        p = m.width * m.channels * 4 + pad
        t = torch.full((max(1, m.height), max(1, p // 4)), float("nan"), dtype=torch.float32)
        if pinned:
            t = t.pin_memory()
        kout.append(t)
        m.data = t.data_ptr()
        m.pitch = p
        outs[i] = m
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):   # twice: slots and landing buffers reused
        _abi.check(L.mpk_pipeline_run_host(stages, len(SPEC), ia, outs, len(xs), 9, 0, stream))
    dev = run_batch([to_stage(d) for d in SPEC], xs, seed=9, index0=0)
    for i, x in enumerate(xs):
        h, w = x.shape[:2]
        got = kout[i][:h, : w * 3].numpy().reshape(h, w, 3)
        assert maxabs(got, dev[i]) <= 1e-6, i
    # image i of the batch draws its parameters with index i
    ref = [oracle_batch(SPEC, [xs[i]], seed=9, index0=i)[0] for i in (2, 4, 7)]
    for r, i in zip(ref, (2, 4, 7)):
        h, w = xs[i].shape[:2]
        assert maxabs(kout[i][:h, : w * 3].numpy().reshape(h, w, 3), r) <= TOL
