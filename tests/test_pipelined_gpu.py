"""GPU: pipelined plans (mpk_tune_set_pipeline) -- chunks of a batch whose
stages run on two streams, the second stage of one chunk overlapping the
first stage of the next, intermediates rotating through three scratch slots
-- give the oracle's results, directly and replayed from a CUDA graph
captured on one stream."""
import ctypes as C
import math

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs
from test_pipeline_gpu import check_spec, dev_image, alloc_like, host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture
def pipelined():
    L = _abi.lib()
    _abi.check(L.mpk_tune_set_pipeline(2 << 20))     # 2 MB chunks: many chunks, every slot reused
    yield L
    _abi.check(L.mpk_tune_set_pipeline(0))


def test_uniform_and_ragged_chains(gpu, pipelined):
    rng = np.random.default_rng(61)
    uni = [dict(op="rgb2grey"), dict(op="gaussian", lo=(3.0,)), dict(op="rotate", lo=(17.0,)),
           dict(op="adjust_gamma", lo=(0.8, 1.0))]
    check_spec(uni, [rng.random((300, 280, 3), dtype=np.float32) for _ in range(9)])
    rag = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
           dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
           dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
           dict(op="brightness", random=True, lo=(-0.2,), hi=(0.2,)), dict(op="fliplr", probability=0.5)]
    xs = []
    for _ in range(30):
        h, w = (int(round(math.exp(rng.uniform(math.log(16), math.log(900))))) for _ in range(2))
        xs.append(rng.random((h, w, 3), dtype=np.float32))
    check_spec(rag, xs, seed=13)
    # three segments (rotate, gaussian, transpose) and mixed signatures
    three = [dict(op="rotate", lo=(20.0,)), dict(op="gaussian", lo=(1.2,)), dict(op="transpose"),
             dict(op="rotate", probability=0.5, lo=(-10.0,))]
    check_spec(three, [rng.random((120 + 7 * i, 90 + 5 * i, 3), dtype=np.float32) for i in range(12)], seed=4)


def test_graph_replay(gpu, pipelined):
    L = pipelined
    rng = np.random.default_rng(62)
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 2.0), _abi.stage("rotate", 33.0))
    xs = [rng.random((256, 256, 3), dtype=np.float32) for _ in range(12)]
    keep, ins = [], []
    for x in xs:
        t, m = dev_image(x)
        keep.append(t)
        ins.append(m)
    ia = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(st, 3, ia, outs, len(xs), 0, 0))
    ob = [alloc_like(outs[i]) for i in range(len(xs))]
    s = torch.cuda.Stream()
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(st, 3, ia, outs, len(xs), 0, 0, C.c_void_p(s.cuda_stream), C.byref(plan)))
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        _abi.check(L.mpk_plan_launch(plan, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    for _ in range(3):
        for t in ob:
            t.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        for i, x in enumerate(xs):
            ref = O.run_ops(x, [("rgb2grey",), ("gaussian", 2.0), ("rotate", 33.0)])
            assert maxabs(host(ob[i], outs[i]), ref) <= TOL
    _abi.check(L.mpk_plan_destroy(plan))
    torch.cuda.synchronize()
