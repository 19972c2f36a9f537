"""GPU parity of the fused gaussian -> rotate kernel (the blurred image kept
in shared memory, one launch): every case runs with fusion on and off and
both results are held to the FP64 oracle at 1e-5.  Cases: the uniform
batch's chain, 1- and 3-channel sources, every compiled radius, angles
including 0, +-45, 90, 180 and 271.3 degrees, a pointwise op between the blur
and the rotate (applied before the rotate's zero fill), epilogues and a
mirror after the rotate, images smaller than one 64 x 64 tile and odd
sizes, a ragged batch with per-image random parameters."""
import ctypes as C
import math

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs
from test_pipeline_gpu import check_spec, dev_image, alloc_like

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture
def fusion():
    L = _abi.lib()
    yield L
    _abi.check(L.mpk_tune_set_fuse(1))


def both(L, spec, xs, seed=0):
    outs = []
    for mode in (1, 0):
        _abi.check(L.mpk_tune_set_fuse(mode))
        outs.append(check_spec(spec, xs, seed=seed))
    return outs


def test_uniform_chain_fused_and_split(gpu, fusion):
    rng = np.random.default_rng(31)
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(3.0,)), dict(op="rotate", lo=(17.0,)),
            dict(op="adjust_gamma", lo=(0.8, 1.0))]
    xs = [rng.random((256, 320, 3), dtype=np.float32) for _ in range(3)]
    f, u = both(fusion, spec, xs)
    for a, b in zip(f, u):
        assert maxabs(a, b) <= 2 * TOL


def test_every_radius_and_angle(gpu, fusion):
    rng = np.random.default_rng(32)
    x3 = rng.random((150, 133, 3), dtype=np.float32)
    x1 = rng.random((97, 201), dtype=np.float32)
    for r in range(1, 13):
        sigma = r / 3.0 - 0.01
        for angle in (0.0, 45.0, -45.0, 90.0, 180.0, 271.3, 13.7):
            if (r + int(angle)) % 3:      # a third of the grid per source keeps the run short
                continue
            spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(sigma,)), dict(op="rotate", lo=(angle,))]
            both(fusion, spec, [x3])
            both(fusion, spec[1:], [x1])


def test_pointwise_between_blur_and_rotate_and_after(gpu, fusion):
    # brightness between the blur and the rotate must not leak into the
    # rotate's zero fill; gamma and a mirror after the rotate
    rng = np.random.default_rng(33)
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(2.2,)), dict(op="brightness", lo=(0.3,)),
            dict(op="rotate", lo=(31.0,)), dict(op="adjust_gamma", lo=(1.7, 0.9)), dict(op="fliplr")]
    xs = [rng.random((120, 170, 3), dtype=np.float32), rng.random((65, 63, 3), dtype=np.float32)]
    both(fusion, spec, xs)


def test_small_and_odd_images(gpu, fusion):
    rng = np.random.default_rng(34)
    spec = [dict(op="rgb2grey"), dict(op="gaussian", lo=(1.5,)), dict(op="rotate", lo=(-22.0,)),
            dict(op="brightness", lo=(-0.05,))]
    xs = [rng.random(s, dtype=np.float32) for s in [(1, 1, 3), (5, 3, 3), (63, 65, 3), (64, 64, 3), (65, 129, 3),
                                                     (700, 513, 3)]]
    both(fusion, spec, xs)


def test_ragged_random_parameters(gpu, fusion):
    rng = np.random.default_rng(35)
    spec = [dict(op="rgb2grey"), dict(op="gaussian", random=True, lo=(0.4,), hi=(4.0,)),
            dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)), dict(op="fliplr", probability=0.5)]
    xs = []
    for _ in range(20):
        h, w = (int(round(math.exp(rng.uniform(math.log(16), math.log(600))))) for _ in range(2))
        xs.append(rng.random((h, w, 3), dtype=np.float32))
    both(fusion, spec, xs, seed=77)


def test_fused_plan_is_one_launch(gpu, fusion):
    L = fusion
    rng = np.random.default_rng(36)
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 3.0), _abi.stage("rotate", 17.0),
                     _abi.stage("adjust_gamma", 0.8, 1.0))
    x = rng.random((200, 240, 3), dtype=np.float32)
    t, m = dev_image(x)
    ins = _abi.images([m])
    outs = _abi.images([_abi.MPImage()])
    _abi.check(L.mpk_pipeline_shapes(st, 4, ins, outs, 1, 0, 0))
    keep = alloc_like(outs[0])
    counts = []
    for mode in (1, 0):
        _abi.check(L.mpk_tune_set_fuse(mode))
        plan = C.c_void_p()
        _abi.check(L.mpk_plan_create(st, 4, ins, outs, 1, 0, 0, None, C.byref(plan)))
        counts.append(L.mpk_plan_num_launches(plan))
        kind = C.c_int()
        L.mpk_plan_launch_info(plan, 0, C.byref(kind), None, None, None)
        if mode == 1:
            assert kind.value == 9
        _abi.check(L.mpk_plan_destroy(plan))
    assert counts == [1, 2]
    torch.cuda.synchronize()
    del keep, t
