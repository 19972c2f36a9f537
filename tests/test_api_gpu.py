"""GPU: the Python API (CPython extension) -- the reference's own test cases
in spirit (tests/millipyde_tests.py) on seeded synthetic images, checked
against the FP64 oracle."""
import numpy as np
import numpy.testing as npt
import pytest

import millipyde_gb300 as mp
from oracle import oracle as O

from helpers import TOL, maxabs

pytestmark = pytest.mark.gpu


@pytest.fixture
def rng():
    return np.random.default_rng(99)


def img(rng, h=61, w=83, c=3):
    return rng.random((h, w, c) if c > 1 else (h, w), dtype=np.float32)


def test_create_gpuarray_roundtrips(gpu):
    a = np.array([1, 2, 3, 4])
    assert np.array_equal(np.array(mp.gpuarray(a)), a)
    assert np.array_equal(np.array(mp.gpuarray([1, 2, 3, 4])), a)
    assert not np.array_equal(np.array(mp.gpuarray([4, 3, 2, 1])), a)
    with pytest.raises(ValueError):
        mp.gpuarray(None)
    with pytest.raises(TypeError):
        mp.gpuarray()


def test_create_gpuimage_roundtrips(gpu):
    for a in (np.array([[1, 2, 3, 4], [4, 5, 6, 7]]),
              np.array([[[1, 2, 3], [4, 5, 6]], [[1, 2, 3], [4, 5, 6]]]),
              np.arange(7 * 5 * 4, dtype=np.uint8).reshape(7, 5, 4),
              np.random.default_rng(0).random((13, 9, 3))):
        g = mp.gpuimage(a)
        assert np.array_equal(np.array(g), a)
        assert g.shape == a.shape and g.dtype == a.dtype
    with pytest.raises(ValueError):
        mp.gpuimage(np.array([1, 2, 3, 4]))
    with pytest.raises(ValueError):
        mp.gpuimage(np.zeros((2, 2, 2, 2)))


def test_numpy_protocols(gpu):
    lst = [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    npt.assert_equal(np.transpose(np.array(lst)), np.transpose(mp.gpuarray(lst)))
    npt.assert_equal(np.transpose(np.array(lst)), np.transpose(mp.gpuimage(lst)))
    npt.assert_equal(np.add(mp.gpuarray(lst), 1), np.array(lst) + 1)
    npt.assert_equal(np.concatenate([mp.gpuarray([1, 2]), mp.gpuarray([3])]), [1, 2, 3])


def test_methods_match_oracle(gpu, rng):
    x = img(rng)
    cases = [
        (lambda g: g.rgb2grey(), lambda a: O.rgb2grey(a)),
        (lambda g: g.rgb2gray(), lambda a: O.rgb2grey(a)),
        (lambda g: g.transpose(), lambda a: O.transpose(a)),
        (lambda g: g.fliplr(), lambda a: O.fliplr(a)),
        (lambda g: g.gaussian(2), lambda a: O.gaussian(a, 2)),
        (lambda g: g.rotate(30), lambda a: O.rotate(a, 30)),
        (lambda g: g.adjust_gamma(2.2), lambda a: O.adjust_gamma(a, 2.2)),
        (lambda g: g.adjust_gamma(2, 1), lambda a: O.adjust_gamma(a, 2, 1)),
        (lambda g: g.brightness(0.1), lambda a: O.brightness(a, 0.1)),
        (lambda g: g.colorize(1.2, 0.8, 1.0), lambda a: O.colorize(a, 1.2, 0.8, 1.0)),
    ]
    for fn, ref in cases:
        g = mp.gpuimage(x)
        assert fn(g) is None
        assert maxabs(np.array(g), ref(x)) <= TOL


def test_grey_and_transpose(gpu, rng):
    x = img(rng)
    g = mp.gpuimage(x)
    g.rgb2grey()
    g.transpose()
    assert (g.height, g.width) == (x.shape[1], x.shape[0])
    assert maxabs(np.array(g), np.transpose(O.rgb2grey(x))) <= TOL


def test_brightness_range_check(gpu, rng):
    g = mp.gpuimage(img(rng))
    with pytest.raises(ValueError):
        g.brightness(1.0)
    with pytest.raises(ValueError):
        g.gaussian(0)


def test_unsupported_dtype_raises(gpu):
    g = mp.gpuimage(np.ones((4, 4, 3), dtype=np.int16))
    with pytest.raises(TypeError):
        g.rotate(10)


def test_random_methods_in_range(gpu, rng):
    x = img(rng, 40, 50, 3)
    mp.seed(5)
    for call in (lambda g: g.random_rotate(-10, 10), lambda g: g.random_gaussian(0.5, 2),
                 lambda g: g.random_brightness(-0.2, 0.2), lambda g: g.random_adjust_gamma([0.5, 2], [1, 1]),
                 lambda g: g.random_adjust_gamma(0.5, 2.0), lambda g: g.random_colorize([0.5, 1.5], [0.5, 1.5], [0.5, 1.5])):
        g = mp.gpuimage(x)
        assert call(g) is None
        y = np.array(g)
        assert y.shape == x.shape and np.all(y >= 0) and np.all(y <= 1)


def test_operation_run_on(gpu, rng):
    x = img(rng)
    g = mp.gpuimage(x)
    for op in [mp.Operation("rgb2grey"), mp.Operation("transpose")]:
        op.run_on(g)
    assert maxabs(np.array(g), O.transpose(O.rgb2grey(x))) <= TOL


def test_clone_is_independent(gpu, rng):
    x = img(rng)
    g = mp.gpuimage(x)
    c = g.clone()
    c.rgb2grey()
    assert np.array_equal(np.array(g), x)
    assert maxabs(np.array(c), O.rgb2grey(x)) <= TOL
    a = mp.gpuarray(np.array([[1, 2, 3], [4, 5, 6]]))
    assert np.array_equal(np.array(a.clone()), np.array(a))


def test_long_pipeline_equals_sequential_methods(gpu, rng):
    """tests/millipyde_tests.py:349-395 on 8 images."""
    x = img(rng, 120, 140, 3)
    control = mp.gpuimage(x)
    control.gaussian(2)
    control.rgb2grey()
    control.transpose()
    control.transpose()
    control.rotate(45)
    control = np.array(control)
    ims = [mp.gpuimage(x) for _ in range(8)]
    ops = [mp.Operation("gaussian", 2), mp.Operation("rgb2grey"), mp.Operation("transpose"),
           mp.Operation("transpose"), mp.Operation("rotate", 45)]
    mp.Pipeline(ims, ops).run()
    ref = O.run_ops(x, [("gaussian", 2), ("rgb2grey",), ("transpose",), ("transpose",), ("rotate", 45)])
    for g in ims:
        y = np.array(g)
        assert maxabs(y, control) <= TOL
        assert maxabs(y, ref) <= TOL


def test_pipeline_run_unfused_and_fused_agree(gpu, rng):
    xs = [img(rng, 50 + 3 * i, 70 - 2 * i, 3) for i in range(6)]
    ops = [mp.Operation("rgb2grey"), mp.Operation("gaussian", 3), mp.Operation("rotate", 17),
           mp.Operation("adjust_gamma", 0.8)]
    a = [mp.gpuimage(x) for x in xs]
    b = [mp.gpuimage(x) for x in xs]
    mp.Pipeline(a, ops).run()
    mp.Pipeline(b, ops).run_unfused()
    for ga, gb, x in zip(a, b, xs):
        ref = O.run_ops(x, [("rgb2grey",), ("gaussian", 3), ("rotate", 17), ("adjust_gamma", 0.8)])
        assert maxabs(np.array(ga), ref) <= TOL
        assert maxabs(np.array(gb), ref) <= TOL


def test_pipeline_same_image_twice_applies_twice(gpu, rng):
    x = img(rng, 20, 24, 1)
    g = mp.gpuimage(x)
    mp.Pipeline([g, g], [mp.Operation("fliplr"), mp.Operation("brightness", 0.1)]).run()
    ref = O.brightness(O.fliplr(O.brightness(O.fliplr(x), 0.1)), 0.1)
    assert maxabs(np.array(g), ref) <= TOL


def test_pipeline_connect_to(gpu, rng):
    x = img(rng)
    g = mp.gpuimage(x)
    p1 = mp.Pipeline([g], [mp.Operation("rgb2grey")])
    p2 = mp.Pipeline([], [mp.Operation("transpose")])
    p1.connect_to(p2)
    p1.run()
    assert maxabs(np.array(g), O.transpose(O.rgb2grey(x))) <= TOL


def test_pipeline_seeded_random_is_reproducible(gpu, rng):
    x = img(rng, 48, 40, 3)
    ops = [mp.Operation("random_rotate", -45, 45), mp.Operation("random_gaussian", 0.5, 4),
           mp.Operation("fliplr", probability=0.5)]
    a = [mp.gpuimage(x) for _ in range(4)]
    b = [mp.gpuimage(x) for _ in range(4)]
    mp.Pipeline(a, ops, seed=42).run()
    mp.Pipeline(b, ops, seed=42).run()
    for ga, gb in zip(a, b):
        assert np.array_equal(np.array(ga), np.array(gb))


def test_generator_order_and_outputs(gpu, rng):
    xs = [img(rng, 20 + i, 30, 3) for i in range(3)]
    ins = [mp.gpuimage(x) for x in xs]
    g = mp.Generator(ins, [mp.Operation("rgb2grey")])
    for i in range(7):
        out = next(g)
        assert maxabs(np.array(out), O.rgb2grey(xs[i % 3])) <= TOL
    g = mp.Generator(ins, [mp.Operation("rgb2grey")], return_to_host=True, outputs=4)
    outs = list(g)
    assert len(outs) == 4 and isinstance(outs[0], np.ndarray)
    assert maxabs(outs[3], O.rgb2grey(xs[0])) <= TOL
    for x, h in zip(xs, ins):
        assert np.array_equal(np.array(h), x)   # inputs untouched


def test_generator_seeded_matches_oracle(gpu, rng):
    xs = [img(rng, 33 + 5 * i, 41 - 2 * i, 3) for i in range(3)]
    ins = [mp.gpuimage(x) for x in xs]
    ops = [mp.Operation("random_rotate", -45, 45), mp.Operation("random_gaussian", 0.5, 4),
           mp.Operation("random_adjust_gamma", 0.5, 2.0), mp.Operation("random_brightness", -0.2, 0.2),
           mp.Operation("fliplr", probability=0.5)]
    spec = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="gaussian", random=True, lo=(0.5,), hi=(4,)),
            dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
            dict(op="brightness", random=True, lo=(-0.2,), hi=(0.2,)),
            dict(op="fliplr", probability=0.5)]
    g = mp.Generator(ins, ops, seed=2024, outputs=10, return_to_host=True)
    outs = list(g)
    assert len(outs) == 10
    for i, out in enumerate(outs):
        opl = []
        for s, d in enumerate(spec):
            run, p = O.resolve_stage(d, 2024, i, s)
            if run:
                nargs = {"gaussian": 1, "rotate": 1, "brightness": 1, "adjust_gamma": 2}.get(d["op"], 0)
                opl.append((d["op"],) + tuple(p[:nargs]))
        assert maxabs(out, O.run_ops(xs[i % 3], opl)) <= TOL


def test_generator_with_python_callable_uses_reference_path(gpu, rng):
    calls = []
    x = img(rng, 10, 12, 3)
    g = mp.Generator([mp.gpuimage(x)], [mp.Operation(lambda: calls.append(1)), mp.Operation("fliplr")],
                     outputs=3)
    outs = list(g)
    assert len(outs) == 3 and len(calls) == 3
    assert np.array_equal(np.array(outs[0]), O.fliplr(x))


def test_device_context(gpu):
    with mp.Device(0) as d:
        assert d == 0
        assert mp.get_current_device() == 0
        a = mp.gpuarray([1.0, 2.0])
    assert np.array_equal(np.array(a), [1.0, 2.0])
    with pytest.raises(ValueError):
        with mp.Device(99):
            pass
    with pytest.raises(KeyError):
        with mp.Device(0):
            raise KeyError("propagates")
