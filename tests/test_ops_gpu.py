"""GPU parity: every per-op entry point (mpimg_*) through the C-ABI against
the FP64 oracle, on seeded float32 inputs in [0,1], including sizes that do
not divide the tile shapes (tile-edge and halo cases)."""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs, obj_free, obj_from_host, obj_to_host, rand_image, run_op

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (1, 17), (3, 5), (63, 65), (1023, 1), (64, 64), (127, 200), (512, 512)]
CHANNELS = [1, 3, 4]


@pytest.fixture
def rng():
    return np.random.default_rng(20260303)


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("c", CHANNELS)
def test_transpose_bit_exact(gpu, rng, h, w, c):
    x = rand_image(rng, h, w, c)
    y = run_op(x, "mpimg_transpose")
    assert np.array_equal(y, O.transpose(x))


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("c", CHANNELS)
def test_fliplr_bit_exact(gpu, rng, h, w, c):
    x = rand_image(rng, h, w, c)
    y = run_op(x, "mpimg_fliplr")
    assert np.array_equal(y, O.fliplr(x))


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("c", [3, 4])
def test_rgb2grey(gpu, rng, h, w, c):
    x = rand_image(rng, h, w, c)
    y = run_op(x, "mpimg_color_to_greyscale")
    assert y.shape == (h, w)
    assert maxabs(y, O.rgb2grey(x)) <= TOL


def test_rgb2grey_of_grey_is_identity(gpu, rng):
    x = rand_image(rng, 9, 11, 1)
    assert np.array_equal(run_op(x, "mpimg_color_to_greyscale"), x)


@pytest.mark.parametrize("h,w", [(1, 1), (3, 5), (63, 65), (1023, 1), (1, 1023), (200, 300), (512, 512)])
@pytest.mark.parametrize("c", CHANNELS)
@pytest.mark.parametrize("sigma", [0.3, 1.0, 2.0, 3.0])
def test_gaussian(gpu, rng, h, w, c, sigma):
    x = rand_image(rng, h, w, c)
    y = run_op(x, "mpimg_gaussian", _abi.GaussianArgs(sigma))
    assert maxabs(y, O.gaussian(x, sigma)) <= TOL


@pytest.mark.parametrize("sigma", [4.0, 5.5, 8.0, 12.0, 16.0])
@pytest.mark.parametrize("c", [1, 3])
def test_gaussian_large_radius(gpu, rng, sigma, c):
    x = rand_image(rng, 150, 170, c)
    y = run_op(x, "mpimg_gaussian", _abi.GaussianArgs(sigma))
    assert maxabs(y, O.gaussian(x, sigma)) <= TOL


def test_gaussian_rejects_bad_sigma(gpu, rng):
    L = _abi.lib()
    x = rand_image(rng, 8, 8, 1)
    o = obj_from_host(x)
    try:
        assert L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(0.0))) == _abi.MP_ERROR_INVALID_ARGS
        assert L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(20.0))) == _abi.MP_ERROR_TOO_LARGE
        assert np.array_equal(obj_to_host(o), x)   # failed calls leave the image untouched
    finally:
        obj_free(o)


@pytest.mark.parametrize("h,w", [(1, 1), (3, 5), (63, 65), (64, 64), (127, 200), (512, 512)])
@pytest.mark.parametrize("c", CHANNELS)
@pytest.mark.parametrize("angle", [0.0, 17.0, 30.0, -45.0, 90.0, 180.0, 271.3])
def test_rotate(gpu, rng, h, w, c, angle):
    x = rand_image(rng, h, w, c)
    y = run_op(x, "mpimg_rotate", _abi.RotateArgs(angle))
    assert maxabs(y, O.rotate(x, angle)) <= TOL


def test_rotate_large_image_coordinates(gpu, rng):
    # 4096-wide rows: the fixed-point source coordinates must keep the
    # bilinear fractions accurate far from the centre.
    x = rand_image(rng, 64, 4096, 1)
    y = run_op(x, "mpimg_rotate", _abi.RotateArgs(0.37))
    assert maxabs(y, O.rotate(x, 0.37)) <= TOL


@pytest.mark.parametrize("c", CHANNELS)
@pytest.mark.parametrize("delta", [-0.99, -0.2, 0.1, 0.5])
def test_brightness(gpu, rng, c, delta):
    x = rand_image(rng, 37, 41, c)
    y = run_op(x, "mpimg_brightness", _abi.BrightnessArgs(delta))
    assert maxabs(y, O.brightness(x, delta)) <= TOL


@pytest.mark.parametrize("c", CHANNELS)
@pytest.mark.parametrize("gamma,gain", [(2.2, 1.0), (0.8, 1.0), (0.5, 1.3), (1.0, 0.5)])
def test_adjust_gamma(gpu, rng, c, gamma, gain):
    x = rand_image(rng, 37, 41, c)
    x[0, 0] = 0.0
    y = run_op(x, "mpimg_adjust_gamma", _abi.GammaArgs(gamma, gain))
    assert maxabs(y, O.adjust_gamma(x, gamma, gain)) <= TOL


@pytest.mark.parametrize("c", CHANNELS)
def test_colorize(gpu, rng, c):
    x = rand_image(rng, 19, 23, c)
    y = run_op(x, "mpimg_colorize", _abi.ColorizeArgs(1.5, 0.5, 2.0))
    assert maxabs(y, O.colorize(x, 1.5, 0.5, 2.0)) <= TOL


def test_zero_size_images(gpu):
    for shape in [(0, 5), (4, 0), (0, 0, 3)]:
        x = np.zeros(shape, dtype=np.float32)
        for fn, args in [("mpimg_fliplr", None), ("mpimg_transpose", None),
                         ("mpimg_gaussian", _abi.GaussianArgs(1.0)), ("mpimg_rotate", _abi.RotateArgs(10.0)),
                         ("mpimg_brightness", _abi.BrightnessArgs(0.1))]:
            y = run_op(x, fn, args)
            assert y.size == 0


def test_unsupported_dtype_is_an_error_not_a_noop(gpu):
    L = _abi.lib()
    x = np.ones((4, 4, 3), dtype=np.int16)
    o = obj_from_host(x)
    try:
        assert L.mpimg_rotate(C.byref(o), C.byref(_abi.RotateArgs(10.0))) == _abi.MP_ERROR_UNSUPPORTED_TYPE
    finally:
        obj_free(o)


def test_sequence_of_ops_matches_oracle(gpu, rng):
    """The reference's long-pipeline sequence (tests/millipyde_tests.py:349-395)."""
    L = _abi.lib()
    x = rand_image(rng, 97, 131, 3)
    o = obj_from_host(x)
    try:
        _abi.check(L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(2.0))))
        _abi.check(L.mpimg_color_to_greyscale(C.byref(o), None))
        _abi.check(L.mpimg_transpose(C.byref(o), None))
        _abi.check(L.mpimg_transpose(C.byref(o), None))
        _abi.check(L.mpimg_rotate(C.byref(o), C.byref(_abi.RotateArgs(45.0))))
        y = obj_to_host(o)
    finally:
        obj_free(o)
    ref = O.run_ops(x, [("gaussian", 2.0), ("rgb2grey",), ("transpose",), ("transpose",), ("rotate", 45.0)])
    assert maxabs(y, ref) <= TOL
