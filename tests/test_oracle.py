"""CPU: the FP64 oracle against independent witnesses (scipy.ndimage) and
size-independent properties.  Golden vectors from the reference's own
kernels are checked in test_golden.py."""
import math

import numpy as np
import pytest
from scipy import ndimage

from oracle import oracle as O


@pytest.fixture
def rng():
    return np.random.default_rng(1234)


@pytest.mark.parametrize("sigma", [0.5, 1.0, 2.0, 3.0, 4.0, 8.0])
def test_gaussian_matches_scipy_correlate1d(rng, sigma):
    x = rng.random((37, 53))
    r = O.gaussian_radius(sigma)
    w = O.gaussian_weights(sigma, r)
    ref = ndimage.correlate1d(ndimage.correlate1d(x, w, axis=0, mode="constant", cval=0.0),
                              w, axis=1, mode="constant", cval=0.0)
    assert np.max(np.abs(O.gaussian(x, sigma) - ref)) < 1e-13


def test_gaussian_radius_rule():
    assert O.gaussian_radius(2) == 6 and O.gaussian_radius(3) == 9 and O.gaussian_radius(8) == 24
    assert O.gaussian_radius(0.5) == 2 and O.gaussian_radius(4) == 12


def test_gaussian_weights_normalised_symmetric():
    for s in (0.5, 1.7, 3, 8):
        w = O.gaussian_weights(s, O.gaussian_radius(s))
        assert abs(w.sum() - 1) < 1e-15
        assert np.array_equal(w, w[::-1])


def test_gaussian_rgb_is_per_channel(rng):
    x = rng.random((20, 30, 3))
    y = O.gaussian(x, 1.5)
    for c in range(3):
        assert np.allclose(y[..., c], O.gaussian(x[..., c], 1.5), atol=1e-15)


@pytest.mark.parametrize("angle", [0.0, 17.0, 30.0, -45.0, 90.0, 123.4])
def test_rotate_bilinear_matches_map_coordinates(rng, angle):
    h, w = 41, 58
    x = rng.random((h, w))
    sx, sy = O.rotate_source_coords(h, w, angle)
    ref = ndimage.map_coordinates(x, [sy, sx], order=1, mode="grid-constant", cval=0.0)
    assert np.max(np.abs(O.rotate(x, angle) - ref)) < 1e-12


def test_rotate_zero_is_identity(rng):
    x = rng.random((16, 24, 3))
    assert np.allclose(O.rotate(x, 0.0), x, atol=1e-15)


def test_rotate_180_even_sizes_is_exact_flip(rng):
    # centre (W/2, H/2) on even sizes maps p -> W - p: a flip shifted by one
    x = rng.random((8, 10))
    y = O.rotate(x, 180.0)
    assert np.allclose(y[1:, 1:], x[::-1, ::-1][:-1, :-1], atol=1e-9)


def test_rotate_nearest_truncates_toward_zero():
    x = np.arange(12, dtype=np.float64).reshape(3, 4)
    y = O.rotate(x, 0.0, mode="nearest")
    assert np.array_equal(y, x)


def test_grey_weights_and_clamp(rng):
    x = rng.random((5, 7, 3))
    g = O.rgb2grey(x)
    assert np.allclose(g, 0.2125 * x[..., 0] + 0.7154 * x[..., 1] + 0.0721 * x[..., 2])
    assert O.rgb2grey(np.ones((2, 2, 3))).max() <= 1.0
    rgba = np.concatenate([x, rng.random((5, 7, 1))], axis=2)
    assert np.array_equal(O.rgb2grey(rgba), g)


def test_pointwise_keep_alpha(rng):
    x = rng.random((4, 4, 4))
    for y in (O.brightness(x, 0.3), O.adjust_gamma(x, 2.2), O.colorize(x, 1.5, 0.5, 2.0)):
        assert np.array_equal(y[..., 3], x[..., 3])
        assert y.min() >= 0 and y.max() <= 1


def test_transpose_fliplr_exact(rng):
    x = rng.random((7, 9, 3)).astype(np.float32)
    assert np.array_equal(O.transpose(x), np.transpose(x, (1, 0, 2)))
    assert np.array_equal(O.fliplr(x), x[:, ::-1])
    assert np.array_equal(O.fliplr(O.fliplr(x)), x)


def test_gaussian_linearity(rng):
    a, b = rng.random((23, 31)), rng.random((23, 31))
    assert np.allclose(O.gaussian(2 * a + 3 * b, 2.0), 2 * O.gaussian(a, 2.0) + 3 * O.gaussian(b, 2.0))


def test_counter_uniform_range_and_determinism():
    u = [O.counter_uniform(7, i, 2, 1) for i in range(2000)]
    assert all(0.0 <= v < 1.0 for v in u)
    assert abs(np.mean(u) - 0.5) < 0.03
    assert u == [O.counter_uniform(7, i, 2, 1) for i in range(2000)]
    assert O.counter_uniform(7, 0, 2, 1) != O.counter_uniform(8, 0, 2, 1)


def test_gaussian_rotate_window_equals_whole_image():
    """The windowed oracle (used for the 8192^2 parity case) reproduces the
    whole-image oracle on every window, edges and corners included."""
    rng = np.random.default_rng(5)
    for shape, sigma, angle in [((150, 170, 3), 2.0, 37.0), ((97, 61), 1.2, -44.0), ((64, 200, 3), 4.0, 90.0)]:
        x = rng.random(shape)
        full = O.rotate(O.gaussian(x, sigma), angle)
        h, w = shape[:2]
        for rows, cols in [((0, 20), (0, 30)), ((h // 3, h // 2), (w // 4, w // 2)), ((h - 9, h), (w - 13, w)),
                           ((0, h), (w - 3, w))]:
            win = O.gaussian_rotate_window(x, sigma, angle, rows, cols)
            assert np.abs(win - full[rows[0]:rows[1], cols[0]:cols[1]]).max() <= 1e-12
