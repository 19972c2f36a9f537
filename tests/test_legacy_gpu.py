"""GPU: the reference's own layouts through the C-ABI -- uint8 RGBA (and
uint8 RGB for rgb2grey) and float64 greyscale -- against golden vectors made
by the reference's kernels (tests/golden/reference_ops.npz): bit-exact for
byte outputs, 1e-12 for float64 outputs (1e-6 where the reference calls the
single-precision powf, whose last bit differs between math libraries)."""
import os

import numpy as np
import pytest

import millipyde_gb300 as mp
from millipyde_gb300 import _abi
from oracle import legacy as LG

from helpers import run_op

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_ops.npz")
FN = {"rgb2grey": ("mpimg_color_to_greyscale", None), "transpose": ("mpimg_transpose", None),
      "fliplr": ("mpimg_fliplr", None), "rotate": ("mpimg_rotate", lambda p: _abi.RotateArgs(p[0])),
      "gaussian": ("mpimg_gaussian", lambda p: _abi.GaussianArgs(p[0])),
      "brightness": ("mpimg_brightness", lambda p: _abi.BrightnessArgs(p[0])),
      "adjust_gamma": ("mpimg_adjust_gamma", lambda p: _abi.GammaArgs(p[0], p[1])),
      "colorize": ("mpimg_colorize", lambda p: _abi.ColorizeArgs(p[0], p[1], p[2]))}


def _cases():
    z = np.load(GOLD)
    names = sorted({k.split("__")[0] for k in z.files})
    return {n: (str(z[n + "__op"]), z[n + "__in"], z[n + "__params"], z[n + "__out"]) for n in names}


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_legacy_matches_reference_kernels(gpu, name):
    op, x, p, y = CASES[name]
    fn, mk = FN[op]
    got = run_op(x, fn, mk(p) if mk else None)
    assert got.shape == y.shape and got.dtype == y.dtype
    if y.dtype == np.uint8:
        assert np.array_equal(got, y), np.argwhere(got != y)[:5]
    else:
        tol = 1e-6 if op == "adjust_gamma" else 1e-12
        assert np.max(np.abs(got - y)) <= tol


def test_legacy_python_api_and_pipeline(gpu):
    rng = np.random.default_rng(5)
    rgba = rng.integers(0, 256, size=(40, 64, 4), dtype=np.uint8)
    g = mp.gpuimage(rgba)
    g.gaussian(2)
    g.rgb2grey()
    g.transpose()
    g.rotate(30)
    ref = LG.rotate_nearest(LG.apply("transpose", LG.rgb2grey(LG.gaussian_rgba(rgba, 2.0)), ()), 30.0)
    out = np.array(g)
    assert out.dtype == np.float64 and out.shape == ref.shape
    assert np.max(np.abs(out - ref)) <= 1e-12
    ims = [mp.gpuimage(rgba) for _ in range(3)]
    mp.Pipeline(ims, [mp.Operation("adjust_gamma", 2, 1), mp.Operation("fliplr"),
                      mp.Operation("brightness", 0.1)]).run()
    ref2 = LG.brightness_rgba(LG.apply("fliplr", LG.gamma_rgba(rgba, 2.0, 1.0), ()), 0.1)
    for im in ims:
        assert np.array_equal(np.array(im), ref2)


def test_legacy_rejects_layouts_the_reference_did_not_handle(gpu):
    g = mp.gpuimage(np.zeros((4, 5, 3), dtype=np.uint8))
    with pytest.raises(TypeError):
        g.rotate(10)
    g.rgb2grey()                       # uint8 RGB -> float64 grey is handled
    assert np.array(g).dtype == np.float64
