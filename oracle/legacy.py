"""CPU restatement of the reference's uint8-RGBA / float64-greyscale kernels
-- TEST INFRASTRUCTURE ONLY (never imported by the product).

These are the reference's exact per-pixel formulas for its two native
layouts (src/millipyde_image.cpp:50-524): packed little-endian RGBA bytes and
float64 greyscale, including the truncations and byte-lane quirks of its RGBA
gaussian.  They are pinned against outputs of the reference's own kernels
(tests/golden/reference_ops.npz, test_golden.py), and are the oracle of the
library's legacy path.

Single-precision library calls the reference makes (expf for the gaussian
weights, powf for gamma) are taken from the C math library via ctypes, so the
restatement reproduces the reference's rounding.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

from . import oracle as O

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.expf.restype = ctypes.c_float
_libm.expf.argtypes = [ctypes.c_float]
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]

KERNEL_RADIUS = 8          # src/include/millipyde_image.h:11


def gaussian_weights(sigma, radius=KERNEL_RADIUS):
    """d_kernel as the host builds it: expf of a double argument converted to
    float, normalised in double (src/millipyde_image.cpp:745-756)."""
    e = np.array([_libm.expf(-1.0 * ((d * d) / (2.0 * sigma * sigma)))
                  for d in range(-radius, radius + 1)], dtype=np.float64)
    return e / e.sum()


def _powf(x, g):
    f = np.frompyfunc(lambda v: _libm.powf(float(v), float(g)), 1, 1)
    return f(np.asarray(x)).astype(np.float64)


# ---------------------------------------------------------------- greyscale
def rgb2grey(img):
    """uint8 (H, W, C>=3) -> float64: fmin(1, (0.2125 r + 0.7154 g + 0.0721 b) / 255)
    (src/millipyde_image.cpp:50-66)."""
    x = np.asarray(img).astype(np.float64)
    return np.minimum(1.0, (0.2125 * x[..., 0] + 0.7154 * x[..., 1] + 0.0721 * x[..., 2]) / 255)


def gaussian_grey(x, sigma):
    """Row pass then column pass with fmax(0, .), radius 8, zero padding
    (src/millipyde_image.cpp:146-244)."""
    w = gaussian_weights(sigma)
    x = np.asarray(x, dtype=np.float64)
    r = KERNEL_RADIUS
    h, wd = x.shape
    rowp = np.pad(x, ((0, 0), (r, r)))
    t = np.zeros_like(x)
    for i in range(2 * r + 1):   # sum += data[pos + k] * d_kernel[R - k], k = -R..R
        k = i - r
        t += rowp[:, r + k: r + k + wd] * w[r - k]
    colp = np.pad(t, ((r, r), (0, 0)))
    out = np.zeros_like(x)
    for i in range(2 * r + 1):
        k = i - r
        out += colp[r + k: r + k + h, :] * w[r - k]
    return np.maximum(0.0, out)


def brightness_grey(x, delta):
    """clamp01(x + delta)  (src/millipyde_image.cpp:384-398)."""
    return np.clip(np.asarray(x, dtype=np.float64) + delta, 0.0, 1.0)


def gamma_grey(x, gamma, gain):
    """clamp01(gain * powf(x, gamma)) with single-precision powf
    (src/millipyde_image.cpp:438-454)."""
    return np.clip(gain * _powf(x, gamma), 0.0, 1.0)


# ---------------------------------------------------------------- RGBA bytes
def _char(v):
    """C conversion of a double to (signed) char on the reference's x86 host:
    truncation toward zero, then two's-complement wrap."""
    i = int(math.trunc(v)) & 0xFF
    return i - 256 if i >= 128 else i


def brightness_rgba(img, delta):
    """Per colour byte: saturating add of char(delta*255); alpha kept
    (src/millipyde_image.cpp:401-435, :613)."""
    d = _char(delta * 255)
    x = np.asarray(img).astype(np.int32)
    out = x.copy()
    if d > 0:
        out[..., :3] = np.minimum(255, x[..., :3] + d)
    else:
        out[..., :3] = np.maximum(0, x[..., :3] + d)
    return out.astype(np.uint8)


def gamma_rgba(img, gamma, gain):
    """Per colour byte: gain * 255 * powf(b/255, gamma), clamped, truncated
    to a byte; alpha kept (src/millipyde_image.cpp:457-491)."""
    x = np.asarray(img)
    out = x.copy()
    t = gain * (255.0 * _powf(x[..., :3].astype(np.float64) / 255, gamma))
    t = np.where(t < 0, 0.0, t)
    out[..., :3] = np.where(t > 255, 255, np.trunc(t)).astype(np.uint8)
    return out


def colorize_rgba(img, r_mult, g_mult, b_mult):
    """Per colour byte: min(255, trunc(b * mult)); alpha kept
    (src/millipyde_image.cpp:494-524)."""
    x = np.asarray(img)
    out = x.copy()
    for k, m in enumerate((r_mult, g_mult, b_mult)):
        t = x[..., k].astype(np.float64) * m
        out[..., k] = np.where(t > 255, 255, np.trunc(t)).astype(np.uint8)
    return out


def gaussian_rgba(img, sigma):
    """The reference's packed-byte gaussian (src/millipyde_image.cpp:247-381):
    each byte lane is summed separately, every tap product truncated to int
    before summing and the sum kept modulo 256; the column pass forces the
    top byte (alpha, channel 3) to 0xff.  Zero padding at the borders."""
    w = gaussian_weights(sigma)
    x = np.asarray(img).astype(np.int64)
    h, wd, _ = x.shape
    r = KERNEL_RADIUS

    def lane_pass(a, axis):
        pad = [(0, 0)] * 3
        pad[axis] = (r, r)
        ap = np.pad(a, pad)
        n = a.shape[axis]
        acc = np.zeros_like(a)
        for i in range(2 * r + 1):
            k = i - r
            sl = [slice(None)] * 3
            sl[axis] = slice(r + k, r + k + n)
            acc += np.trunc(ap[tuple(sl)] * w[r - k]).astype(np.int64)
        return acc & 0xFF

    t = lane_pass(x, 1)
    out = lane_pass(t, 0)
    out[..., 3] = 0xFF
    return out.astype(np.uint8)


def rotate_nearest(img, angle):
    """Nearest-by-truncation rotation of any layout (src/millipyde_image.cpp:114-139)."""
    y = O.rotate(np.asarray(img).astype(np.float64), angle, mode="nearest")
    return y.astype(np.asarray(img).dtype)


def apply(op, x, params):
    """Reference op on its native layouts: uint8 RGBA (H, W, 4) or float64 (H, W)."""
    x = np.asarray(x)
    rgba = x.ndim == 3
    if op == "rgb2grey":
        return rgb2grey(x)
    if op == "transpose":
        return O.transpose(x)
    if op == "fliplr":
        return O.fliplr(x)
    if op == "rotate":
        return rotate_nearest(x, params[0])
    if op == "gaussian":
        return gaussian_rgba(x, params[0]) if rgba else gaussian_grey(x, params[0])
    if op == "brightness":
        return brightness_rgba(x, params[0]) if rgba else brightness_grey(x, params[0])
    if op == "adjust_gamma":
        return gamma_rgba(x, params[0], params[1]) if rgba else gamma_grey(x, params[0], params[1])
    if op == "colorize":
        return colorize_rgba(x, *params[:3]) if rgba else x
    raise ValueError(op)
