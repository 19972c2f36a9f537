"""FP64 CPU oracle of millipyde's image hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker the GPU kernels are compared against.  Only the
tests, the smoke check and bench.py's CPU-baseline / reference legs may import
it; the product (millipyde_gb300) never does, and has no CPU fallback.

Each function restates the reference's per-pixel formula in float64 numpy,
citing the reference file:line it follows (paths within jasbury1/millipyde).
Where the build's float32 semantics differ from the reference's uint8/FP64
kernels (bilinear rotate, radius ceil(3*sigma)), the function takes a
parameter that selects the reference behaviour too, so the shared parts
(weights, padding, geometry, centre) can be pinned against outputs of the
reference's own kernels (tests/golden/, generated by oracle/ref_golden.py).

Layout: images are (H, W) greyscale or (H, W, C) interleaved, C in {1,3,4};
channel 3 of a 4-channel image is alpha and is left unchanged by the colour
ops, as in the reference's RGBA kernels.
"""
from __future__ import annotations

import math

import numpy as np

# src/millipyde_image.cpp:64
GREY_WEIGHTS = (0.2125, 0.7154, 0.0721)
# src/millipyde_image.cpp:702 (degrees -> radians)
DEG2RAD = 0.01745329252


def _f64(img):
    return np.asarray(img, dtype=np.float64)


def _split_alpha(x):
    """(colour, alpha-or-None) views of an (H, W[, C]) image."""
    if x.ndim == 3 and x.shape[2] == 4:
        return x[..., :3], x[..., 3:]
    return x, None


def _join_alpha(col, alpha):
    return col if alpha is None else np.concatenate([col, alpha], axis=2)


def rgb2grey(img):
    """min(1, 0.2125 R + 0.7154 G + 0.0721 B)  (src/millipyde_image.cpp:50-66).

    The reference divides by 255 for its uint8 input; float inputs in [0,1]
    take the weights directly.  A 1-channel image is returned unchanged."""
    x = _f64(img)
    if x.ndim == 2 or x.shape[2] < 3:
        return x
    g = GREY_WEIGHTS[0] * x[..., 0] + GREY_WEIGHTS[1] * x[..., 1] + GREY_WEIGHTS[2] * x[..., 2]
    return np.minimum(1.0, g)


def transpose(img):
    """out[x][y] = in[y][x]  (src/millipyde_image.cpp:73-96)."""
    x = np.asarray(img)
    return np.ascontiguousarray(np.swapaxes(x, 0, 1))


def fliplr(img):
    """out[y][W-1-x] = in[y][x]  (src/millipyde_image.cpp:99-111)."""
    return np.ascontiguousarray(np.asarray(img)[:, ::-1])


def gaussian_radius(sigma):
    """Build radius ceil(3 sigma); the reference fixed it at 8
    (src/include/millipyde_image.h:11)."""
    return int(math.ceil(3.0 * sigma))


def gaussian_weights(sigma, radius):
    """exp(-k^2 / (2 sigma^2)), k = -r..r, normalised to sum 1
    (src/millipyde_image.cpp:745-756)."""
    k = np.arange(-radius, radius + 1, dtype=np.float64)
    e = np.exp(-(k * k) / (2.0 * sigma * sigma))
    return e / e.sum()


def _correlate_axis(x, w, axis):
    """Zero-padded correlation along `axis` (src/millipyde_image.cpp:170-172,
    :218-221: samples outside the image read as 0)."""
    r = (len(w) - 1) // 2
    pad = [(0, 0)] * x.ndim
    pad[axis] = (r, r)
    xp = np.pad(x, pad)
    out = np.zeros_like(x)
    n = x.shape[axis]
    for k in range(len(w)):
        sl = [slice(None)] * x.ndim
        sl[axis] = slice(k, k + n)
        out += w[k] * xp[tuple(sl)]
    return out


def gaussian(img, sigma, radius=None):
    """Separable zero-padded gaussian blur, columns then rows as in the
    reference's two passes (src/millipyde_image.cpp:146-244).  radius defaults
    to ceil(3 sigma); pass radius=8 for the reference's fixed radius."""
    x = _f64(img)
    r = gaussian_radius(sigma) if radius is None else int(radius)
    w = gaussian_weights(sigma, r)
    return _correlate_axis(_correlate_axis(x, w, 1), w, 0)


def rotate_source_coords(h, w, angle):
    """Source position of every output pixel:
    s = R(theta) (p - c) + c, c = (W/2, H/2)  (src/millipyde_image.cpp:114-139).
    Returns (sx, sy) float64 arrays of shape (h, w)."""
    th = angle * DEG2RAD
    c, s = math.cos(th), math.sin(th)
    ys, xs = np.meshgrid(np.arange(h, dtype=np.float64), np.arange(w, dtype=np.float64), indexing="ij")
    dx, dy = xs - w / 2.0, ys - h / 2.0
    return c * dx - s * dy + w / 2.0, s * dx + c * dy + h / 2.0


def rotate(img, angle, mode="bilinear"):
    """Rotate by `angle` degrees about (W/2, H/2), same output size, zero fill.

    mode="bilinear" (the build): the 4 neighbours of the source position,
    neighbours outside the image contribute 0.
    mode="nearest" (the reference): source index truncated toward zero, 0 when
    outside (src/millipyde_image.cpp:120-137)."""
    x = _f64(img)
    h, w = x.shape[0], x.shape[1]
    sx, sy = rotate_source_coords(h, w, angle)
    chan = x.shape[2:] if x.ndim == 3 else ()
    if mode == "nearest":
        ix, iy = np.trunc(sx).astype(np.int64), np.trunc(sy).astype(np.int64)
        ok = (ix >= 0) & (ix < w) & (iy >= 0) & (iy < h)
        out = np.zeros((h, w) + chan)
        out[ok] = x[iy[ok], ix[ok]]
        return out
    x0, y0 = np.floor(sx).astype(np.int64), np.floor(sy).astype(np.int64)
    fx, fy = sx - x0, sy - y0

    def tap(ix, iy):
        ok = (ix >= 0) & (ix < w) & (iy >= 0) & (iy < h)
        v = np.zeros((h, w) + chan)
        v[ok] = x[iy[ok], ix[ok]]
        return v

    a, b = tap(x0, y0), tap(x0 + 1, y0)
    c, d = tap(x0, y0 + 1), tap(x0 + 1, y0 + 1)
    if chan:
        fx, fy = fx[..., None], fy[..., None]
    return (1 - fy) * ((1 - fx) * a + fx * b) + fy * ((1 - fx) * c + fx * d)


def gaussian_rotate_window(img, sigma, angle, rows, cols):
    """Output pixels [rows[0]:rows[1], cols[0]:cols[1]] of
    rotate(gaussian(img, sigma), angle), computed from the source rows and
    columns that window needs only (for images too large for the whole-image
    oracle).  Same formulas as gaussian() and rotate(): the blur is evaluated
    on the bounding box of the window's bilinear neighbours, from a source
    crop r pixels wider on every side that is not an image edge, so zero
    padding applies only at the real image edges
    (src/millipyde_image.cpp:170-172, :114-139)."""
    x = img    # only the crop below is read: any array with .shape, .ndim and 2-D slicing
    h, w = x.shape[0], x.shape[1]
    chan = x.shape[2:] if x.ndim == 3 else ()
    th = angle * DEG2RAD
    c, s = math.cos(th), math.sin(th)
    ys, xs = np.meshgrid(np.arange(rows[0], rows[1], dtype=np.float64),
                         np.arange(cols[0], cols[1], dtype=np.float64), indexing="ij")
    dx, dy = xs - w / 2.0, ys - h / 2.0
    sx, sy = c * dx - s * dy + w / 2.0, s * dx + c * dy + h / 2.0
    x0, y0 = np.floor(sx).astype(np.int64), np.floor(sy).astype(np.int64)
    fx, fy = sx - x0, sy - y0
    out_shape = sx.shape + chan
    # bounding box (inside the image) of every neighbour the window reads
    bx0, bx1 = max(0, int(x0.min())), min(w - 1, int(x0.max()) + 1)
    by0, by1 = max(0, int(y0.min())), min(h - 1, int(y0.max()) + 1)
    if bx0 > bx1 or by0 > by1:
        return np.zeros(out_shape)
    r = gaussian_radius(sigma)
    cx0, cx1 = max(0, bx0 - r), min(w - 1, bx1 + r)
    cy0, cy1 = max(0, by0 - r), min(h - 1, by1 + r)
    crop = _f64(np.asarray(x[cy0:cy1 + 1, cx0:cx1 + 1]))
    wts = gaussian_weights(sigma, r)
    blur = _correlate_axis(_correlate_axis(crop, wts, 1), wts, 0)

    def tap(ix, iy):
        ok = (ix >= 0) & (ix < w) & (iy >= 0) & (iy < h)
        v = np.zeros(out_shape)
        v[ok] = blur[iy[ok] - cy0, ix[ok] - cx0]
        return v

    a, b = tap(x0, y0), tap(x0 + 1, y0)
    cc, d = tap(x0, y0 + 1), tap(x0 + 1, y0 + 1)
    if chan:
        fx, fy = fx[..., None], fy[..., None]
    return (1 - fy) * ((1 - fx) * a + fx * b) + fy * ((1 - fx) * cc + fx * d)


def brightness(img, delta):
    """clamp01(x + delta) on colour channels  (src/millipyde_image.cpp:384-398)."""
    col, alpha = _split_alpha(_f64(img))
    return _join_alpha(np.clip(col + delta, 0.0, 1.0), alpha)


def adjust_gamma(img, gamma, gain=1.0):
    """clamp01(gain * x^gamma) on colour channels
    (src/millipyde_image.cpp:438-454)."""
    col, alpha = _split_alpha(_f64(img))
    return _join_alpha(np.clip(gain * np.power(col, gamma), 0.0, 1.0), alpha)


def colorize(img, r_mult, g_mult, b_mult):
    """min(1, c * mult_c) on R, G, B; alpha kept; greyscale unchanged
    (src/millipyde_image.cpp:494-524, float form of the byte clamp)."""
    x = _f64(img)
    if x.ndim == 2 or x.shape[2] < 3:
        return x
    out = x.copy()
    for k, m in enumerate((r_mult, g_mult, b_mult)):
        out[..., k] = np.minimum(1.0, x[..., k] * m)
    return out


OPS = {
    "rgb2grey": lambda x: rgb2grey(x),
    "rgb2gray": lambda x: rgb2grey(x),
    "transpose": lambda x: transpose(x),
    "fliplr": lambda x: fliplr(x),
    "gaussian": lambda x, s: gaussian(x, s),
    "rotate": lambda x, a: rotate(x, a),
    "brightness": lambda x, d: brightness(x, d),
    "adjust_gamma": lambda x, g, k=1.0: adjust_gamma(x, g, k),
    "colorize": lambda x, r, g, b: colorize(x, r, g, b),
}


def run_ops(img, ops):
    """Apply [(name, *args), ...] in order (the Pipeline / method sequence of
    src/gpupipeline.c:351-403)."""
    x = _f64(img)
    for op in ops:
        x = OPS[op[0]](x, *op[1:])
    return x


# ---------------------------------------------------------------------------
# Counter RNG (restated from the library's mp_counter_uniform) so tests can
# regenerate the per-image parameters of a seeded Pipeline / Generator run.
# ---------------------------------------------------------------------------
_M64 = (1 << 64) - 1


def _mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & _M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


def counter_uniform(seed, index, stage, slot):
    h = _mix64(seed & _M64)
    h = _mix64(h ^ (index & _M64))
    h = _mix64(h ^ (((stage & 0xFFFFFFFF) << 32) | (slot & 0xFFFFFFFF)))
    return (h >> 11) * (1.0 / 9007199254740992.0)


def resolve_stage(stage, seed, index, s):
    """(run, params) for one stage dict {op, lo, hi, random, probability}."""
    lo, hi = stage.get("lo", (0.0, 0.0, 0.0)), stage.get("hi", (0.0, 0.0, 0.0))
    lo = tuple(lo) + (0.0,) * (3 - len(lo))
    hi = tuple(hi) + (0.0,) * (3 - len(hi))
    if stage.get("random"):
        p = tuple(lo[k] + counter_uniform(seed, index, s, k) * (hi[k] - lo[k]) for k in range(3))
    else:
        p = lo
    prob = stage.get("probability", -1.0)
    run = True
    if 0.0 < prob < 1.0:
        run = counter_uniform(seed, index, s, 3) <= prob
    return run, p
