"""Image file loading: image_from_path / images_from_path.

The reference read files with scikit-image (src/gpuimage.c:574-688), which is
not a dependency here.  This module decodes PNG with the standard library
(zlib) with the row filters reversed in C (the extension's _png_unfilter):
8- and 16-bit greyscale, grey+alpha, RGB and RGBA, non-interlaced, all
five row filters.  Results are uint8 (or uint16) arrays of shape (H, W)
or (H, W, C), as skimage.io.imread returns them.  Directory listings are
sorted by file name (the reference used readdir order, which depends on the
filesystem).
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

_EXTS = (".png", ".jpg", ".jpeg", ".tiff", ".bmp")  # src/gpuimage.c:800-824
_CHANNELS = {0: 1, 2: 3, 4: 2, 6: 4}


def read_png(path: str) -> np.ndarray:
    """Decode a PNG file into a numpy array."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("%s: not a PNG file" % path)
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if ctype == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
    if hdr is None:
        raise ValueError("%s: missing IHDR" % path)
    w, h, depth, color, _, _, interlace = hdr
    if interlace or color not in _CHANNELS or depth not in (8, 16):
        raise ValueError("%s: unsupported PNG (colour type %d, depth %d, interlace %d)"
                         % (path, color, depth, interlace))
    ch = _CHANNELS[color]
    bpp = ch * depth // 8
    stride = w * bpp
    from ._millipyde import _png_unfilter
    out = np.frombuffer(_png_unfilter(zlib.decompress(b"".join(idat)), h, stride, bpp), dtype=np.uint8)
    out = out.reshape(h, stride)
    if depth == 8:
        img = out.reshape(h, w, ch).copy()
    else:
        b = out.astype(np.uint16).reshape(h, w * ch, 2)
        img = ((b[..., 0] << 8) | b[..., 1]).reshape(h, w, ch)
    return img[..., 0] if ch == 1 else img


def image_from_path(path: str):
    """Load one image file into a gpuimage (src/gpuimage.c:574-631)."""
    from . import gpuimage
    if not str(path).lower().endswith(".png"):
        raise ValueError("%s: only PNG files can be decoded" % path)
    return gpuimage(read_png(str(path)))


def images_from_path(path: str):
    """Load every PNG file of a directory into a list of gpuimages
    (src/gpuimage.c:639-688)."""
    names = sorted(n for n in os.listdir(path)
                   if n.lower().endswith(".png") and os.path.isfile(os.path.join(path, n)))
    return [image_from_path(os.path.join(path, n)) for n in names]
