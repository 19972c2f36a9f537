"""Image file loading (image_from_path / images_from_path).

The reference loaded files with scikit-image (src/gpuimage.c:574-688) and
tested it on its own PNG fixtures (tests/millipyde_tests.py:427-444).  Here
the files are written by an independent encoder in this test: every colour
type, 8 and 16 bits, every row filter (each row encoded with a different
one), several IDAT chunks; the decoder must return the exact pixels.  The
GPU cases load a directory of such files into gpuimages and run rgb2grey on
a loaded RGBA image, as the reference's tests do.
"""
import os
import struct
import zlib

import numpy as np
import pytest

from millipyde_gb300 import _io
from oracle import legacy as LG


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def encode_png(img, depth=8, filters=(0, 1, 2, 3, 4), idat_parts=3):
    """PNG bytes of an (H, W) or (H, W, C) uint8 / uint16 array; row y uses
    filter filters[y % len(filters)] (PNG specification, section 9)."""
    a = np.asarray(img)
    h, w = a.shape[:2]
    ch = 1 if a.ndim == 2 else a.shape[2]
    color = {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    if depth == 16:
        a16 = a.astype(">u2").reshape(h, w * ch)
        rows = np.frombuffer(a16.tobytes(), dtype=np.uint8).reshape(h, w * ch * 2).astype(np.int64)
    else:
        rows = a.astype(np.uint8).reshape(h, w * ch).astype(np.int64)
    bpp = ch * depth // 8
    out = bytearray()
    prev = np.zeros(rows.shape[1], dtype=np.int64)
    for y in range(h):
        cur = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int64), cur[:-bpp]])
        ul = np.concatenate([np.zeros(bpp, np.int64), prev[:-bpp]])
        ft = filters[y % len(filters)]
        pred = {0: 0 * cur, 1: left, 2: prev, 3: (left + prev) >> 1, 4: _paeth(left, prev, ul)}[ft]
        out.append(ft)
        out += ((cur - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = cur
    z = zlib.compress(bytes(out), 6)
    parts = [z[i * len(z) // idat_parts:(i + 1) * len(z) // idat_parts] for i in range(idat_parts)]
    hdr = struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", hdr) + _chunk(b"tEXt", b"Comment\x00test")
            + b"".join(_chunk(b"IDAT", p) for p in parts) + _chunk(b"IEND", b""))


@pytest.mark.parametrize("ch", [1, 2, 3, 4])
@pytest.mark.parametrize("depth", [8, 16])
def test_decoder_returns_exact_pixels(tmp_path, ch, depth):
    rng = np.random.default_rng(ch * 10 + depth)
    hi = 256 if depth == 8 else 65536
    shape = (37, 29) if ch == 1 else (37, 29, ch)
    img = rng.integers(0, hi, size=shape).astype(np.uint8 if depth == 8 else np.uint16)
    p = tmp_path / "x.png"
    p.write_bytes(encode_png(img, depth))
    got = _io.read_png(str(p))
    assert got.dtype == img.dtype and got.shape == img.shape
    assert np.array_equal(got, img)


def test_decoder_every_single_filter_and_smooth_content(tmp_path):
    # smooth content makes Average / Paeth choose every predictor branch
    y, x = np.mgrid[0:64, 0:80]
    img = np.stack([(x * 3 + y) % 256, (x * y) % 256, (255 - x - y) % 256, np.full_like(x, 200)], -1).astype(np.uint8)
    for ft in range(5):
        p = tmp_path / ("f%d.png" % ft)
        p.write_bytes(encode_png(img, 8, filters=(ft,), idat_parts=1))
        assert np.array_equal(_io.read_png(str(p)), img), ft


def test_decoder_rejects_what_it_cannot_read(tmp_path):
    p = tmp_path / "bad.png"
    p.write_bytes(b"not a png")
    with pytest.raises(ValueError):
        _io.read_png(str(p))
    img = np.zeros((4, 4, 3), np.uint8)
    data = bytearray(encode_png(img, 8, filters=(0,), idat_parts=1))
    data[8 + 8 + 12] = 1          # interlace method byte of the IHDR body
    data[8 + 8 + 13:8 + 8 + 13 + 4] = struct.pack(">I", zlib.crc32(bytes(data[12:8 + 8 + 13])) & 0xFFFFFFFF)
    p.write_bytes(bytes(data))
    with pytest.raises(ValueError):
        _io.read_png(str(p))


def _write_dir(tmp_path):
    rng = np.random.default_rng(3)
    imgs = {"b.png": rng.integers(0, 256, (50, 70, 4)).astype(np.uint8),
            "a.png": rng.integers(0, 256, (33, 20, 4)).astype(np.uint8),
            "c.PNG": rng.integers(0, 256, (16, 24, 3)).astype(np.uint8)}
    for name, img in imgs.items():
        (tmp_path / name).write_bytes(encode_png(img))
    (tmp_path / "notes.txt").write_text("not an image")
    os.mkdir(tmp_path / "sub.png")   # a directory named like a file is skipped
    return imgs


@pytest.mark.gpu
def test_images_from_path_loads_sorted_pngs(gpu, tmp_path):
    imgs = _write_dir(tmp_path)
    got = _io.images_from_path(str(tmp_path))
    names = sorted(imgs)
    assert len(got) == len(names)
    for g, n in zip(got, names):
        assert np.array_equal(np.array(g), imgs[n])


@pytest.mark.gpu
def test_image_from_path_then_rgb2grey(gpu, tmp_path):
    """As the reference's test_image_from_path2: load an RGBA PNG, rgb2grey on
    the device, compare with the reference's arithmetic (uint8 RGBA -> FP64
    grey)."""
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (45, 61, 4)).astype(np.uint8)
    p = tmp_path / "charlie_like.png"
    p.write_bytes(encode_png(img))
    g = _io.image_from_path(str(p))
    assert np.array_equal(np.array(g), img)
    g.rgb2grey()
    out = np.array(g)
    assert out.dtype == np.float64
    assert np.abs(out - LG.rgb2grey(img)).max() <= 1e-12
