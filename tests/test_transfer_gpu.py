"""GPU: object transfers between host arrays and device objects.

Every layout must round-trip exactly: pitched image rows (row bytes not a
multiple of 16), packed rows, byte images, 1-D arrays, large and small."""
import numpy as np
import pytest

import millipyde_gb300 as mp

from helpers import obj_free, obj_from_host, obj_to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,dtype", [
    ((2000, 1801, 3), np.float32),     # pitched rows, 43 MB
    ((1200, 1200, 3), np.float32),     # packed rows (14400 B), 17 MB
    ((3000, 2001, 4), np.uint8),       # pitched byte rows, 24 MB
    ((300, 301, 3), np.float32),       # 1 MB
    ((4 << 20,), np.float32),          # 1-D, 16 MB
    ((5_000_001,), np.float32),        # 1-D, odd length
])
def test_roundtrip_through_the_c_abi(gpu, shape, dtype):
    rng = np.random.default_rng(sum(shape))
    if dtype == np.uint8:
        x = rng.integers(0, 256, size=shape).astype(np.uint8)
    else:
        x = rng.random(shape, dtype=np.float32)
    o = obj_from_host(x, image=len(shape) >= 2)
    try:
        y = obj_to_host(o)
    finally:
        obj_free(o)
    assert y.dtype == x.dtype and y.shape == x.shape
    assert np.array_equal(x, y)


def test_python_objects_roundtrip_and_compute(gpu):
    rng = np.random.default_rng(5)
    x = rng.random((1500, 1333, 3), dtype=np.float32)
    img = mp.gpuimage(x)
    assert np.array_equal(np.array(img), x)
    img.fliplr()
    assert np.array_equal(np.array(img), x[:, ::-1])
    a = rng.random(3_000_000).astype(np.float32)
    assert np.array_equal(np.array(mp.gpuarray(a)), a)
