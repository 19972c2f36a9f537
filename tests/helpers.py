"""Helpers shared by the parity tests: C-ABI object round trips and tolerances."""
import ctypes as C

import numpy as np

from millipyde_gb300 import _abi

# Max-abs tolerance of every float32 op against the FP64 oracle on inputs in
# [0, 1] (the bar the path is held to).
TOL = 1e-5


def obj_from_host(arr, image=True):
    L = _abi.lib()
    arr = np.ascontiguousarray(arr)
    o = _abi.MPObjData()
    shape = (C.c_int64 * max(1, arr.ndim))(*arr.shape)
    _abi.check(L.mpobj_copy_from_host(C.byref(o), arr.ctypes.data_as(C.c_void_p), arr.ndim, shape,
                                      arr.dtype.num, arr.dtype.itemsize, 1 if image else 0))
    return o


def obj_to_host(o):
    L = _abi.lib()
    shape = [o.dims[i] for i in range(o.ndims)]
    out = np.empty(shape, dtype=_np_type(o.type))
    _abi.check(L.mpobj_copy_to_host(C.byref(o), out.ctypes.data_as(C.c_void_p)))
    return out


def _np_type(num):
    for t in (np.float32, np.float64, np.uint8, np.int64, np.int32, np.uint16, np.int16, np.int8):
        if np.dtype(t).num == num:
            return t
    raise ValueError(num)


def obj_free(o):
    _abi.lib().mpobj_dealloc_device_data(C.byref(o))


def run_op(arr, fn_name, args=None):
    """Copy arr to the device, run mpimg_<fn_name>, copy back."""
    L = _abi.lib()
    o = obj_from_host(arr)
    try:
        fn = getattr(L, fn_name)
        st = fn(C.byref(o), C.byref(args) if args is not None else None)
        _abi.check(st)
        return obj_to_host(o)
    finally:
        obj_free(o)


def rand_image(rng, h, w, c, dtype=np.float32):
    shape = (h, w) if c == 1 else (h, w, c)
    return rng.random(shape).astype(dtype)


def maxabs(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.max(np.abs(a - b))) if a.size else 0.0
