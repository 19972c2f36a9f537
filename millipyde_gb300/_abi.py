"""ctypes view of the C-ABI in include/millipyde_gb300.h.

This is how Python code other than the CPython extension reaches the library:
the autograd wrapper, the parity tests and bench.py call the exported C
functions directly, with device buffers owned by the caller (for example
torch tensors) described by MPImage records.  Loading fails loudly if the
library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmillipyde_gb300.so")

# MPOpCode
OP_NONE, OP_RGB2GREY, OP_TRANSPOSE, OP_GAUSSIAN, OP_FLIPLR, OP_ROTATE, OP_BRIGHTNESS, \
    OP_ADJUST_GAMMA, OP_COLORIZE = range(9)
OP_CODES = {
    "rgb2grey": OP_RGB2GREY, "rgb2gray": OP_RGB2GREY, "transpose": OP_TRANSPOSE,
    "gaussian": OP_GAUSSIAN, "fliplr": OP_FLIPLR, "rotate": OP_ROTATE,
    "brightness": OP_BRIGHTNESS, "adjust_gamma": OP_ADJUST_GAMMA, "colorize": OP_COLORIZE,
}

MILLIPYDE_SUCCESS = 0
MP_ERROR_NO_DEVICE = 1000
MP_ERROR_CUDA = 1001
MP_ERROR_OUT_OF_MEMORY = 1002
MP_ERROR_INVALID_ARGS = 1003
MP_ERROR_UNSUPPORTED_TYPE = 1004
MP_ERROR_UNSUPPORTED_DIMS = 1005
MP_ERROR_NULL_DATA = 1006
MP_ERROR_KERNEL_TIMEOUT = 1007
MP_ERROR_BAD_DESCRIPTOR = 1008
MP_ERROR_TOO_LARGE = 1009
MP_MAX_RADIUS = 48


class MPObjData(C.Structure):
    _fields_ = [("device_data", C.c_void_p), ("ndims", C.c_int), ("dims", C.POINTER(C.c_int)),
                ("type", C.c_int), ("mem_loc", C.c_int), ("stream", C.c_void_p),
                ("pinned", C.c_int), ("nbytes", C.c_size_t)]


class MPImage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("height", C.c_int), ("width", C.c_int),
                ("channels", C.c_int), ("pitch", C.c_int)]


class MPStage(C.Structure):
    _fields_ = [("op", C.c_int), ("random", C.c_int), ("lo", C.c_double * 3),
                ("hi", C.c_double * 3), ("probability", C.c_double)]


class RotateArgs(C.Structure):
    _fields_ = [("angle", C.c_double)]


class GaussianArgs(C.Structure):
    _fields_ = [("sigma", C.c_double)]


class BrightnessArgs(C.Structure):
    _fields_ = [("delta", C.c_double)]


class ColorizeArgs(C.Structure):
    _fields_ = [("r_mult", C.c_double), ("g_mult", C.c_double), ("b_mult", C.c_double)]


class GammaArgs(C.Structure):
    _fields_ = [("gamma", C.c_double), ("gain", C.c_double)]


# Every symbol include/millipyde_gb300.h declares: name -> (restype, argtypes)
_P = C.c_void_p
_ST = C.c_int
SIGNATURES = {
    "mperr_str": (C.c_char_p, [_ST]),
    "mp_last_cuda_error": (C.c_char_p, []),
    "random_int_in_range": (_ST, [C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "random_double_in_range": (_ST, [C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "mp_seed": (None, [C.c_uint64]),
    "mp_counter_uniform": (C.c_double, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32]),
    "mpimg_color_to_greyscale": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_transpose": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_gaussian": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_fliplr": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_rotate": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_brightness": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_colorize": (_ST, [C.POINTER(MPObjData), _P]),
    "mpimg_adjust_gamma": (_ST, [C.POINTER(MPObjData), _P]),
    "mpobj_copy_from_host": (_ST, [C.POINTER(MPObjData), _P, C.c_int, C.POINTER(C.c_int64),
                                   C.c_int, C.c_int, C.c_int]),
    "mpobj_host_nbytes": (C.c_size_t, [C.POINTER(MPObjData)]),
    "mpobj_copy_to_host": (_ST, [C.POINTER(MPObjData), _P]),
    "mpobj_clone_data": (C.POINTER(MPObjData), [C.POINTER(MPObjData), C.c_int, C.c_int]),
    "mpobj_dealloc_device_data": (None, [C.POINTER(MPObjData)]),
    "mp_type_itemsize": (C.c_int, [C.c_int]),
    "mpdev_initialize": (_ST, []),
    "mpdev_get_device_count": (C.c_int, []),
    "mpdev_get_recommended_device": (C.c_int, []),
    "mpdev_get_target_device": (C.c_int, []),
    "mpdev_set_target_device": (None, [C.c_int]),
    "mpdev_is_valid_device": (C.c_int, [C.c_int]),
    "mpdev_get_stream": (_P, [C.c_int, C.c_int]),
    "mpdev_synchronize": (_ST, []),
    "mpdev_get_device_name": (_ST, [C.c_int, C.c_char_p, C.c_int]),
    "mpdev_stream_synchronize": (_ST, [_P]),
    "mpdev_pool_usage": (_ST, [C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "mpdev_pool_reset_peak": (_ST, [C.c_int]),
    "mpdev_set_alloc_limit": (None, [C.c_size_t]),
    "mpdev_selftest_wait_timeout": (_ST, [C.c_uint32, _P]),
    "mpk_pipeline_shapes": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage),
                                  C.POINTER(MPImage), C.c_int, C.c_uint64, C.c_uint64]),
    "mpk_pipeline_run": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage),
                               C.POINTER(MPImage), C.c_int, C.c_uint64, C.c_uint64, _P]),
    "mpk_pipeline_run_unfused": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage),
                                       C.POINTER(MPImage), C.c_int, C.c_uint64, C.c_uint64, _P]),
    "mpk_plan_create": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage), C.POINTER(MPImage),
                              C.c_int, C.c_uint64, C.c_uint64, _P, C.POINTER(_P)]),
    "mpk_plan_launch": (_ST, [_P, _P]),
    "mpk_plan_num_launches": (C.c_int, [_P]),
    "mpk_plan_destroy": (_ST, [_P]),
    "mpk_plan_launch_range": (_ST, [_P, C.c_int, C.c_int, _P]),
    "mpk_plan_launch_info": (_ST, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "mpk_pipeline_run_host": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage),
                                    C.POINTER(MPImage), C.c_int, C.c_uint64, C.c_uint64, _P]),
    "mpk_tune_set_gauss_tile": (_ST, [C.c_int] * 7),
    "mpk_tune_get_gauss_tile": (_ST, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]),
    "mpk_tune_set_stream": (_ST, [C.c_int] * 2),
    "mpk_tune_set_chunk_bytes": (_ST, [C.c_size_t]),
    "mpk_tune_set_fuse": (_ST, [C.c_int]),
    "mpk_tune_set_kernel": (_ST, [C.c_int, C.c_int, C.c_int]),
    "mpk_tune_get_kernel": (_ST, [C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "mpk_tune_clear": (None, []),
    "mpk_chain_shape": (_ST, [C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int,
                              C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mpk_chain_forward": (_ST, [C.POINTER(C.c_int), C.c_int, _P, _P, _P, C.c_int, C.c_int, C.c_int,
                                C.c_int, _P]),
    "mpk_chain_backward": (_ST, [C.POINTER(C.c_int), C.c_int, _P, _P, _P, _P, _P, C.c_int, C.c_int,
                                 C.c_int, C.c_int, _P]),
    "mpk_chain_backward_masked": (_ST, [C.POINTER(C.c_int), C.c_int, _P, _P, _P, _P, _P, C.POINTER(C.c_int),
                                        C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mpk_chain_saved_layout": (_ST, [C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_size_t),
                                     C.POINTER(C.c_size_t)]),
    "mpk_chain_forward_saved": (_ST, [C.POINTER(C.c_int), C.c_int, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int,
                                      C.c_int, _P]),
    "mpk_chain_backward_saved": (_ST, [C.POINTER(C.c_int), C.c_int, _P, _P, _P, _P, _P, _P, _P,
                                       C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mpk_pipeline_run_noalloc": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(MPImage),
                                       C.POINTER(MPImage), C.c_int, C.c_uint64, C.c_uint64, _P]),
    "mpk_pipeline_run_objects": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(C.POINTER(MPObjData)),
                                       C.c_int, C.c_uint64, C.c_uint64, C.c_int]),
    "mpk_pipeline_produce": (_ST, [C.POINTER(MPStage), C.c_int, C.POINTER(C.POINTER(MPObjData)),
                                   C.POINTER(C.POINTER(MPObjData)), C.c_int, C.c_uint64, C.c_uint64]),
    "mpk_pipeline_resolve": (_ST, [C.POINTER(MPStage), C.c_int, C.c_int, C.c_uint64, C.c_uint64,
                                   C.POINTER(C.c_double)]),
}

_lib = None


def lib():
    """The loaded library with prototypes set (raises OSError if unbuilt)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libmillipyde_gb300.so is not built (%s)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class MPError(RuntimeError):
    def __init__(self, status):
        L = lib()
        msg = L.mperr_str(status).decode()
        cuda = L.mp_last_cuda_error().decode()
        super().__init__("%s (status %d)%s" % (msg, status, (": " + cuda) if cuda else ""))
        self.status = status


def check(status):
    if status != MILLIPYDE_SUCCESS:
        raise MPError(status)


def stage(op, *params, random=False, lo=None, hi=None, probability=-1.0):
    """Build an MPStage: stage("rotate", 17.0) or stage("rotate", random=True,
    lo=(-45,), hi=(45,))."""
    s = MPStage()
    s.op = OP_CODES[op] if isinstance(op, str) else int(op)
    s.random = 1 if random else 0
    vals = list(lo if lo is not None else params) + [0.0] * 3
    his = list(hi if hi is not None else params) + [0.0] * 3
    for k in range(3):
        s.lo[k] = float(vals[k])
        s.hi[k] = float(his[k])
    s.probability = float(probability)
    return s


def stages(*items):
    arr = (MPStage * len(items))()
    for i, it in enumerate(items):
        arr[i] = it
    return arr


def image(ptr, height, width, channels, pitch):
    m = MPImage()
    m.data = ptr
    m.height, m.width, m.channels, m.pitch = height, width, channels, pitch
    return m


def images(items):
    arr = (MPImage * max(1, len(items)))()
    for i, it in enumerate(items):
        arr[i] = it
    return arr
