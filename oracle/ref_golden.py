"""Generates tests/golden/reference_ops.npz from the reference's OWN kernels.

Test infrastructure.  Builds oracle/_ref/libmillipyde_ref.so (the
reference's src/millipyde_image.cpp compiled for the CPU against
oracle/ref_shim, see oracle/Makefile), runs every mpimg_* entry point of the
reference on small seeded inputs -- uint8 RGBA images and float64 greyscale
images, the two layouts the reference handles -- and stores inputs, op
parameters and outputs.  Run here, where the reference checkout exists:

    python oracle/ref_golden.py --reference <path of the reference checkout>

The .npz is committed; tests read it without the reference.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(ROOT, "tests", "golden", "reference_ops.npz")
LIB = os.path.join(HERE, "_ref", "libmillipyde_ref.so")

OPS = {"rgb2grey": 0, "transpose": 1, "gaussian": 2, "fliplr": 3, "rotate": 4,
       "brightness": 5, "colorize": 6, "adjust_gamma": 7}
NPY_UBYTE, NPY_DOUBLE = 2, 12


def build(reference):
    subprocess.run(["make", "-C", HERE, "REF=" + reference], check=True, capture_output=True)
    lib = C.CDLL(LIB)
    lib.ref_run.restype = C.c_long
    lib.ref_run.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p,
                            C.c_long, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_long,
                            C.POINTER(C.c_int)]
    return lib


def run(lib, op, arr, p=(0.0, 0.0, 0.0)):
    arr = np.ascontiguousarray(arr)
    nd = C.c_int(arr.ndim)
    dims = (C.c_int * 8)(*(list(arr.shape) + list(arr.strides)))
    cap = arr.size * 8 + 64
    out = np.zeros(cap, dtype=np.uint8)
    tout = C.c_int()
    n = lib.ref_run(OPS[op], arr.dtype.num, C.byref(nd), dims, arr.ctypes.data, arr.nbytes,
                    p[0], p[1], p[2], out.ctypes.data, cap, C.byref(tout))
    assert n >= 0
    shape = [dims[i] for i in range(nd.value)]
    dt = np.uint8 if tout.value == NPY_UBYTE else np.float64
    return np.frombuffer(out[:n].tobytes(), dtype=dt).reshape(shape)


def cases():
    rng = np.random.default_rng(20240611)
    rgba = rng.integers(0, 256, size=(48, 64, 4), dtype=np.uint8)       # W multiple of 16 (see below)
    rgba_odd = rng.integers(0, 256, size=(37, 53, 4), dtype=np.uint8)
    rgb_odd = rng.integers(0, 256, size=(37, 53, 3), dtype=np.uint8)
    grey = rng.random((48, 64))
    grey_odd = rng.random((37, 53))
    # The reference's column gaussian pass writes past the row end when the
    # width is not a multiple of 16 (src/millipyde_image.cpp:208-243 has no
    # x bound), so gaussian cases use 64-wide images.
    return [
        ("rgb2grey_rgba", "rgb2grey", rgba_odd, ()),
        ("rgb2grey_rgb", "rgb2grey", rgb_odd, ()),
        ("transpose_grey", "transpose", grey_odd, ()),
        ("transpose_rgba", "transpose", rgba_odd, ()),
        ("fliplr_grey", "fliplr", grey_odd, ()),
        ("fliplr_rgba", "fliplr", rgba_odd, ()),
        ("rotate30_grey", "rotate", grey_odd, (30.0,)),
        ("rotate-45_grey", "rotate", grey_odd, (-45.0,)),
        ("rotate90_grey", "rotate", grey, (90.0,)),
        ("rotate17_rgba", "rotate", rgba_odd, (17.0,)),
        ("gaussian2_grey", "gaussian", grey, (2.0,)),
        ("gaussian1p5_grey", "gaussian", grey, (1.5,)),
        ("gaussian2_rgba", "gaussian", rgba, (2.0,)),
        ("brightness0p1_grey", "brightness", grey_odd, (0.1,)),
        ("brightness-0p3_grey", "brightness", grey_odd, (-0.3,)),
        ("brightness0p1_rgba", "brightness", rgba_odd, (0.1,)),
        ("brightness-0p2_rgba", "brightness", rgba_odd, (-0.2,)),
        ("gamma2p2_grey", "adjust_gamma", grey_odd, (2.2, 1.0)),
        ("gamma0p5g1p2_grey", "adjust_gamma", grey_odd, (0.5, 1.2)),
        ("gamma2_rgba", "adjust_gamma", rgba_odd, (2.0, 1.0)),
        ("colorize_rgba", "colorize", rgba_odd, (1.5, 0.5, 1.0)),
    ]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path of the reference checkout")
    args = ap.parse_args()
    lib = build(args.reference)
    blob = {}
    for name, op, arr, p in cases():
        pp = tuple(p) + (0.0,) * (3 - len(p))
        y = run(lib, op, arr, pp)
        blob[name + "__in"] = arr
        blob[name + "__out"] = y
        blob[name + "__params"] = np.array(pp)
        blob[name + "__op"] = np.array(op)
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    np.savez_compressed(OUT, **blob)
    print("wrote", OUT, len(blob) // 4, "cases")


if __name__ == "__main__":
    main()
