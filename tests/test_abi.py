"""CPU: the C-ABI library loads and exports every symbol the public header
declares; host-only entry points (status strings, RNG, planning) behave."""
import ctypes as C
import os
import re

import numpy as np

from millipyde_gb300 import _abi
from oracle import oracle as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "millipyde_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*[A-Za-z_][A-Za-z0-9_ \*]*?\b([a-z][a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if not n.startswith("typedef")))


def test_header_parses_to_many_functions():
    names = declared_functions()
    assert "mpimg_gaussian" in names and "mpk_pipeline_run" in names and len(names) > 30


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(_abi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_signature_table_covers_header():
    assert set(declared_functions()) <= set(_abi.SIGNATURES)


def test_status_strings():
    L = _abi.lib()
    assert L.mperr_str(0) == b"success"
    assert b"probability" in L.mperr_str(35)  # GPUOPERATION_ERROR_INVALID_PROBABILITY
    assert b"CUDA device" in L.mperr_str(_abi.MP_ERROR_NO_DEVICE)
    assert L.mperr_str(99999) == b"unknown failure"


def test_reference_status_values_kept():
    # positions from src/include/millipyde.h:27-94
    L = _abi.lib()
    assert b"gpuimage" in L.mperr_str(33)   # GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_DIMS
    assert b"Pipeline" in L.mperr_str(44)   # GPUPIPELINE_ERROR_CONSTRUCTION_NAMED_ARGS
    assert b"Generator" in L.mperr_str(54)  # GPUGENERATOR_ERROR_NONLIST_OPERATIONS


def test_counter_rng_matches_oracle_restatement():
    L = _abi.lib()
    for seed, idx, st, sl in [(0, 0, 0, 0), (1, 2, 3, 1), (2**63 + 5, 999, 7, 3), (42, 10**12, 0, 2)]:
        assert L.mp_counter_uniform(seed, idx, st, sl) == O.counter_uniform(seed, idx, st, sl)


def test_seeded_random_range():
    L = _abi.lib()
    L.mp_seed(5)
    a = C.c_double()
    vals = []
    for _ in range(100):
        assert L.random_double_in_range(-2.0, 3.0, C.byref(a)) == 0
        vals.append(a.value)
    assert min(vals) >= -2.0 and max(vals) < 3.0
    L.mp_seed(5)
    again = []
    for _ in range(100):
        L.random_double_in_range(-2.0, 3.0, C.byref(a))
        again.append(a.value)
    assert vals == again
    i = C.c_int()
    for _ in range(200):
        L.random_int_in_range(3, 5, C.byref(i))
        assert 3 <= i.value <= 5


def test_pipeline_shapes_host_logic():
    L = _abi.lib()
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("transpose"), _abi.stage("gaussian", 2.0))
    ins = _abi.images([_abi.image(None, 10, 30, 3, 368), _abi.image(None, 5, 7, 1, 32)])
    outs = _abi.images([_abi.MPImage(), _abi.MPImage()])
    assert L.mpk_pipeline_shapes(st, 3, ins, outs, 2, 0, 0) == 0
    assert (outs[0].height, outs[0].width, outs[0].channels, outs[0].pitch) == (30, 10, 1, 48)
    assert (outs[1].height, outs[1].width, outs[1].channels) == (7, 5, 1)


def test_pipeline_resolve_matches_oracle():
    L = _abi.lib()
    spec = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
            dict(op="gaussian", random=True, lo=(0.5,), hi=(4,)),
            dict(op="fliplr", probability=0.5)]
    st = _abi.stages(_abi.stage("rotate", random=True, lo=(-45,), hi=(45,)),
                     _abi.stage("gaussian", random=True, lo=(0.5,), hi=(4,)),
                     _abi.stage("fliplr", probability=0.5))
    n = 50
    out = (C.c_double * (n * 3 * 4))()
    assert L.mpk_pipeline_resolve(st, 3, n, 77, 100, out) == 0
    flips = 0
    for i in range(n):
        for s, d in enumerate(spec):
            run, p = O.resolve_stage(d, 77, 100 + i, s)
            base = (i * 3 + s) * 4
            assert out[base + 3] == (1.0 if run else 0.0)
            if d.get("random"):
                assert out[base] == p[0]
        flips += out[(i * 3 + 2) * 4 + 3] == 1.0
    assert 10 < flips < 40


def test_invalid_stage_rejected_on_host():
    L = _abi.lib()
    st = _abi.stages(_abi.stage("gaussian", -1.0))
    ins = _abi.images([_abi.image(None, 4, 4, 1, 16)])
    outs = _abi.images([_abi.MPImage()])
    assert L.mpk_pipeline_shapes(st, 1, ins, outs, 1, 0, 0) == _abi.MP_ERROR_INVALID_ARGS
    st = _abi.stages(_abi.stage("gaussian", 17.0))   # radius 51 > MP_MAX_RADIUS
    assert L.mpk_pipeline_shapes(st, 1, ins, outs, 1, 0, 0) == _abi.MP_ERROR_TOO_LARGE
    bad = _abi.stages(_abi.stage(99))
    assert L.mpk_pipeline_shapes(bad, 1, ins, outs, 1, 0, 0) == _abi.MP_ERROR_BAD_DESCRIPTOR
    ins2 = _abi.images([_abi.image(None, 4, 4, 2, 32)])   # 2 channels unsupported
    assert L.mpk_pipeline_shapes(st, 1, ins2, outs, 1, 0, 0) == _abi.MP_ERROR_BAD_DESCRIPTOR


def test_itemsize_table():
    L = _abi.lib()
    for t in (np.uint8, np.float32, np.float64, np.int64, np.int16):
        assert L.mp_type_itemsize(np.dtype(t).num) == np.dtype(t).itemsize


def test_chain_backward_masked_host_checks():
    # argument and descriptor checks happen on the host, before any device
    # call: negative batch, missing buffers, unsupported channels, unknown ops
    L = _abi.lib()
    ops = (C.c_int * 2)(_abi.OP_ROTATE, _abi.OP_GAUSSIAN)
    mask = (C.c_int * 2)(1, 0)
    params = (C.c_double * 6)(10.0, 0, 0, 2.0, 0, 0)
    f = L.mpk_chain_backward_masked
    assert f(ops, 2, params, None, None, None, None, mask, -1, 8, 8, 3, None) == _abi.MP_ERROR_INVALID_ARGS
    assert f(ops, 2, params, None, None, None, None, mask, 1, 8, 8, 3, None) == _abi.MP_ERROR_INVALID_ARGS
    assert f(ops, 2, params, None, None, None, None, mask, 0, 8, 8, 2, None) == _abi.MP_ERROR_BAD_DESCRIPTOR
    bad = (C.c_int * 1)(99)
    assert f(bad, 1, params, None, None, None, None, mask, 0, 8, 8, 3, None) == _abi.MP_ERROR_BAD_DESCRIPTOR
    assert f(ops, 2, params, None, None, None, None, mask, 0, 8, 8, 3, None) == _abi.MILLIPYDE_SUCCESS


def test_chain_saved_layout():
    """Saved forward intermediates of a differentiable chain: the inputs of
    the ops that open the forward plan's later segments (host arithmetic
    only, no device call)."""
    import ctypes as C
    from millipyde_gb300 import _abi
    L = _abi.lib()

    def layout(names, B=2, H=5, W=4, Cc=3):
        codes = {"rotate": _abi.OP_ROTATE, "gaussian": _abi.OP_GAUSSIAN, "adjust_gamma": _abi.OP_ADJUST_GAMMA,
                 "rgb2grey": _abi.OP_RGB2GREY, "brightness": _abi.OP_BRIGHTNESS,
                 "transpose": _abi.OP_TRANSPOSE, "fliplr": _abi.OP_FLIPLR}
        n = len(names)
        ops = (C.c_int * max(1, n))(*[codes[x] for x in names])
        cnt, nb = C.c_int(), C.c_size_t()
        idx, off = (C.c_int * max(1, n))(), (C.c_size_t * max(1, n))()
        assert L.mpk_chain_saved_layout(ops, n, B, H, W, Cc, C.byref(cnt), idx, off, C.byref(nb)) == 0
        return [idx[i] for i in range(cnt.value)], [off[i] for i in range(cnt.value)], nb.value

    # rgb2grey after a colour gaussian opens a pointwise segment of its own,
    # taking the gaussian's epilogue along (the boundary is the blur's output)
    assert layout(["rotate", "gaussian", "adjust_gamma", "rgb2grey"]) == ([1, 2], [0, 480], 2 * 480)
    # with a flip in the gaussian's segment only the grey moves
    assert layout(["gaussian", "fliplr", "adjust_gamma", "rgb2grey"]) == ([3], [0], 480)
    assert layout(["gaussian", "rotate", "brightness"]) == ([1], [0], 2 * 5 * 4 * 3 * 4)
    # the grey prologue joins the gaussian; the intermediate has one channel
    assert layout(["rgb2grey", "gaussian", "rotate", "adjust_gamma"]) == ([2], [0], 2 * 5 * 4 * 1 * 4)
    # transpose and fliplr share a segment; the rotate opens the next
    assert layout(["transpose", "fliplr", "rotate"]) == ([2], [0], 2 * 4 * 5 * 3 * 4)
    assert layout(["rotate", "gaussian", "rotate"]) == ([1, 2], [0, 480], 960)
    assert layout(["brightness", "adjust_gamma"]) == ([], [], 0)
    assert layout([]) == ([], [], 0)
