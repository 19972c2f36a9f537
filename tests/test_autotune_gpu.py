"""GPU: the tuned kernel geometry is what the planner uses, results stay
exact against the oracle under every setting, and the autotuner's search
runs end to end on a small batch."""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi, autotune

from helpers import TOL
from test_pipeline_gpu import check_spec, dev_image, alloc_like

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RAGGED = [dict(op="rotate", random=True, lo=(-45,), hi=(45,)),
          dict(op="gaussian", random=True, lo=(0.5,), hi=(4.0,)),
          dict(op="adjust_gamma", random=True, lo=(0.5, 1.0), hi=(2.0, 1.0)),
          dict(op="fliplr", probability=0.5)]


@pytest.fixture
def clean():
    L = _abi.lib()
    yield L
    L.mpk_tune_clear()
    autotune.load()


def _plan_tiles(L, spec_stages, nst, xs, seed):
    keep, ins = [], []
    for x in xs:
        t, m = dev_image(x)
        keep.append(t)
        ins.append(m)
    ia = _abi.images(ins)
    outs = _abi.images([_abi.MPImage() for _ in xs])
    _abi.check(L.mpk_pipeline_shapes(spec_stages, nst, ia, outs, len(xs), seed, 0))
    keep += [alloc_like(outs[i]) for i in range(len(xs))]
    plan = C.c_void_p()
    _abi.check(L.mpk_plan_create(spec_stages, nst, ia, outs, len(xs), seed, 0, None, C.byref(plan)))
    res = []
    for i in range(L.mpk_plan_num_launches(plan)):
        kind, tiles = C.c_int(), C.c_int()
        L.mpk_plan_launch_info(plan, i, C.byref(kind), None, C.byref(tiles), None)
        res.append((kind.value, tiles.value))
    _abi.check(L.mpk_plan_destroy(plan))
    torch.cuda.synchronize()
    return res


def test_tuned_geometry_changes_the_plan_and_stays_exact(gpu, clean):
    L = clean
    rng = np.random.default_rng(41)
    # one streaming-gaussian launch big enough that rows per work item are
    # not at their floor (32 rows)
    big = [rng.random((900, 900, 3), dtype=np.float32) for _ in range(12)]
    gstages = _abi.stages(_abi.stage("gaussian", 2.0))
    xs = [rng.random((int(h), int(w), 3), dtype=np.float32)
          for h, w in rng.integers(40, 700, size=(10, 2))]
    # the built-in geometry (the loaded table may already set some knobs)
    L.mpk_tune_clear()
    base = dict(_plan_tiles(L, gstages, 1, big, 0))
    settings = [(8, 0, 1), (8, 0, 16), (8, 2, 64), (8, 1, 1), (5, 1, 1)]
    for kind, param, value in settings:
        L.mpk_tune_clear()
        _abi.check(L.mpk_tune_set_kernel(kind, param, value))
        got = C.c_int()
        _abi.check(L.mpk_tune_get_kernel(kind, param, C.byref(got)))
        assert got.value == value
        tiles = dict(_plan_tiles(L, gstages, 1, big, 0))
        if (kind, param) in ((8, 0), (8, 2)):
            # work items of the streaming gaussian follow the setting
            assert tiles[8] != base[8], (kind, param, value, tiles, base)
        check_spec([dict(op="gaussian", lo=(2.0,))], big[:2])
        check_spec(RAGGED, xs, seed=5)


def test_kernel_setting_validation(gpu, clean):
    L = clean
    assert L.mpk_tune_set_kernel(3, 0, 1) == _abi.MP_ERROR_INVALID_ARGS      # not a persistent kind
    assert L.mpk_tune_set_kernel(5, 0, 4) == _abi.MP_ERROR_INVALID_ARGS      # items: streaming gaussian only
    assert L.mpk_tune_set_kernel(8, 2, 60) == _abi.MP_ERROR_INVALID_ARGS     # strip: multiple of 8 from 64
    assert L.mpk_tune_set_kernel(8, 1, -1) == _abi.MP_ERROR_INVALID_ARGS
    assert L.mpk_tune_set_fuse(2) == _abi.MP_ERROR_INVALID_ARGS


def test_search_runs_on_a_small_batch(gpu, clean):
    entries = autotune.tune_kernels(ragged_images=6, uniform_images=2)
    assert entries[0]["fuse"] in (0, 1) and set(entries[0]["ms"]) == {"fused", "split"}
    kinds = {(e["kernel_kind"], e["param"]) for e in entries[1:]}
    assert kinds == {(k, p) for k, p, _ in autotune.KERNEL_CANDIDATES}
    for e in entries[1:]:
        cand = [v for k, p, vs in autotune.KERNEL_CANDIDATES if (k, p) == (e["kernel_kind"], e["param"]) for v in vs]
        assert e["value"] in cand
