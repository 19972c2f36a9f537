"""GPU: failure paths, made to happen without faulting the GPU.

The reference ended the process on any failed HIP call
(src/include/millipyde_hip_util.h:7-16).  Here a failure is a status the
caller reads, and the device context stays usable afterwards:
  - a device-side wait that gives up (the bounded mbarrier wait every kernel
    uses, on a barrier phase that nothing completes) reports
    MP_ERROR_KERNEL_TIMEOUT and the error word is cleared again;
  - a device allocation that fails (injected on the host: requests above a
    limit fail as if the device were full) returns MP_ERROR_OUT_OF_MEMORY and
    leaves the object as it was.
"""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs, obj_free, obj_from_host, obj_to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_bounded_wait_times_out_and_context_survives(gpu):
    L = _abi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # ~2048 fast polls then ~2000 polls of about 1 us: a few ms
    assert L.mpdev_selftest_wait_timeout(4096, stream) == _abi.MP_ERROR_KERNEL_TIMEOUT
    # the error word was cleared: the next check reports nothing
    _abi.check(L.mpdev_synchronize())
    # and the context still runs real work correctly
    x = np.random.default_rng(1).random((33, 45, 3), dtype=np.float32)
    o = obj_from_host(x)
    try:
        _abi.check(L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(2.0))))
        _abi.check(L.mpdev_synchronize())
        assert maxabs(obj_to_host(o), O.gaussian(x, 2.0)) <= TOL
    finally:
        obj_free(o)


def test_selftest_rejects_bad_limits(gpu):
    L = _abi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.mpdev_selftest_wait_timeout(0, stream) == _abi.MP_ERROR_INVALID_ARGS
    assert L.mpdev_selftest_wait_timeout(1 << 22, stream) == _abi.MP_ERROR_INVALID_ARGS


def test_allocation_failure_leaves_object_unchanged(gpu):
    L = _abi.lib()
    x = np.random.default_rng(2).random((64, 80, 3), dtype=np.float32)
    o = obj_from_host(x)
    try:
        ptr, nd = o.device_data, o.ndims
        dims = [o.dims[i] for i in range(2 * nd)]
        L.mpdev_set_alloc_limit(1024)
        try:
            assert L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(1.5))) == _abi.MP_ERROR_OUT_OF_MEMORY
            assert L.mpimg_rotate(C.byref(o), C.byref(_abi.RotateArgs(12.0))) == _abi.MP_ERROR_OUT_OF_MEMORY
            assert L.mpimg_transpose(C.byref(o), None) == _abi.MP_ERROR_OUT_OF_MEMORY
        finally:
            L.mpdev_set_alloc_limit(0)
        assert o.device_data == ptr and o.ndims == nd
        assert [o.dims[i] for i in range(2 * nd)] == dims
        assert np.array_equal(obj_to_host(o), x)
        # with the limit gone the same call succeeds
        _abi.check(L.mpimg_gaussian(C.byref(o), C.byref(_abi.GaussianArgs(1.5))))
        assert maxabs(obj_to_host(o), O.gaussian(x, 1.5)) <= TOL
    finally:
        obj_free(o)


def test_batch_allocation_failure_is_a_status(gpu):
    """The fused batch allocates its job tables and intermediates from the
    pool; a failure there is MP_ERROR_OUT_OF_MEMORY, and the same batch runs
    once the limit is lifted."""
    L = _abi.lib()
    x = torch.rand(2, 48, 48 * 3, device="cuda")
    y = torch.full((2, 48, 48), 5.0, device="cuda")
    st = _abi.stages(_abi.stage("rgb2grey"), _abi.stage("gaussian", 2.0), _abi.stage("rotate", 9.0))
    ins = _abi.images([_abi.image(x[i].data_ptr(), 48, 48, 3, 576) for i in range(2)])
    outs = _abi.images([_abi.image(y[i].data_ptr(), 48, 48, 1, 192) for i in range(2)])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.mpdev_set_alloc_limit(64)
    try:
        assert L.mpk_pipeline_run(st, 3, ins, outs, 2, 0, 0, stream) == _abi.MP_ERROR_OUT_OF_MEMORY
    finally:
        L.mpdev_set_alloc_limit(0)
    torch.cuda.synchronize()
    assert bool((y == 5.0).all())
    _abi.check(L.mpk_pipeline_run(st, 3, ins, outs, 2, 0, 0, stream))
    torch.cuda.synchronize()
    xs = x[0].view(48, 48, 3).cpu().numpy()
    ref = O.run_ops(xs, [("rgb2grey",), ("gaussian", 2.0), ("rotate", 9.0)])
    assert maxabs(y[0].cpu().numpy(), ref) <= TOL
