"""CPU: Python API validation that needs no device (the reference's
ValueError cases, tests/millipyde_tests.py:140-202, :259-309)."""
import numpy as np
import pytest

import millipyde_gb300 as mp
from millipyde_gb300 import Operation


def test_module_surface():
    for name in ("gpuarray", "gpuimage", "Operation", "Pipeline", "Generator", "Device",
                 "device_count", "get_current_device", "best_device", "image_from_path",
                 "images_from_path", "DEVICE_COUNT"):
        assert hasattr(mp, name), name
    for meth in ("rgb2gray", "rgb2grey", "rgba2gray", "rgba2grey", "transpose", "gaussian",
                 "random_gaussian", "brightness", "random_brightness", "adjust_gamma",
                 "random_adjust_gamma", "colorize", "random_colorize", "fliplr", "rotate",
                 "random_rotate", "clone"):
        assert hasattr(mp.gpuimage, meth), meth


def test_create_invalid_operation():
    with pytest.raises(ValueError):
        Operation()


@pytest.mark.parametrize("p", [7, 1, 0, -1, 1.0, 0.0, -0.5, 1.5, "0.5"])
def test_invalid_probability(p):
    with pytest.raises(ValueError):
        Operation(lambda: None, probability=p)


def test_invalid_operation_kwarg():
    with pytest.raises(ValueError):
        Operation("rgb2grey", probability=0.5, other=1)


def test_run_operation():
    def add(x, y):
        return x + y
    assert Operation(add, 4, 6).run() == 10
    assert Operation(add, 4, 6, probability=0.6) is not None


def test_run_on_needs_string_method():
    with pytest.raises(ValueError):
        Operation(lambda: 1).run_on(object())
    with pytest.raises(ValueError):
        Operation("no_such_method").run_on(object())


def test_create_pipeline_empty():
    p = mp.Pipeline([], [])
    assert p is not None
    p.run()


@pytest.mark.parametrize("args", [(1, []), ([], 1), (np.array([1, 2, 3]), []), ([], np.array([1, 2]))])
def test_create_invalid_pipeline(args):
    with pytest.raises(ValueError):
        mp.Pipeline(*args)


def test_pipeline_bad_kwargs():
    with pytest.raises(ValueError):
        mp.Pipeline([], [], device=5.3)
    with pytest.raises(ValueError):
        mp.Pipeline([], [], device="nah")
    with pytest.raises(ValueError):
        mp.Pipeline([], [], device=0, unused="test")
    with pytest.raises(ValueError):
        mp.Pipeline([1], [])
    with pytest.raises(ValueError):
        mp.Pipeline([], ["rgb2grey"])


def test_generator_validation():
    with pytest.raises(ValueError):
        mp.Generator(5, [])
    with pytest.raises(ValueError):
        mp.Generator([], 5)
    with pytest.raises(ValueError):
        mp.Generator([], [], outputs=-1)
    with pytest.raises(ValueError):
        mp.Generator([], [], outputs=2.0)
    with pytest.raises(ValueError):
        mp.Generator([], [], return_to_host=1)
    with pytest.raises(ValueError):
        mp.Generator([], [], bogus=1)
    g = mp.Generator([], [], outputs=0)
    assert list(g) == []


def test_pipeline_stage_argument_errors():
    p = mp.Pipeline([], [Operation("gaussian", "x")])
    with pytest.raises(TypeError):
        p.run()
    p = mp.Pipeline([], [Operation("brightness", 1.5)])
    with pytest.raises(ValueError):
        p.run()
    p = mp.Pipeline([], [Operation("gaussian", -1.0)])
    with pytest.raises(ValueError):
        p.run()


def test_no_device_raises_runtime_error_not_crash():
    if mp.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        mp.gpuarray([1, 2, 3])
    with pytest.raises(ValueError):
        mp.gpuarray(None)
    with pytest.raises(TypeError):
        mp.gpuarray()
    with pytest.raises(ValueError):
        mp.gpuimage(np.array([1, 2, 3]))


def test_seed_and_counter():
    assert 0.0 <= mp._millipyde._counter_uniform(1, 2, 3, 0) < 1.0
    mp.seed(3)


def test_autograd_wrapper_validates_on_cpu():
    torch = pytest.importorskip("torch")
    from millipyde_gb300.autograd import pipeline
    with pytest.raises(TypeError):
        pipeline(torch.zeros(1, 4, 4, 3), [("rotate", 1.0)])
