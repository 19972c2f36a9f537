"""millipyde_gb300 -- GB300-native (sm_103a) drop-in for millipyde's image hot path.

Same Python surface as the reference module `millipyde`
(src/millipyde_module.c:112-120, :225-299): gpuarray, gpuimage, Operation,
Pipeline, Generator, Device, device_count, get_current_device, best_device,
image_from_path, images_from_path and DEVICE_COUNT.  `import millipyde_gb300
as millipyde` is the switch.

The compute path is the compiled extension `_millipyde` over the C-ABI
library `libmillipyde_gb300.so`; there is no CPU fallback.  Importing fails
with ImportError when the extension has not been built (run
`python millipyde_gb300/_build.py`).
"""
from __future__ import annotations

import os as _os

try:
    from ._millipyde import (  # noqa: F401
        DEVICE_COUNT,
        Device,
        Generator,
        Operation,
        Pipeline,
        best_device,
        device_count,
        get_current_device,
        gpuarray,
        gpuimage,
        seed,
        synchronize,
    )
except ImportError as e:  # pragma: no cover - exercised only without a build
    raise ImportError(
        "millipyde_gb300: the compiled extension is missing (%s); build it with "
        "`python millipyde_gb300/_build.py`" % e
    ) from e

from ._io import image_from_path, images_from_path  # noqa: E402,F401

try:  # tuned gaussian tiles for this GPU (no-op without a GPU or a table)
    from . import autotune as _autotune

    _autotune.load()
except (OSError, ValueError, KeyError):  # pragma: no cover
    pass

LIBRARY_PATH = _os.path.join(_os.path.dirname(__file__), "libmillipyde_gb300.so")

__all__ = [
    "DEVICE_COUNT",
    "Device",
    "Generator",
    "Operation",
    "Pipeline",
    "best_device",
    "device_count",
    "get_current_device",
    "gpuarray",
    "gpuimage",
    "image_from_path",
    "images_from_path",
    "seed",
    "synchronize",
]
