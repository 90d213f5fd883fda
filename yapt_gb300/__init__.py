"""yapt_gb300: GB300-native spectral path-tracing integrators (uni / NEE / BDPT).

The compute path is libyaptgpu.so (CUDA for sm_103a behind the C ABI of
include/yapt_gpu.h); this package holds the Python-side scene description, the
seeded benchmark scenes and a thin handle on the native context. Importing it
does not need a GPU; creating a Context does, and fails loudly when the native
library or the device is missing.
"""
from . import _native  # noqa: F401
from .scene import Scene, CameraDesc, MATERIAL_DEFAULTS  # noqa: F401
from . import configs  # noqa: F401


def Context(device=0):
    from .runtime import Context as _Ctx
    return _Ctx(device)


__all__ = ["Context", "Scene", "CameraDesc", "configs", "MATERIAL_DEFAULTS"]
