"""GB300 (sm_103a) stochastic progressive photon mapping: a drop-in for glslppm's GPU path.

The compute path is the native library ``_lib/libsppm.so`` (hand-written CUDA kernels behind the C
ABI of ``include/sppm.h``); this package is its host-side mirror.  Importing the package fails with
``NativeLibraryMissing`` when the library has not been built.
"""
from .native import NativeLibraryMissing, SppmError, device_count  # noqa: F401
from .renderer import (Mesh, Renderer, default_config, look_at, pinned_empty, scene_from_arrays,  # noqa: F401
                       tune_hash_slots, write_image)
from . import native, scenes  # noqa: F401
from .batch import Batch, PreparedScene, PreparedState, Server  # noqa: F401

__all__ = ["Batch", "PreparedScene", "PreparedState", "Server", "Mesh", "Renderer", "default_config", "look_at", "pinned_empty", "scene_from_arrays", "tune_hash_slots", "write_image", "SppmError",
           "NativeLibraryMissing", "device_count", "native", "scenes"]
