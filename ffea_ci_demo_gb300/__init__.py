"""GB300-native (sm_103a) engine for FFEA's per-timestep blob update.

The product is the CUDA library behind the C ABI in include/ffea_gpu.h;
``lib.Blob`` is the Python face of that ABI and ``mesh`` writes and
generates the reference's structure files.
"""
from . import mesh  # noqa: F401

__all__ = ["mesh", "lib", "build"]
