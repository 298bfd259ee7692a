"""GB300-native per-stage DG shallow-water operator (oceano's perform_stage_hydro).

The product is the CUDA library ``liboceano_gpu.so`` behind the C ABI of
``include/oceano_gpu.h``; this package holds its build script, the ctypes
binding, the host-side mirror of the reference operator interface, the
integrators that drive it and the synthetic mesh/initial-data generators.
"""
from .mesh import Mesh, QuadForest, channel_mesh, random_hp_mesh, uniform_mesh, vortex_mesh  # noqa: F401

__all__ = ["Mesh", "QuadForest", "uniform_mesh", "vortex_mesh", "channel_mesh", "random_hp_mesh"]
