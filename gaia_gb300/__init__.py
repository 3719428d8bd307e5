"""GB300-native Vertex Block Descent step (drop-in for Gaia's VBDPhysics step and
the VBD path of its VBDClothSimulationFramework).

The compute path is libgaia_vbd.so (hand-written sm_103a CUDA behind a C ABI,
include/gaia_vbd.h and include/gaia_cloth.h). This package holds its ctypes
binding, Python mirrors of the reference's VBDPhysics and cloth framework entry
points, the build recipe and the synthetic-scene writer.
"""
from ._lib import GaiaError, lib  # noqa: F401
from .cloth import VBDClothSimulationFramework, color_trimesh  # noqa: F401
from .physics import VBDPhysics, color_gpu, color_greedy, color_mcs, write_coloring, write_t  # noqa: F401

__all__ = ["VBDPhysics", "VBDClothSimulationFramework", "GaiaError", "lib", "color_greedy", "color_mcs", "color_gpu",
           "color_trimesh", "write_coloring", "write_t"]
