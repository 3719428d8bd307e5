"""GB300-native Vertex Block Descent step (drop-in for Gaia's VBDPhysics step).

The compute path is libgaia_vbd.so (hand-written sm_103a CUDA behind a C ABI,
include/gaia_vbd.h). This package holds its ctypes binding, a Python mirror
of the reference's VBDPhysics entry points, the build recipe and the
synthetic-scene writer.
"""
from ._lib import GaiaError, lib  # noqa: F401
from .physics import VBDPhysics, color_greedy, color_mcs, write_coloring, write_t  # noqa: F401

__all__ = ["VBDPhysics", "GaiaError", "lib", "color_greedy", "color_mcs", "write_coloring", "write_t"]
