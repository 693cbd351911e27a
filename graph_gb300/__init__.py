"""graph_gb300 — GB300-native force-layout engine for cosmos.gl's Graph simulation.

The compute path is the CUDA library built from graph_gb300/csrc (sm_103a),
reached through the C ABI in include/cgl.h.  `Graph` mirrors the reference's
simulation surface; `Engine` is the thin typed binding of the C ABI.
Importing the package does not load the library; creating an Engine does, and
raises if the library is missing or no CUDA device is usable.
"""
from . import _abi  # noqa: F401

__all__ = ["Graph", "Engine", "load_library"]


def __getattr__(name):
    if name == "Graph":
        from .graph import Graph
        return Graph
    if name == "Engine":
        from .engine import Engine
        return Engine
    if name == "load_library":
        from .engine import load_library
        return load_library
    raise AttributeError(name)
