"""GB300-native physical-optics far-field engine (the PO path of WaveFiber3d).

The compute path is libwavepo.so (hand-written CUDA for sm_103a behind the C
ABI in include/wavepo.h).  This package holds the Python mirror of the
reference's operators (api), the ctypes binding (_lib), input geometry
(geometry), angular grids (grids) and the in-tree build (build).
"""
from . import geometry, grids  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # the CUDA-backed API is imported on first use so that geometry/grids work without the library
    if name in ("api", "Solver", "Config", "Illumination"):
        import importlib
        mod = importlib.import_module(__name__ + ".api")
        return mod if name == "api" else getattr(mod, name)
    raise AttributeError(name)
