"""GB300-native sort-middle rasterizer with the host API of tcoppex/cudaraster-linux.

The package holds the CUDA sources (csrc/), the build recipe (build.py), the
ctypes binding of the C ABI (_lib.py), the Python mirror of the reference's
host classes (raster.py) and the seeded synthetic scenes (scenes.py). The
directory name contains a hyphen, so import it with
importlib.import_module("cudaraster-linux_gb300").
"""
from .raster import (Buffer, CudaRaster, CudaSurface, DebugParams, RasterError, Stats, clear_depth_from_float,  # noqa: F401
                     color_to_abgr, encode_depth, pipe_info, pipe_names, write_ppm)
