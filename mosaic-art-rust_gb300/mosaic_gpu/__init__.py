"""mosaic_gpu -- Python binding of the GB300 tile matching-and-placement library.

The compute path is the CUDA library behind include/mosaic_gpu.h; this package
binds it with ctypes (``_capi``), builds it (``build``), generates seeded
synthetic inputs (``synth``) and assembles whole jobs (``job``).
"""
from . import build
from ._capi import (MG_SIM_FULL, MG_SIM_TRIANGULAR, Context, MosaicError, check, color_adjustment_new,
                    improvement_percentage, library_path, load)

__all__ = ["build", "Context", "MosaicError", "check", "load", "library_path", "MG_SIM_FULL", "MG_SIM_TRIANGULAR",
           "color_adjustment_new", "improvement_percentage"]
