"""GB300-native DCGrid adaptive-grid simulation step.

The compute path is the CUDA library libdcgrid_gb300.so (C ABI in
include/dcg.h); this package holds its sources (csrc/), the build script and
a ctypes host API mirroring the reference's simulation interface.
"""
from . import capi
from .capi import DcgInfo, DcgParams, DcgStats, DcgTuning
from .sim import (Batch, DcgError, FluidSimulationDCGrid, FluidSimulationUniform, Simulation,
                  default_params, lib)

__all__ = ["capi", "DcgParams", "DcgInfo", "DcgStats", "DcgTuning", "DcgError", "Simulation", "Batch",
           "FluidSimulationDCGrid", "FluidSimulationUniform", "default_params", "lib"]
