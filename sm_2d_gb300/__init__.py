"""GB300 (sm_103a) build of the SM_2D deterministic phase-space transport step.

The compute path is libsm2d.so (hand-written CUDA kernels behind a C ABI,
include/sm2d.h); this package is its host-side mirror.
"""
from .surrogate import Surrogate  # noqa: F401
from .runtime import (Config, Sm2dError, Transport, angular_grid, bragg_metrics, bragg_peak_row,  # noqa: F401
                      depth_dose, energy_grid_log, energy_grid_piecewise, fermi_eyges, lib, range_lut,
                      write_dose_2d, write_pdd, DEFAULT_ENERGY_GROUPS, LAYOUT_B128, LAYOUT_REF)

__all__ = ["Config", "Transport", "Surrogate", "Sm2dError", "lib", "energy_grid_log", "energy_grid_piecewise",
           "angular_grid", "range_lut", "fermi_eyges", "depth_dose", "bragg_peak_row", "bragg_metrics",
           "write_dose_2d", "write_pdd",
           "DEFAULT_ENERGY_GROUPS", "LAYOUT_REF", "LAYOUT_B128"]
