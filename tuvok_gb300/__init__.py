"""tuvok_gb300 -- Tuvok's volume-rendering hot path on a GB300 (sm_103a).

The product is ``libtvk.so`` (C ABI in ``include/tvk.h``): GPU bricking with
ghost voxels, per-brick min/max and histograms, and the brick-by-brick
GLRaycaster ray march.  This package holds the build recipe, a ctypes binding
and a thin Python mirror of Tuvok's AbstrRenderer / dataset interfaces.
"""
from ._native import TvkError, lib  # noqa: F401  (raises if libtvk.so is missing)
from .renderer import (Batch, Pool, Renderer, TransferFunction1D, Volume,  # noqa: F401
                       generate_volume_device, read_uvf_blocks)

__all__ = ["Batch", "Pool", "Renderer", "TransferFunction1D", "Volume", "TvkError",
           "generate_volume_device", "lib", "read_uvf_blocks"]
