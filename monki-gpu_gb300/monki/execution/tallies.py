"""Batch requests and owned tally buffers (python/monki/execution/tallies.py:8-32)."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class BatchControls:
    """One complete statistical round, numbered from one within a session."""

    round_index: int
    photons_per_column: int

    def __post_init__(self):
        for value in (self.round_index, self.photons_per_column):
            if type(value) is not int or not 0 < value < 2**31:
                raise ValueError("batch counts must be positive 32-bit integers")


@dataclass(frozen=True)
class RawTallies:
    """Unnormalized Fortran-order sums owned by the caller.

    ``stokes`` is (component, x, y, angle); ``weighted_paths`` is (x, y, layer, angle)
    including the vacuum layer; ``weights`` is (x, y, angle). ``orders`` (scattering-order
    diagnostics, when requested) holds ``single`` (component, x, y, angle) and
    ``locations`` / ``single_locations`` (component, x, y, layer, angle; layer 0 = the
    surface, then the physical layers).
    """

    controls: BatchControls
    stokes: np.ndarray
    weighted_paths: np.ndarray | None = None
    weights: np.ndarray | None = None
    orders: dict | None = None
