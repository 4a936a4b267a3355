"""Transport backends behind the shared ``Backend`` strategy interface."""

from .backend import Backend
from .cuda import CUDA
from .tallies import BatchControls, RawTallies

__all__ = ["Backend", "CUDA", "BatchControls", "RawTallies"]
