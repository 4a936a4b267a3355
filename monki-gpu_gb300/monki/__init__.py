"""MONKI photon transport on GB300: the reference's public API over sm_103a kernels.

Same entry points as the reference package (python/monki/__init__.py:3-9): ``simulate``,
``ReferenceCase``, ``AMFConvergence``, ``SimulationResult``; the transport backend is
``monki.execution.CUDA``. ``monki.scenes`` builds prepared synthetic scenes.
"""

from .convergence import AMFConvergence, RadianceConvergence
from .guided import Guided
from .input import ReferenceCase
from .output import SimulationResult
from .scenes import TransportScene
from .simulation import simulate

__all__ = [
    "AMFConvergence",
    "Guided",
    "RadianceConvergence",
    "ReferenceCase",
    "SimulationResult",
    "TransportScene",
    "simulate",
]
