"""Lifecycle shared by interchangeable transport implementations.

The same strategy interface as the reference (python/monki/execution/backend.py:10-72):
``prepare`` retains scene tables, ``run_batch`` returns owned raw tallies of one
statistical round, ``run_batches`` may schedule several rounds together but preserves
order, and ``close`` is idempotent. The driver owns rounds, convergence and
normalization.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from types import TracebackType

from ..output import SimulationResult


class Backend(ABC):
    """Strategy consumed by ``monki.simulate``."""

    metadata: SimulationResult | None = None
    provenance: dict = {}

    @abstractmethod
    def prepare(self, scene: object) -> None:
        """Validate and retain scene tables; repreparing replaces prior state."""

        raise NotImplementedError

    @abstractmethod
    def run_batch(self, controls: object) -> object:
        """Return owned, unnormalized tallies of one complete round."""

        raise NotImplementedError

    def run_batches(self, controls: list) -> list:
        """One owned result per requested round, in order."""

        return [self.run_batch(request) for request in controls]

    @abstractmethod
    def close(self) -> None:
        """Release resources; safe before preparation and on repeated calls."""

        raise NotImplementedError

    def __enter__(self):
        return self

    def __exit__(
        self,
        exception_type: type[BaseException] | None,
        exception: BaseException | None,
        traceback: TracebackType | None,
    ) -> None:
        self.close()
