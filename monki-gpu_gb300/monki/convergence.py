"""Precision-based stopping rules shared by every transport backend.

``AMFConvergence`` / ``AMFMoments`` / ``AMFStopping`` follow the reference
(python/monki/convergence.py:10-152): online (Welford) moments of each round's path and
weight sums, the delta-method standard error of the layer AMF ratio with the
numerator/denominator covariance kept, and a stop only after ``consecutive_checks``
passing checks at multiples of ``check_every`` from ``minimum_rounds`` on.

``RadianceConvergence`` adds the radiance rule the box-cloud workload needs: stop when
the round standard error of I is below ``relative_error`` x |I| in every pixel and view,
with the same standard-error formula the driver reports (simulation.py:131-144).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .execution.tallies import BatchControls, RawTallies


@dataclass(frozen=True)
class AMFConvergence:
    """Stop when every physical layer/pixel/view AMF has relative SE below the target."""

    relative_error: float = 0.01
    minimum_rounds: int = 128
    check_every: int = 32
    consecutive_checks: int = 3

    def __post_init__(self):
        if not np.isfinite(self.relative_error) or not 0 < self.relative_error < 1:
            raise ValueError("relative_error must be finite and in (0, 1)")

        for name in ("minimum_rounds", "check_every", "consecutive_checks"):
            value = getattr(self, name)

            if type(value) is not int or value < 1:
                raise ValueError(f"{name} must be a positive integer")

        if self.minimum_rounds < 32:
            raise ValueError("minimum_rounds must be at least 32")


@dataclass(frozen=True)
class RadianceConvergence(AMFConvergence):
    """Stop when SE(I) < relative_error * |I| in every pixel and view."""


class AMFMoments:
    """Online covariance of per-round path and weight sums; memory is constant in rounds."""

    def __init__(self):
        self.count = 0
        self.path_mean = self.weight_mean = None
        self.path_m2 = self.weight_m2 = self.covariance = None

    def add(self, batch: RawTallies) -> None:
        """Add one complete round, excluding the vacuum layer."""

        if batch.weighted_paths is None or batch.weights is None:
            raise ValueError("AMF stopping requires layer path diagnostics")

        paths = batch.weighted_paths[:, :, :-1, :]
        weights = batch.weights[:, :, None, :]

        if not np.all(np.isfinite(paths)) or not np.all(np.isfinite(weights)):
            raise ValueError("Nonfinite AMF tallies")

        if self.count == 0:
            self.path_mean = np.zeros_like(paths)
            self.weight_mean = np.zeros_like(weights)
            self.path_m2 = np.zeros_like(paths)
            self.weight_m2 = np.zeros_like(weights)
            self.covariance = np.zeros_like(paths)

        self.count += 1
        dp = paths - self.path_mean
        dw = weights - self.weight_mean
        self.path_mean += dp / self.count
        self.weight_mean += dw / self.count
        self.path_m2 += dp * (paths - self.path_mean)
        self.weight_m2 += dw * (weights - self.weight_mean)
        self.covariance += dp * (weights - self.weight_mean)

    def estimate(self, thickness):
        """AMF and its standard error per (x, y, layer, view)."""

        if self.count < 2:
            raise ValueError("At least two rounds are needed for AMF uncertainty")

        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = self.path_mean / self.weight_mean
            # sum((P - ratio W)^2) from the centred moments.
            residual = self.path_m2 - 2 * ratio * self.covariance + ratio**2 * self.weight_m2
            scale = self.path_m2 + 2 * np.abs(ratio * self.covariance) + ratio**2 * self.weight_m2

            if np.any(residual < -128 * np.finfo(float).eps * np.maximum(scale, 1e-300)):
                raise ArithmeticError("Negative AMF variance exceeds roundoff")

            error = np.sqrt(np.maximum(residual, 0) / (self.count - 1) / self.count)
            error /= self.weight_mean
            shape = np.asarray(thickness)[None, None, :, None]
            return ratio / shape, error / shape


class RadianceMoments:
    """Running sums of normalized round radiance and its square (simulation.py:90-93)."""

    def __init__(self, photons_per_column: int):
        self.photons = photons_per_column
        self.count = 0
        self.total = self.squares = None

    def add(self, batch: RawTallies) -> None:
        values = batch.stokes / self.photons

        if self.total is None:
            self.total = np.zeros_like(values)
            self.squares = np.zeros_like(values)

        self.count += 1
        self.total += values
        self.squares += values**2

    def estimate(self):
        """Mean radiance and the standard error of the mean over rounds."""

        if self.count < 2:
            raise ValueError("At least two rounds are needed for radiance uncertainty")

        n = self.count
        mean = self.total / n
        variance = np.maximum(self.squares - self.total**2 / n, 0) / (n - 1)
        return mean, np.sqrt(variance) / np.sqrt(n)


class AMFStopping:
    """Schedule rounds in groups of ``check_every`` and stop after sustained precision.

    The rounds before the first check (the first group end at or after
    ``minimum_rounds``) are requested as one group: the checks, and so every result, are
    those of the reference schedule, and a GPU backend runs them in one dispatch instead
    of draining its photon pool once per group.
    """

    def __init__(self, policy: AMFConvergence, thickness):
        self.policy = policy
        self.thickness = thickness
        self.moments = AMFMoments()
        self.history: list[dict] = []
        self.streak = 0
        self.converged = False

    def _relative(self):
        amf, error = self.moments.estimate(self.thickness)
        return np.divide(error, np.abs(amf), out=np.full_like(error, np.inf), where=amf != 0)

    def _add(self, batch: RawTallies) -> None:
        self.moments.add(batch)

    def groups(self, rounds: int):
        """(first, last, checked) round groups of the schedule."""

        first = 1

        for start in range(1, rounds + 1, self.policy.check_every):
            end = min(start + self.policy.check_every - 1, rounds)

            if end < self.policy.minimum_rounds and end < rounds:
                continue  # no check before the minimum: extend the first group

            yield first, end, end >= self.policy.minimum_rounds
            first = end + 1

    def check(self, end: int) -> None:
        """Judge the moments after round ``end`` and update the streak."""

        relative = self._relative()
        maximum = float(np.max(relative))
        passed = bool(np.all(np.isfinite(relative)) and maximum < self.policy.relative_error)
        self.streak = self.streak + 1 if passed else 0
        self.converged = self.streak >= self.policy.consecutive_checks
        self.history.append(
            {
                "rounds": end,
                "max_relative_se": maximum if np.isfinite(maximum) else None,
                "below_target": passed,
                "streak": self.streak,
            }
        )

    def rounds_estimate(self):
        """Rounds the target needs by the last check (the standard error falls as one over the
        square root of the rounds), or None before a check or with an infinite error."""

        if not self.history or self.history[-1]["max_relative_se"] is None:
            return None
        last = self.history[-1]
        return last["rounds"] * (last["max_relative_se"] / self.policy.relative_error) ** 2

    def load(self, statistics: dict) -> None:
        """Take the moments from device round statistics (``CUDA.statistics``)."""

        m = self.moments
        m.count = statistics["rounds"]
        m.path_mean = statistics["path_mean"][:, :, :-1, :]
        m.path_m2 = statistics["path_m2"][:, :, :-1, :]
        m.covariance = statistics["covariance"][:, :, :-1, :]
        m.weight_mean = statistics["weight_mean"][:, :, None, :]
        m.weight_m2 = statistics["weight_m2"][:, :, None, :]

    def batches(self, backend, case):
        for first, end, checked in self.groups(case.rounds):
            requests = [BatchControls(i, case.photons_per_column) for i in range(first, end + 1)]
            batches = backend.run_batches(requests)

            if len(batches) != len(requests):
                raise ValueError("Backend returned the wrong number of statistical rounds")

            for request, batch in zip(requests, batches, strict=True):
                if not isinstance(batch, RawTallies) or batch.controls != request:
                    raise ValueError("Backend returned invalid round tallies")

                self._add(batch)
                yield batch

            if checked:
                self.check(end)

                if self.converged:
                    return


class RadianceStopping(AMFStopping):
    """The same schedule, judged on SE(I)/|I| over every pixel and view."""

    def __init__(self, policy: RadianceConvergence, photons_per_column: int):
        super().__init__(policy, None)
        self.moments = RadianceMoments(photons_per_column)

    def load(self, statistics: dict) -> None:
        self.moments.count = statistics["rounds"]
        self.moments.total = statistics["sum"]
        self.moments.squares = statistics["squares"]

    def _relative(self):
        mean, error = self.moments.estimate()
        intensity, se = mean[0], error[0]
        return np.divide(se, np.abs(intensity), out=np.full_like(se, np.inf), where=intensity != 0)
