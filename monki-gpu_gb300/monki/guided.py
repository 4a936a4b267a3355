"""Importance-guided transport settings.

The guided method keeps the analog estimator's expectation exactly and changes only its
variance and cost (python/monki/convergence.py's stopping rules and the statistics of
simulation.py:73-156 apply unchanged):

* detector directional importance sampling (DDIS; Buras & Mayer 2011, "Efficient
  unbiased variance reduction techniques for Monte Carlo simulations of radiative transfer
  in cloudy atmospheres: The solution", JQSRT 112, 434-447): at a particle scatter, with
  probability ``epsilon`` the new direction is drawn about one of the view directions
  from the particle's own phase-function proposal; the weight is multiplied by
  p_analog / ((1 - epsilon) p_analog + epsilon p_detector). ``cap`` limits it to photons
  lighter than ``cap``: the factor reaches 1 / (1 - epsilon) on the analog branch, so
  without a cap a photon that keeps that branch through a long history in a thick cloud
  grows heavy and the estimator, though still unbiased, gets tails too heavy for its
  standard error to mean much;
* Russian roulette after every scatter: a photon lighter than the roulette weight W of
  its cell survives with probability weight / W, at weight W. W = ``roulette`` times an
  optional per-cell scale (``CUDA.set_roulette_scale``), which the learned importance
  model supplies;
* splitting, the upper bound of the same weight window: after an atmospheric scatter a
  photon heavier than ``split`` x W continues as n = min(weight / W, 8) copies of weight /
  n, each with its own random stream, run one after another in the photon's slot (at most
  8 waiting per history, which also bounds n). Photons that reach important cells
  (small W) with weight gathered in unimportant ones are spread over more histories.
  ``split`` = 0 turns it off; it needs a roulette weight and a scene without layer paths.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Guided:
    epsilon: float = 0.0
    roulette: float = 1.0
    cap: float = 0.0
    split: float = 0.0

    def __post_init__(self):
        for name, low, high, closed in (("epsilon", 0.0, 1.0, False), ("roulette", 0.0, 1.0, True)):
            value = getattr(self, name)
            if not isinstance(value, (int, float)) or not np.isfinite(value) or value < low or (
                value > high if closed else value >= high
            ):
                raise ValueError(f"{name} must be in [{low}, {high}{']' if closed else ')'}")

        if not isinstance(self.cap, (int, float)) or not np.isfinite(self.cap) or self.cap < 0:
            raise ValueError("cap must be finite and non-negative (0 = no cap)")

        if not isinstance(self.split, (int, float)) or not np.isfinite(self.split) or not (
            self.split == 0 or self.split >= 1
        ):
            raise ValueError("split must be 0 (off) or at least 1")

        if self.split and not self.roulette:
            raise ValueError("splitting needs a roulette weight")

    def config(self) -> str:
        """The create-time configuration items of the native session."""

        return (f",epsilon={float(self.epsilon)!r},roulette={float(self.roulette)!r},cap={float(self.cap)!r}"
                + (f",split={float(self.split)!r}" if self.split else ""))

    def oracle(self) -> tuple[float, float, float, float]:
        """The same settings as the CPU oracle's guide argument."""

        return (float(self.epsilon), float(self.roulette), float(self.cap), float(self.split))

    def describe(self) -> dict:
        return {"epsilon": self.epsilon, "roulette": self.roulette, "cap": self.cap, "split": self.split}
