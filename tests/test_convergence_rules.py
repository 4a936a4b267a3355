"""Stopping-policy validation and the AMF rule's edge cases, as the reference's own
convergence tests hold them (tests/unit/test_convergence.py:30-89)."""

from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.parametrize(
    "settings",
    [
        {"relative_error": 0},
        {"relative_error": 1},
        {"relative_error": np.nan},
        {"minimum_rounds": 31},
        {"check_every": 0},
        {"consecutive_checks": True},
        {"consecutive_checks": 0},
    ],
)
@pytest.mark.parametrize("policy", ["amf", "radiance"])
def test_invalid_stopping_policy(settings, policy):
    from monki import AMFConvergence, RadianceConvergence

    with pytest.raises(ValueError):
        (AMFConvergence if policy == "amf" else RadianceConvergence)(**settings)


def test_zero_amf_cannot_satisfy_relative_precision():
    from monki import AMFConvergence
    from monki.convergence import AMFStopping
    from monki.execution.tallies import RawTallies

    class Synthetic:
        def run_batches(self, requests):
            return [RawTallies(r, np.ones((3, 1, 1, 1)), np.zeros((1, 1, 2, 1)), np.ones((1, 1, 1))) for r in requests]

    case = type("Case", (), {"rounds": 32, "photons_per_column": 100})
    stopping = AMFStopping(AMFConvergence(minimum_rounds=32, consecutive_checks=1), np.array([1.0]))
    list(stopping.batches(Synthetic(), case()))
    assert not stopping.converged
    assert stopping.history[-1]["max_relative_se"] is None


def test_constant_amf_converges_at_the_first_checks():
    from monki import AMFConvergence
    from monki.convergence import AMFStopping
    from monki.execution.tallies import RawTallies

    class Synthetic:
        def run_batches(self, requests):
            return [RawTallies(r, np.ones((3, 1, 1, 1)), np.ones((1, 1, 2, 1)), np.ones((1, 1, 1))) for r in requests]

    case = type("Case", (), {"rounds": 256, "photons_per_column": 100})
    stopping = AMFStopping(AMFConvergence(minimum_rounds=32, check_every=16, consecutive_checks=2), np.array([1.0]))
    assert len(list(stopping.batches(Synthetic(), case()))) == 48
    assert stopping.converged
    assert [h["streak"] for h in stopping.history] == [1, 2]
