"""Held lookahead groups in the device-statistics driver (monki.simulation._device_rounds).

A backend with held groups (run_held / fold_next) runs, after the first check, the rounds the
last check says are still needed in one dispatch and folds them one at a time. Checked here
on a host stand-in of the device statistics (the reference driver's fixed rounds of
tests/golden/driver_statistics.npz): the same rounds are folded, the same checks are made
and the product is the one of round-by-round dispatches, in fewer dispatches.
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _device_backend(golden, lookahead):
    from test_boundary import _fixed_backend

    base = _fixed_backend(golden)
    ppc = int(golden["photons_per_column"])

    class Device(type(base)):
        def __init__(self):
            super().__init__()
            self.lookahead = lookahead
            self.dispatches = 0
            self.rounds = 0
            shape = golden["stokes"].shape[1:]
            self.total, self.sum, self.squares = np.zeros(shape), np.zeros(shape), np.zeros(shape)
            self._held = []

        def device_statistics_available(self, photons_per_column):
            return True

        def held_capacity(self, photons_per_column):
            return 8

        def _fold(self, batch):
            x = batch.stokes
            n = x / ppc
            self.total += x
            self.sum += n
            self.squares += n * n
            self.rounds += 1
            return n.sum(axis=(1, 2, 3))

        def accumulate(self, controls):
            self.dispatches += 1
            return np.stack([self._fold(self.run_batch(c)) for c in controls])

        def run_held(self, controls):
            self.dispatches += 1
            self._held = [self.run_batch(c) for c in controls]

        def fold_next(self):
            return self._fold(self._held.pop(0))

        def statistics(self):
            return {"rounds": self.rounds, "total": self.total.copy(), "sum": self.sum.copy(),
                    "squares": self.squares.copy()}

    return Device()


def test_held_groups_fold_the_rounds_of_round_by_round_dispatches(tmp_path):
    from monki import RadianceConvergence, simulate
    from monki.convergence import RadianceStopping

    golden = dict(np.load(GOLDEN / "driver_statistics.npz"))
    rounds = golden["stokes"].shape[0]
    ppc = int(golden["photons_per_column"])
    case = type("Case", (), {"photons_per_column": ppc, "rounds": rounds, "backward": False})
    # A target the fixed rounds meet part way: the largest relative error after 48 rounds.
    probe = RadianceStopping(RadianceConvergence(0.5, minimum_rounds=32), ppc)
    x = golden["stokes"][:48] / ppc
    probe.moments.count, probe.moments.total, probe.moments.squares = 48, x.sum(0), (x * x).sum(0)
    target = float(np.max(probe._relative())) * 1.0001
    rule = RadianceConvergence(target, minimum_rounds=32, check_every=1, consecutive_checks=1)

    results, receipts, dispatches = {}, {}, {}
    for lookahead in (False, True):
        backend = _device_backend(golden, lookahead)
        out = tmp_path / f"{lookahead}.nc"
        results[lookahead] = simulate(case(), backend, out, convergence=rule)
        receipts[lookahead] = json.loads(out.with_suffix(".run.json").read_text())
        dispatches[lookahead] = backend.dispatches

    assert 32 < receipts[False]["completed_rounds"] <= 48
    assert receipts[True]["completed_rounds"] == receipts[False]["completed_rounds"]
    for name in ("radiance", "std_radiance", "DOP", "radiance_convergence"):
        np.testing.assert_array_equal(results[True].values[name], results[False].values[name], err_msg=name)
    assert dispatches[True] < dispatches[False], dispatches


def test_rounds_estimate_follows_the_square_root_law():
    from monki import RadianceConvergence
    from monki.convergence import RadianceStopping

    stopping = RadianceStopping(RadianceConvergence(0.01, minimum_rounds=32), 100)
    assert stopping.rounds_estimate() is None
    stopping.history.append({"rounds": 32, "max_relative_se": 0.02, "below_target": False, "streak": 0})
    assert stopping.rounds_estimate() == pytest.approx(128.0)


def test_groups_larger_than_a_dispatch_go_through_accumulate(tmp_path):
    from monki import RadianceConvergence, simulate

    golden = dict(np.load(GOLDEN / "driver_statistics.npz"))
    rounds = golden["stokes"].shape[0]
    ppc = int(golden["photons_per_column"])
    case = type("Case", (), {"photons_per_column": ppc, "rounds": rounds, "backward": False})
    # Checks every 12 rounds with room for 8 rounds per held dispatch: every group runs
    # through accumulate, and the products equal the round-by-round driver's.
    rule = RadianceConvergence(1e-9, minimum_rounds=32, check_every=12, consecutive_checks=1)
    results = {}
    for lookahead in (False, True):
        backend = _device_backend(golden, lookahead)
        results[lookahead] = simulate(case(), backend, tmp_path / f"{lookahead}.nc", convergence=rule)
        assert not backend._held
    for name in ("radiance", "std_radiance"):
        np.testing.assert_array_equal(results[True].values[name], results[False].values[name])
