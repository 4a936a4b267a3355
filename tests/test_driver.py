"""``simulate`` and its stopping rules over the oracle, as the reference's CPU-session tests
drive them over its Fortran worker (tests/integration/test_cpu.py:107-178): the 999 sentinel
of short runs, seed replay, an adaptive run equal to the fixed run of the rounds it
completed, and a round cap that is reported as such, never as convergence."""

from __future__ import annotations

import json
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))
from oracle_backend import oracle_backend  # noqa: E402


def _clear(rounds):
    from monki import scenes

    return scenes.clear_sky(50, rounds, nx=4, ny=3)


def _cloud(rounds):
    from monki import scenes

    return scenes.layered_cloud(20, rounds, nx=4, ny=3)


def test_short_run_keeps_the_uncertainty_sentinel(oracle, tmp_path):
    from monki import simulate
    from monki.validation import check_result

    result = simulate(_clear(2), oracle_backend(oracle, 3), tmp_path / "short.nc")
    assert np.all(result.standard_error == 999)
    assert result.values["radiance_convergence"].shape[0] == 2
    assert result.values["n_rounds"].item() == 2
    assert "uncertainty unavailable: need more than 30 completed rounds" in check_result(result)
    assert check_result(result, require_uncertainty=False) == []

    with pytest.raises(FileExistsError):
        simulate(_clear(2), oracle_backend(oracle, 3), result.path)


@pytest.mark.parametrize("rounds,sentinel", [(30, True), (31, False)])
def test_standard_error_exists_from_round_31(oracle, tmp_path, rounds, sentinel):
    from monki import simulate

    result = simulate(_clear(rounds), oracle_backend(oracle, 4), tmp_path / "run.nc")
    assert np.all(result.standard_error == 999) == sentinel
    if not sentinel:
        assert np.all(np.isfinite(result.standard_error)) and np.all(result.standard_error < 999)


def test_seed_replays_and_changes_the_photon_streams(oracle, tmp_path):
    from monki import simulate
    from monki.validation import compare

    runs = [simulate(_clear(2), oracle_backend(oracle, seed), tmp_path / f"{i}.nc")
            for i, seed in enumerate((714103, 714103, 23274))]
    # The oracle's thread partials are summed in completion order: a replay agrees to the
    # last few bits, which the reference's deterministic mode (relative 1e-10) accepts.
    assert compare(runs[0], runs[1], mode="deterministic").passed
    assert not compare(runs[0], runs[2], mode="deterministic").passed
    receipts = [json.loads((tmp_path / f"{i}.run.json").read_text()) for i in range(3)]
    assert [r["seed"] for r in receipts] == [714103, 714103, 23274]


def test_adaptive_run_equals_the_fixed_run_of_its_completed_rounds(oracle, tmp_path):
    from monki import AMFConvergence, simulate

    policy = AMFConvergence(relative_error=0.9, minimum_rounds=32, check_every=16, consecutive_checks=2)
    adaptive = simulate(_cloud(96), oracle_backend(oracle, 9), tmp_path / "adaptive.nc", convergence=policy)
    count = int(adaptive.values["n_rounds"].item())
    assert count == 48
    receipt = json.loads((tmp_path / "adaptive.run.json").read_text())
    assert receipt["status"] == "converged" and receipt["completed_rounds"] == 48
    assert receipt["amf_convergence"]["converged"]

    fixed = simulate(replace(_cloud(96), rounds=count), oracle_backend(oracle, 9), tmp_path / "fixed.nc")
    for name in ("radiance", "AMF_layer", "std_radiance"):
        np.testing.assert_allclose(adaptive.values[name], fixed.values[name], rtol=1e-12, atol=0, err_msg=name)
    assert np.all(np.isfinite(adaptive.values["std_AMF_layer"]))
    assert np.all(adaptive.values["std_AMF_layer"] >= 0)


def test_round_cap_is_not_reported_as_convergence(oracle, tmp_path):
    from monki import AMFConvergence, RadianceConvergence, simulate

    for tag, policy in (("amf", AMFConvergence(relative_error=1e-12, minimum_rounds=32)),
                        ("radiance", RadianceConvergence(relative_error=1e-12, minimum_rounds=32))):
        simulate(_cloud(32), oracle_backend(oracle, 11), tmp_path / f"{tag}.nc", convergence=policy)
        receipt = json.loads((tmp_path / f"{tag}.run.json").read_text())
        assert receipt["status"] == "max_rounds_reached"
        assert receipt["completed_rounds"] == 32
        key = "amf_convergence" if tag == "amf" else "radiance_convergence"
        assert not receipt[key]["converged"]


def test_amf_stopping_needs_layer_paths_and_a_cap_above_the_minimum(oracle, tmp_path):
    from monki import AMFConvergence, simulate

    with pytest.raises(ValueError, match="layer path"):
        simulate(_clear(32), oracle_backend(oracle, 1), tmp_path / "a.nc", convergence=AMFConvergence(minimum_rounds=32))
    with pytest.raises(ValueError, match="minimum_rounds"):
        simulate(_cloud(16), oracle_backend(oracle, 1), tmp_path / "b.nc", convergence=AMFConvergence(minimum_rounds=32))
